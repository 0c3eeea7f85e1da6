"""ctypes mirror of the Perseus solver structs (python/nova/nova_pomdp_perseus.py:47-78),
plus the GPU struct of include/nova/pomdp/algorithms/pomdp_perseus_gpu.h."""
import ctypes as ct

from . import _lib
from . import pomdp
from . import pomdp_alpha_vectors as pav

_nova = _lib.load()


class NovaPOMDPPerseusCPU(ct.Structure):
    """ The C struct NovaPOMDPPerseusCPU object. """
    _fields_ = [("GammaInitial", ct.POINTER(ct.c_float)),
                ("currentHorizon", ct.c_uint),
                ("rGamma", ct.c_uint),
                ("rGammaPrime", ct.c_uint),
                ("rTilde", ct.c_uint),
                ("BTilde", ct.POINTER(ct.c_uint)),
                ("Gamma", ct.POINTER(ct.c_float)),
                ("GammaPrime", ct.POINTER(ct.c_float)),
                ("pi", ct.POINTER(ct.c_uint)),
                ("piPrime", ct.POINTER(ct.c_uint)),
                ]


class NovaPOMDPPerseusGPU(ct.Structure):
    """ The C struct NovaPOMDPPerseusGPU object. """
    _fields_ = [("GammaInitial", ct.POINTER(ct.c_float)),
                ("numThreads", ct.c_uint),
                ("currentHorizon", ct.c_uint),
                ("rGamma", ct.c_uint),
                ("rGammaPrime", ct.c_uint),
                ("rTilde", ct.c_uint),
                ("BTilde", ct.POINTER(ct.c_uint)),
                ("d_Gamma", ct.POINTER(ct.c_float)),
                ("d_GammaPrime", ct.POINTER(ct.c_float)),
                ("d_pi", ct.POINTER(ct.c_uint)),
                ("d_piPrime", ct.POINTER(ct.c_uint)),
                ]


_P = ct.POINTER(pomdp.POMDP)
_A = ct.POINTER(pav.POMDPAlphaVectors)
for _suffix, _S in (("cpu", ct.POINTER(NovaPOMDPPerseusCPU)), ("gpu", ct.POINTER(NovaPOMDPPerseusGPU))):
    getattr(_nova, "pomdp_perseus_initialize_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_perseus_execute_" + _suffix).argtypes = (_P, _S, _A)
    getattr(_nova, "pomdp_perseus_uninitialize_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_perseus_update_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_perseus_get_policy_" + _suffix).argtypes = (_P, _S, _A)
