"""ctypes mirror of POMDPAlphaVectors (python/nova/nova_pomdp_alpha_vectors.py:42-62)."""
import ctypes as ct

from . import _lib

_nova = _lib.load()


class NovaPOMDPAlphaVectors(ct.Structure):
    """ The C struct POMDPAlphaVectors object. """
    _fields_ = [("n", ct.c_uint),
                ("m", ct.c_uint),
                ("r", ct.c_uint),
                ("Gamma", ct.POINTER(ct.c_float)),
                ("pi", ct.POINTER(ct.c_uint)),
                ]


_A = ct.POINTER(NovaPOMDPAlphaVectors)
_nova.pomdp_alpha_vectors_initialize.argtypes = (_A, ct.c_uint, ct.c_uint, ct.c_uint)
_nova.pomdp_alpha_vectors_value_and_action.argtypes = (_A, ct.POINTER(ct.c_float), ct.POINTER(ct.c_float),
                                                       ct.POINTER(ct.c_uint))
_nova.pomdp_alpha_vectors_uninitialize.argtypes = (_A,)

_nova.pomdp_alpha_vectors_value_and_action_batched.argtypes = (ct.POINTER(NovaPOMDPAlphaVectors),
                                                               ct.POINTER(ct.c_float), ct.c_uint,
                                                               ct.POINTER(ct.c_float), ct.POINTER(ct.c_uint))
_nova.pomdp_alpha_vectors_value_batched_gpu.argtypes = (ct.c_void_p, ct.c_void_p, ct.c_uint, ct.c_uint,
                                                        ct.c_void_p, ct.c_uint, ct.c_void_p, ct.c_void_p)
