"""ctypes mirror of the value-iteration structs (python/nova/nova_mdp_vi.py:47-103).
The reference declares mdp_vi_get_policy_gpu with the CPU struct type
(nova_mdp_vi.py:102); here it takes the GPU struct."""
import ctypes as ct

from . import _lib
from . import mdp
from . import mdp_value_function as mvf

_nova = _lib.load()


class NovaMDPValueIterationCPU(ct.Structure):
    """ The C struct MDPValueIterationCPU object. """
    _fields_ = [("Vinitial", ct.POINTER(ct.c_float)),
                ("currentHorizon", ct.c_uint),
                ("V", ct.POINTER(ct.c_float)),
                ("Vprime", ct.POINTER(ct.c_float)),
                ("pi", ct.POINTER(ct.c_uint)),
                ]


class NovaMDPValueIterationGPU(ct.Structure):
    """ The C struct MDPValueIterationGPU object. """
    _fields_ = [("Vinitial", ct.POINTER(ct.c_float)),
                ("numThreads", ct.c_uint),
                ("currentHorizon", ct.c_uint),
                ("d_V", ct.POINTER(ct.c_float)),
                ("d_Vprime", ct.POINTER(ct.c_float)),
                ("d_pi", ct.POINTER(ct.c_uint)),
                ]


_M = ct.POINTER(mdp.MDP)
_F = ct.POINTER(mvf.MDPValueFunction)
for _suffix, _S in (("cpu", ct.POINTER(NovaMDPValueIterationCPU)), ("gpu", ct.POINTER(NovaMDPValueIterationGPU))):
    getattr(_nova, "mdp_vi_initialize_" + _suffix).argtypes = (_M, _S)
    getattr(_nova, "mdp_vi_execute_" + _suffix).argtypes = (_M, _S, _F)
    getattr(_nova, "mdp_vi_uninitialize_" + _suffix).argtypes = (_M, _S)
    getattr(_nova, "mdp_vi_update_" + _suffix).argtypes = (_M, _S)
    getattr(_nova, "mdp_vi_get_policy_" + _suffix).argtypes = (_M, _S, _F)
_G = ct.POINTER(NovaMDPValueIterationGPU)
_nova.mdp_vi_execute_until_converged_gpu.argtypes = (_M, _G, _F, ct.c_double, ct.c_uint, ct.POINTER(ct.c_uint),
                                                     ct.POINTER(ct.c_double))
_nova.mdp_vi_residual_gpu.argtypes = (_M, _G, ct.POINTER(ct.c_double))
_nova.mdp_vi_set_tiling_gpu.argtypes = (ct.c_uint, ct.c_uint)
_nova.mdp_vi_tiling_status_gpu.argtypes = (ct.c_void_p, ct.POINTER(ct.c_uint))

TILING_AUTO = 0
TILING_ALWAYS = 1
TILING_NEVER = 2
