"""ctypes mirror of the PBVI solver structs (python/nova/nova_pomdp_pbvi.py:47-104),
plus the additive nova-gb300 entry points."""
import ctypes as ct

from . import _lib
from . import pomdp
from . import pomdp_alpha_vectors as pav

_nova = _lib.load()


class NovaPOMDPPBVICPU(ct.Structure):
    """ The C struct NovaPOMDPPBVICPU object. """
    _fields_ = [("GammaInitial", ct.POINTER(ct.c_float)),
                ("currentHorizon", ct.c_uint),
                ("Gamma", ct.POINTER(ct.c_float)),
                ("GammaPrime", ct.POINTER(ct.c_float)),
                ("pi", ct.POINTER(ct.c_uint)),
                ]


class NovaPOMDPPBVIGPU(ct.Structure):
    """ The C struct NovaPOMDPPBVIGPU object. """
    _fields_ = [("GammaInitial", ct.POINTER(ct.c_float)),
                ("numThreads", ct.c_uint),
                ("currentHorizon", ct.c_uint),
                ("d_Gamma", ct.POINTER(ct.c_float)),
                ("d_GammaPrime", ct.POINTER(ct.c_float)),
                ("d_pi", ct.POINTER(ct.c_uint)),
                ("d_alphaBA", ct.POINTER(ct.c_float)),
                ]


class NovaPBVIStats(ct.Structure):
    """ nova-gb300 per-update counters (include/nova/nova_gb300.h). """
    _fields_ = [("horizon", ct.c_uint),
                ("scoring", ct.c_uint),
                ("uniqueAlphas", ct.c_uint),
                ("rowsMultiCand", ct.c_uint),
                ("rowsOverflow", ct.c_uint),
                ("candidates", ct.c_uint),
                ("msDedup", ct.c_float),
                ("msProject", ct.c_float),
                ("msScore", ct.c_float),
                ("msRescore", ct.c_float),
                ("msActions", ct.c_float),
                ("msAssemble", ct.c_float),
                ("msTotal", ct.c_float),
                ("msGemm", ct.c_float),
                ("launches", ct.c_uint),
                ("tcGroups", ct.c_uint),
                ]


SCORING_EXACT = 0
SCORING_BF16 = 1
SCORING_FP16 = 2
TABLE_AUTO = 0
TABLE_NEVER = 1

_P = ct.POINTER(pomdp.POMDP)
_C = ct.POINTER(NovaPOMDPPBVICPU)
_G = ct.POINTER(NovaPOMDPPBVIGPU)
_A = ct.POINTER(pav.POMDPAlphaVectors)

for _suffix, _S in (("cpu", _C), ("gpu", _G)):
    getattr(_nova, "pomdp_pbvi_initialize_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_pbvi_execute_" + _suffix).argtypes = (_P, _S, _A)
    getattr(_nova, "pomdp_pbvi_uninitialize_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_pbvi_update_" + _suffix).argtypes = (_P, _S)
    getattr(_nova, "pomdp_pbvi_get_policy_" + _suffix).argtypes = (_P, _S, _A)

_nova.nova_gb300_kernel_launches.restype = ct.c_ulonglong
_nova.pomdp_pbvi_set_scoring_gpu.argtypes = (_G, ct.c_uint)
_nova.pomdp_pbvi_set_table_gpu.argtypes = (_G, ct.c_uint)
_nova.pomdp_pbvi_set_graph_gpu.argtypes = (_G, ct.c_uint)
_nova.pomdp_pbvi_get_stats_gpu.argtypes = (_G, ct.POINTER(NovaPBVIStats))
_nova.pomdp_pbvi_row_detail_gpu.argtypes = (_G, ct.POINTER(ct.c_uint), ct.POINTER(ct.c_uint))
_nova.pomdp_pbvi_value_gpu.argtypes = (_P, _G, ct.POINTER(ct.c_float), ct.POINTER(ct.c_double),
                                       ct.POINTER(ct.c_uint))
_nova.pomdp_pbvi_update_record_gpu.argtypes = (_P, _G, ct.c_void_p, ct.c_void_p)
_nova.pomdp_pbvi_execute_recorded_gpu.argtypes = (_P, _G, ct.c_uint, ct.c_uint, ct.c_void_p, ct.c_void_p,
                                                  ct.c_void_p)
_nova.pomdp_pbvi_adjoint_gpu.argtypes = (_P, ct.c_uint, ct.c_uint, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                         ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                         ct.POINTER(ct.c_double), ct.POINTER(ct.c_uint))
_nova.pomdp_pbvi_value_replay_f64_gpu.argtypes = (_P, ct.c_uint, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                                  ct.c_uint, ct.POINTER(ct.c_double), ct.POINTER(ct.c_uint))
from . import nova_pomdp_alpha_vectors as _npav  # noqa: E402
_nova.pomdp_pbvi_execute_batched_gpu.argtypes = (ct.POINTER(_P), ct.POINTER(_G),
                                                 ct.POINTER(ct.POINTER(_npav.NovaPOMDPAlphaVectors)), ct.c_uint,
                                                 ct.c_uint, ct.c_uint)
_nova.pomdp_pbvi_execute_batched_graph_gpu.argtypes = _nova.pomdp_pbvi_execute_batched_gpu.argtypes
_nova.pomdp_pbvi_execute_batched_persistent_gpu.argtypes = _nova.pomdp_pbvi_execute_batched_gpu.argtypes
