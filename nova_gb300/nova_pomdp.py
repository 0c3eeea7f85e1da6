"""ctypes mirror of the POMDP struct and model functions (python/nova/nova_pomdp.py:38-128).

Field names, order and types equal include/nova/pomdp/pomdp.h (reference
include/nova/pomdp/pomdp.h:61-85).
"""
import ctypes as ct

from . import _lib

_nova = _lib.load()


class NovaPOMDP(ct.Structure):
    """ The C struct POMDP object. """
    _fields_ = [("n", ct.c_uint),
                ("ns", ct.c_uint),
                ("m", ct.c_uint),
                ("z", ct.c_uint),
                ("r", ct.c_uint),
                ("rz", ct.c_uint),
                ("gamma", ct.c_float),
                ("horizon", ct.c_uint),
                ("S", ct.POINTER(ct.c_int)),
                ("T", ct.POINTER(ct.c_float)),
                ("O", ct.POINTER(ct.c_float)),
                ("R", ct.POINTER(ct.c_float)),
                ("Z", ct.POINTER(ct.c_int)),
                ("B", ct.POINTER(ct.c_float)),
                ("d_S", ct.POINTER(ct.c_int)),
                ("d_T", ct.POINTER(ct.c_float)),
                ("d_O", ct.POINTER(ct.c_float)),
                ("d_R", ct.POINTER(ct.c_float)),
                ("d_Z", ct.POINTER(ct.c_int)),
                ("d_B", ct.POINTER(ct.c_float)),
                ]


_P = ct.POINTER(NovaPOMDP)

_nova.pomdp_initialize_cpu.argtypes = (_P, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint,
                                       ct.c_float, ct.c_uint)
_nova.pomdp_belief_update_cpu.argtypes = (_P, ct.POINTER(ct.c_float), ct.c_uint, ct.c_uint,
                                          ct.POINTER(ct.POINTER(ct.c_float)))
_nova.pomdp_add_new_raw_beliefs_cpu.argtypes = (_P, ct.c_uint, ct.POINTER(ct.c_float))
_nova.pomdp_uninitialize_cpu.argtypes = (_P,)
for _name in ("pomdp_initialize_gpu", "pomdp_uninitialize_gpu",
              "pomdp_initialize_successors_gpu", "pomdp_uninitialize_successors_gpu",
              "pomdp_initialize_state_transitions_gpu", "pomdp_uninitialize_state_transitions_gpu",
              "pomdp_initialize_observation_transitions_gpu", "pomdp_uninitialize_observation_transitions_gpu",
              "pomdp_initialize_rewards_gpu", "pomdp_uninitialize_rewards_gpu",
              "pomdp_initialize_nonzero_beliefs_gpu", "pomdp_uninitialize_nonzero_beliefs_gpu",
              "pomdp_initialize_belief_points_gpu", "pomdp_uninitialize_belief_points_gpu"):
    getattr(_nova, _name).argtypes = (_P,)

# Belief-set expansion and sigma approximation (pomdp_expand_cpu.h,
# pomdp_expand_gpu.h, pomdp_sigma_cpu.h), computed on the GPU.
from . import nova_pomdp_alpha_vectors as _npav  # noqa: E402
_nova.pomdp_expand_random_cpu.argtypes = (_P, ct.c_uint)
_nova.pomdp_expand_distinct_beliefs_cpu.argtypes = (_P,)
_nova.pomdp_expand_pema_cpu.argtypes = (_P, ct.POINTER(_npav.NovaPOMDPAlphaVectors))
_nova.pomdp_sigma_cpu.argtypes = (_P, ct.c_uint, ct.POINTER(ct.c_float))
_nova.pomdp_expand_random_gpu.argtypes = (_P, ct.c_uint, ct.c_uint, ct.POINTER(ct.c_uint),
                                          ct.POINTER(ct.POINTER(ct.c_float)))
_nova.nova_gb300_expand_seed.argtypes = (ct.c_uint, ct.c_uint)
_nova.nova_load_raw_pomdp.argtypes = (ct.c_char_p, _P, ct.c_uint)
_nova.nova_load_cassandra_pomdp.argtypes = (ct.c_char_p, _P, ct.POINTER(ct.c_double), ct.POINTER(ct.c_double))
