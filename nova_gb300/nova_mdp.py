"""ctypes mirror of the MDP struct and model functions (python/nova/nova_mdp.py:44-89)."""
import ctypes as ct

from . import _lib

_nova = _lib.load()


class NovaMDP(ct.Structure):
    """ The C struct MDP object. """
    _fields_ = [("n", ct.c_uint),
                ("ns", ct.c_uint),
                ("m", ct.c_uint),
                ("gamma", ct.c_float),
                ("horizon", ct.c_uint),
                ("epsilon", ct.c_float),
                ("s0", ct.c_uint),
                ("ng", ct.c_uint),
                ("goals", ct.POINTER(ct.c_uint)),
                ("S", ct.POINTER(ct.c_int)),
                ("T", ct.POINTER(ct.c_float)),
                ("R", ct.POINTER(ct.c_float)),
                ("d_goals", ct.POINTER(ct.c_uint)),
                ("d_S", ct.POINTER(ct.c_int)),
                ("d_T", ct.POINTER(ct.c_float)),
                ("d_R", ct.POINTER(ct.c_float)),
                ]


_M = ct.POINTER(NovaMDP)
_nova.mdp_initialize_cpu.argtypes = (_M, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_float, ct.c_uint, ct.c_float,
                                     ct.c_uint, ct.c_uint)
_nova.mdp_uninitialize_cpu.argtypes = (_M,)
for _name in ("mdp_initialize_gpu", "mdp_uninitialize_gpu",
              "mdp_initialize_successors_gpu", "mdp_uninitialize_successors_gpu",
              "mdp_initialize_state_transitions_gpu", "mdp_uninitialize_state_transitions_gpu",
              "mdp_initialize_rewards_gpu", "mdp_uninitialize_rewards_gpu",
              "mdp_initialize_goals_gpu", "mdp_uninitialize_goals_gpu"):
    getattr(_nova, _name).argtypes = (_M,)
_nova.nova_load_raw_mdp.argtypes = (ct.c_char_p, ct.POINTER(NovaMDP), ct.c_uint)
