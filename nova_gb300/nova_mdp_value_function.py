"""ctypes mirror of MDPValueFunction (python/nova/nova_mdp_value_function.py:42-59)."""
import ctypes as ct

from . import _lib

_nova = _lib.load()


class NovaMDPValueFunction(ct.Structure):
    """ The C struct NovaMDPValueFunction object. """
    _fields_ = [("n", ct.c_uint),
                ("m", ct.c_uint),
                ("r", ct.c_uint),
                ("S", ct.POINTER(ct.c_uint)),
                ("V", ct.POINTER(ct.c_float)),
                ("pi", ct.POINTER(ct.c_uint)),
                ]


_V = ct.POINTER(NovaMDPValueFunction)
_nova.mdp_value_function_initialize.argtypes = (_V, ct.c_uint, ct.c_uint, ct.c_uint)
_nova.mdp_value_function_uninitialize.argtypes = (_V,)
