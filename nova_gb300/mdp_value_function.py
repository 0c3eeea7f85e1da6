"""MDP value function (python/nova/mdp_value_function.py)."""
import ctypes as ct

import numpy as np

from . import nova_mdp_value_function as nmvf


class MDPValueFunction(nmvf.NovaMDPValueFunction):
    """ The value function representation of an MDP policy. """

    def __init__(self):
        self.n = 0
        self.m = 0
        self.r = 0
        self.S = ct.POINTER(ct.c_uint)()
        self.V = ct.POINTER(ct.c_float)()
        self.pi = ct.POINTER(ct.c_uint)()

    def __del__(self):
        result = nmvf._nova.mdp_value_function_uninitialize(self)
        if result != 0:
            print("Failed to free the value function.")
            raise Exception()

    def V_array(self):
        k = self.r if self.r > 0 else self.n
        return np.ctypeslib.as_array(self.V, shape=(k,)).copy() if k else np.zeros(0, np.float32)

    def pi_array(self):
        k = self.r if self.r > 0 else self.n
        return np.ctypeslib.as_array(self.pi, shape=(k,)).copy() if k else np.zeros(0, np.uint32)

    def __str__(self):
        return "V:\n%s\n\npi:\n%s\n\n" % (str(self.V_array()), str(self.pi_array()))
