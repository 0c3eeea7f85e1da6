"""Alpha-vector policy (python/nova/pomdp_alpha_vectors.py:34-98)."""
import ctypes as ct

import numpy as np

from . import nova_pomdp_alpha_vectors as npav


class POMDPAlphaVectors(npav.NovaPOMDPAlphaVectors):
    """ The alpha-vector representation of a POMDP policy. """

    def __init__(self):
        self.n = 0
        self.m = 0
        self.r = 0
        self.Gamma = ct.POINTER(ct.c_float)()
        self.pi = ct.POINTER(ct.c_uint)()

    def __del__(self):
        result = npav._nova.pomdp_alpha_vectors_uninitialize(self)
        if result != 0:
            print("Failed to free the alpha vectors.")
            raise Exception()

    def gamma_array(self):
        """Gamma as a numpy (r, n) copy."""
        if self.r == 0:
            return np.zeros((0, self.n), dtype=np.float32)
        return np.ctypeslib.as_array(self.Gamma, shape=(self.r * self.n,)).reshape(self.r, self.n).copy()

    def pi_array(self):
        """pi as a numpy (r,) copy."""
        if self.r == 0:
            return np.zeros((0,), dtype=np.uint32)
        return np.ctypeslib.as_array(self.pi, shape=(self.r,)).copy()

    def __str__(self):
        return "Gamma:\n%s\n\npi:\n%s\n\n" % (str(self.gamma_array().T), str(self.pi_array()))

    def value_and_action(self, b):
        """ Compute the optimal value and action at a belief state (nova's FP32 host evaluation).

            Parameters:
                b   --  A numpy array for the belief (n array).

            Returns:
                V   --  The optimal value at this belief.
                a   --  The optimal action at this belief.
        """
        belief = (ct.c_float * self.n)(*np.asarray(b, dtype=np.float32).ravel())
        Vb = ct.c_float(0.0)
        a = ct.c_uint(0)
        result = npav._nova.pomdp_alpha_vectors_value_and_action(self, belief, ct.byref(Vb), ct.byref(a))
        if result != 0:
            print("Failed to compute the optimal value and action.")
            raise Exception()
        return Vb.value, a.value

    def value_and_action_batched(self, B):
        """ V(b) and the action for every row of B (count x n), each with the bits of
            value_and_action, evaluated on the GPU (pomdp_alpha_vectors_value_and_action_batched). """
        B = np.ascontiguousarray(np.asarray(B, dtype=np.float32).reshape(-1, self.n))
        count = B.shape[0]
        V = np.empty(count, np.float32)
        a = np.empty(count, np.uint32)
        result = npav._nova.pomdp_alpha_vectors_value_and_action_batched(
            self, B.ctypes.data_as(ct.POINTER(ct.c_float)), count, V.ctypes.data_as(ct.POINTER(ct.c_float)),
            a.ctypes.data_as(ct.POINTER(ct.c_uint)))
        if result != 0:
            raise RuntimeError("pomdp_alpha_vectors_value_and_action_batched failed with code %d" % result)
        return V, a
