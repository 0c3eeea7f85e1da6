"""Perseus solver objects (python/nova/pomdp_perseus.py:38-142), plus POMDPPerseusGPU."""
import ctypes as ct

import numpy as np

from . import pomdp
from . import pomdp_alpha_vectors as pav
from . import nova_pomdp_perseus as npper
from .pomdp_pbvi import _initial_gamma


def _perseus_text(alg, extra):
    """ The solver's initial alphas (an r x n array once set) and counters as text. """
    r, n = int(alg.pomdp.r), int(alg.pomdp.n)
    g0 = str(np.array([alg.GammaInitial[i] for i in range(r * n)]).reshape((r, n))) if alg.GammaInitial else "(none)"
    return "GammaInitial:\n%s\n\ncurrentHorizon: %d\n\n%srGamma: %d\n\nrGammaPrime: %d\n\nrTilde: %d\n\n" % (
        g0, int(alg.currentHorizon), extra, int(alg.rGamma), int(alg.rGammaPrime), int(alg.rTilde))


class POMDPPerseusCPU(npper.NovaPOMDPPerseusCPU):
    """ The Perseus solver (host buffers). """

    def __init__(self, pomdpObject, GammaInitial=None):
        self.pomdp = pomdpObject
        self.pomdpPtr = ct.POINTER(pomdp.POMDP)(self.pomdp)
        self._GammaInitialBuf = _initial_gamma(self.pomdp, GammaInitial)
        self.GammaInitial = ct.cast(self._GammaInitialBuf, ct.POINTER(ct.c_float))
        self.currentHorizon = int(0)
        self.rGamma = int(0)
        self.rGammaPrime = int(0)
        self.rTilde = int(0)
        self.BTilde = ct.POINTER(ct.c_uint)()
        self.Gamma = ct.POINTER(ct.c_float)()
        self.GammaPrime = ct.POINTER(ct.c_float)()
        self.pi = ct.POINTER(ct.c_uint)()
        self.piPrime = ct.POINTER(ct.c_uint)()
        result = npper._nova.pomdp_perseus_initialize_cpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to initialize the Perseus (CPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = npper._nova.pomdp_perseus_uninitialize_cpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to free the Perseus (CPU) algorithm.")
            raise Exception()

    def __str__(self):
        return _perseus_text(self, "")

    def solve(self):
        policy = pav.POMDPAlphaVectors()
        result = npper._nova.pomdp_perseus_execute_cpu(self.pomdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's CPU POMDP solver.")
            raise Exception()
        return policy


class POMDPPerseusGPU(npper.NovaPOMDPPerseusGPU):
    """ The Perseus solver (device buffers). """

    def __init__(self, pomdpObject, numThreads=1024, GammaInitial=None):
        self.pomdp = pomdpObject
        self.pomdpPtr = ct.POINTER(pomdp.POMDP)(self.pomdp)
        self._GammaInitialBuf = _initial_gamma(self.pomdp, GammaInitial)
        self.GammaInitial = ct.cast(self._GammaInitialBuf, ct.POINTER(ct.c_float))
        self.numThreads = numThreads
        self.currentHorizon = int(0)
        self.rGamma = int(0)
        self.rGammaPrime = int(0)
        self.rTilde = int(0)
        self.BTilde = ct.POINTER(ct.c_uint)()
        self.d_Gamma = ct.POINTER(ct.c_float)()
        self.d_GammaPrime = ct.POINTER(ct.c_float)()
        self.d_pi = ct.POINTER(ct.c_uint)()
        self.d_piPrime = ct.POINTER(ct.c_uint)()
        result = npper._nova.pomdp_perseus_initialize_gpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to initialize the Perseus (GPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = npper._nova.pomdp_perseus_uninitialize_gpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to free the Perseus (GPU) algorithm.")
            raise Exception()

    def __str__(self):
        return _perseus_text(self, "numThreads: %d\n\n" % int(self.numThreads))

    def solve(self):
        policy = pav.POMDPAlphaVectors()
        result = npper._nova.pomdp_perseus_execute_gpu(self.pomdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's GPU POMDP solver.")
            raise Exception()
        return policy
