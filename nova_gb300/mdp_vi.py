"""Value-iteration solver objects (python/nova/mdp_vi.py:38-203)."""
import ctypes as ct

import numpy as np

from . import mdp
from . import mdp_value_function as mvf
from . import nova_mdp_vi as nmvi


def _initial_v(m, Vinitial):
    if Vinitial is None:
        if m.gamma < 1.0:
            rmin = m.Rmin if m.Rmin is not None else float(np.ctypeslib.as_array(m.R, shape=(m.n * m.m,)).min())
            Vinitial = np.full(m.n, np.float32(rmin) / (np.float32(1.0) - np.float32(m.gamma)), dtype=np.float32)
        else:
            Vinitial = np.zeros(m.n, dtype=np.float32)
    Vinitial = np.ascontiguousarray(np.asarray(Vinitial, dtype=np.float32).ravel())
    buf = (ct.c_float * m.n)()
    ct.memmove(buf, Vinitial.ctypes.data, Vinitial.nbytes)
    return buf


def _show(ptr, count):
    """ A host array as text, or '(none)' while it is not allocated. """
    return str(np.array([ptr[i] for i in range(count)])) if ptr else "(none)"


class MDPValueIterationCPU(nmvi.NovaMDPValueIterationCPU):
    """ Value iteration (host buffers). """

    def __init__(self, mdpObject, Vinitial=None):
        self.mdp = mdpObject
        self.mdpPtr = ct.POINTER(mdp.MDP)(self.mdp)
        self._VinitialBuf = _initial_v(self.mdp, Vinitial)
        self.Vinitial = ct.cast(self._VinitialBuf, ct.POINTER(ct.c_float))
        self.currentHorizon = int(0)
        self.V = ct.POINTER(ct.c_float)()
        self.Vprime = ct.POINTER(ct.c_float)()
        self.pi = ct.POINTER(ct.c_uint)()
        result = nmvi._nova.mdp_vi_initialize_cpu(self.mdpPtr, self)
        if result != 0:
            print("Failed to initialize the value iteration (CPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = nmvi._nova.mdp_vi_uninitialize_cpu(self.mdpPtr, self)
        if result != 0:
            print("Failed to free the value iteration (CPU) algorithm.")
            raise Exception()

    def __str__(self):
        n = int(self.mdp.n)
        return "Vinitial:\n%s\n\ncurrentHorizon: %d\n\nV:\n%s\n\nVprime:\n%s\n\npi:\n%s\n\n" % (
            _show(self.Vinitial, n), int(self.currentHorizon), _show(self.V, n), _show(self.Vprime, n),
            _show(self.pi, n))

    def solve(self):
        policy = mvf.MDPValueFunction()
        result = nmvi._nova.mdp_vi_execute_cpu(self.mdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's CPU MDP solver.")
            raise Exception()
        return policy


class MDPValueIterationGPU(nmvi.NovaMDPValueIterationGPU):
    """ Value iteration (device buffers). """

    def __init__(self, mdpObject, numThreads=1024, Vinitial=None):
        self.mdp = mdpObject
        self.mdpPtr = ct.POINTER(mdp.MDP)(self.mdp)
        self._VinitialBuf = _initial_v(self.mdp, Vinitial)
        self.Vinitial = ct.cast(self._VinitialBuf, ct.POINTER(ct.c_float))
        self.currentHorizon = int(0)
        self.numThreads = numThreads
        self.d_V = ct.POINTER(ct.c_float)()
        self.d_Vprime = ct.POINTER(ct.c_float)()
        self.d_pi = ct.POINTER(ct.c_uint)()
        result = nmvi._nova.mdp_vi_initialize_gpu(self.mdpPtr, self)
        if result != 0:
            print("Failed to initialize the value iteration (GPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = nmvi._nova.mdp_vi_uninitialize_gpu(self.mdpPtr, self)
        if result != 0:
            print("Failed to free the value iteration (GPU) algorithm.")
            raise Exception()

    def __str__(self):
        return "Vinitial:\n%s\n\ncurrentHorizon: %d\n\nnumThreads: %d\n\n" % (
            _show(self.Vinitial, int(self.mdp.n)), int(self.currentHorizon), int(self.numThreads))

    def solve(self):
        policy = mvf.MDPValueFunction()
        result = nmvi._nova.mdp_vi_execute_gpu(self.mdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's GPU MDP solver.")
            raise Exception()
        return policy

    def solve_until_converged(self, tol=1e-6, maxSweeps=2000):
        """ Sweeps until the FP64 Bellman residual < tol (mdp_vi_execute_until_converged_gpu).
            Returns (policy, sweeps, residual). """
        policy = mvf.MDPValueFunction()
        sweeps = ct.c_uint(0)
        resid = ct.c_double(0.0)
        result = nmvi._nova.mdp_vi_execute_until_converged_gpu(self.mdpPtr, self, policy, float(tol),
                                                               int(maxSweeps), ct.byref(sweeps), ct.byref(resid))
        if result != 0:
            raise RuntimeError("mdp_vi_execute_until_converged_gpu failed with code %d" % result)
        return policy, sweeps.value, resid.value


def set_tiling(mode, tileStates=0):
    """ Select the Bellman sweep kernel for solvers that build their plan after
    this call (mdp_vi_set_tiling_gpu): nova_mdp_vi.TILING_AUTO, _ALWAYS or
    _NEVER, and the states per shared-memory tile (0 = default). """
    result = nmvi._nova.mdp_vi_set_tiling_gpu(int(mode), int(tileStates))
    if result != 0:
        raise ValueError("mdp_vi_set_tiling_gpu rejected mode=%r tileStates=%r" % (mode, tileStates))


def tiling_status(solver=None):
    """ 0 = no sweep yet, 1 = tiled sweep, 2 = per-row gather sweep, for an
    initialized solver object, or for the plan built last when solver is None. """
    st = ct.c_uint(0)
    ptr = None if solver is None else ct.addressof(solver)
    result = nmvi._nova.mdp_vi_tiling_status_gpu(ptr, ct.byref(st))
    if result != 0:
        raise RuntimeError("mdp_vi_tiling_status_gpu failed with code %d" % result)
    return st.value
