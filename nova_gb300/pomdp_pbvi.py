"""PBVI solver objects (python/nova/pomdp_pbvi.py:38-214).

POMDPPBVICPU keeps nova's host-buffer contract and POMDPPBVIGPU its
device-buffer contract; in this library both run the backup on the GB300.
"""
import ctypes as ct

import numpy as np

from . import pomdp
from . import pomdp_alpha_vectors as pav
from . import nova_pomdp_pbvi as npp


def _initial_gamma(p, GammaInitial):
    """nova's default: Rmin / (1 - gamma) everywhere, or 0 when gamma == 1."""
    if GammaInitial is None:
        if p.gamma < 1.0:
            rmin = p.Rmin if p.Rmin is not None else float(
                np.ctypeslib.as_array(p.R, shape=(p.n * p.m,)).min())
            GammaInitial = np.full(p.r * p.n, np.float32(rmin) / (np.float32(1.0) - np.float32(p.gamma)),
                                   dtype=np.float32)
        else:
            GammaInitial = np.zeros(p.r * p.n, dtype=np.float32)
    GammaInitial = np.ascontiguousarray(np.asarray(GammaInitial, dtype=np.float32).ravel())
    buf = (ct.c_float * (p.r * p.n))()
    ct.memmove(buf, GammaInitial.ctypes.data, GammaInitial.nbytes)
    return buf


class POMDPPBVICPU(npp.NovaPOMDPPBVICPU):
    """ The point-based value iteration solver (host buffers). """

    def __init__(self, pomdpObject, GammaInitial=None):
        self.pomdp = pomdpObject
        self.pomdpPtr = ct.POINTER(pomdp.POMDP)(self.pomdp)
        self._GammaInitialBuf = _initial_gamma(self.pomdp, GammaInitial)
        self.GammaInitial = ct.cast(self._GammaInitialBuf, ct.POINTER(ct.c_float))
        self.currentHorizon = int(0)
        self.Gamma = ct.POINTER(ct.c_float)()
        self.GammaPrime = ct.POINTER(ct.c_float)()
        self.pi = ct.POINTER(ct.c_uint)()
        result = npp._nova.pomdp_pbvi_initialize_cpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to initialize the PBVI (CPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = npp._nova.pomdp_pbvi_uninitialize_cpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to free the PBVI (CPU) algorithm.")
            raise Exception()

    def update(self):
        """ One backup of every belief (pomdp_pbvi_update_cpu). """
        result = npp._nova.pomdp_pbvi_update_cpu(self.pomdpPtr, self)
        if result != 0:
            raise RuntimeError("pomdp_pbvi_update_cpu failed with code %d" % result)

    def solve(self):
        """ Solve the POMDP; returns the POMDPAlphaVectors policy. """
        policy = pav.POMDPAlphaVectors()
        result = npp._nova.pomdp_pbvi_execute_cpu(self.pomdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's CPU POMDP solver.")
            raise Exception()
        return policy

    def get_policy(self):
        policy = pav.POMDPAlphaVectors()
        result = npp._nova.pomdp_pbvi_get_policy_cpu(self.pomdpPtr, self, policy)
        if result != 0:
            raise RuntimeError("pomdp_pbvi_get_policy_cpu failed with code %d" % result)
        return policy

    def __str__(self):
        return "currentHorizon: %i\n\n" % self.currentHorizon


class POMDPPBVIGPU(npp.NovaPOMDPPBVIGPU):
    """ The point-based value iteration solver (device buffers). """

    def __init__(self, pomdpObject, numThreads=1024, GammaInitial=None):
        self.pomdp = pomdpObject
        self.pomdpPtr = ct.POINTER(pomdp.POMDP)(self.pomdp)
        self._GammaInitialBuf = _initial_gamma(self.pomdp, GammaInitial)
        self.GammaInitial = ct.cast(self._GammaInitialBuf, ct.POINTER(ct.c_float))
        self.currentHorizon = int(0)
        self.numThreads = numThreads
        self.d_Gamma = ct.POINTER(ct.c_float)()
        self.d_GammaPrime = ct.POINTER(ct.c_float)()
        self.d_pi = ct.POINTER(ct.c_uint)()
        self.d_alphaBA = ct.POINTER(ct.c_float)()
        result = npp._nova.pomdp_pbvi_initialize_gpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to initialize the PBVI (GPU) algorithm.")
            raise Exception()

    def __del__(self):
        result = npp._nova.pomdp_pbvi_uninitialize_gpu(self.pomdpPtr, self)
        if result != 0:
            print("Failed to free the PBVI (GPU) algorithm.")
            raise Exception()

    def set_scoring(self, mode):
        """ npp.SCORING_EXACT, npp.SCORING_BF16 or npp.SCORING_FP16 (pomdp_pbvi_set_scoring_gpu). """
        result = npp._nova.pomdp_pbvi_set_scoring_gpu(self, int(mode))
        if result != 0:
            raise RuntimeError("pomdp_pbvi_set_scoring_gpu failed with code %d" % result)

    def set_table(self, mode):
        """ npp.TABLE_AUTO (build the projection table when it fits) or npp.TABLE_NEVER
            (score and assemble straight from the alphas; same bits) (pomdp_pbvi_set_table_gpu). """
        result = npp._nova.pomdp_pbvi_set_table_gpu(self, int(mode))
        if result != 0:
            raise RuntimeError("pomdp_pbvi_set_table_gpu failed with code %d" % result)

    def set_graph(self, enable=True):
        """ Graph mode for later updates (pomdp_pbvi_set_graph_gpu): once the tensor-core
            schedule is tuned, each update replays a captured CUDA graph. """
        result = npp._nova.pomdp_pbvi_set_graph_gpu(self, 1 if enable else 0)
        if result != 0:
            raise RuntimeError("pomdp_pbvi_set_graph_gpu failed with code %d" % result)

    def update(self):
        """ One backup of every belief (pomdp_pbvi_update_gpu). """
        result = npp._nova.pomdp_pbvi_update_gpu(self.pomdpPtr, self)
        if result != 0:
            raise RuntimeError("pomdp_pbvi_update_gpu failed with code %d" % result)

    def stats(self):
        s = npp.NovaPBVIStats()
        result = npp._nova.pomdp_pbvi_get_stats_gpu(self, ct.byref(s))
        if result != 0:
            raise RuntimeError("pomdp_pbvi_get_stats_gpu failed with code %d" % result)
        return {name: getattr(s, name) for name, _ in s._fields_}

    def row_detail(self):
        """ Per-belief (candidates re-scored exactly, rows scanned exactly) of the last
            tensor-core update (pomdp_pbvi_row_detail_gpu), as two uint32 arrays of r. """
        r = self.pomdp.r
        cand = np.zeros(r, np.uint32)
        exact = np.zeros(r, np.uint32)
        result = npp._nova.pomdp_pbvi_row_detail_gpu(self, cand.ctypes.data_as(ct.POINTER(ct.c_uint)),
                                                     exact.ctypes.data_as(ct.POINTER(ct.c_uint)))
        if result != 0:
            raise RuntimeError("pomdp_pbvi_row_detail_gpu failed with code %d" % result)
        return cand, exact

    def value(self, b):
        """ FP64 V(b) and action over the current device alpha set (pomdp_pbvi_value_gpu). """
        b = np.ascontiguousarray(np.asarray(b, dtype=np.float32).ravel())
        Vb = ct.c_double(0.0)
        a = ct.c_uint(0)
        result = npp._nova.pomdp_pbvi_value_gpu(self.pomdpPtr, self, b.ctypes.data_as(ct.POINTER(ct.c_float)),
                                                ct.byref(Vb), ct.byref(a))
        if result != 0:
            raise RuntimeError("pomdp_pbvi_value_gpu failed with code %d" % result)
        return Vb.value, a.value

    def solve(self):
        """ Solve the POMDP; returns the POMDPAlphaVectors policy. """
        policy = pav.POMDPAlphaVectors()
        result = npp._nova.pomdp_pbvi_execute_gpu(self.pomdpPtr, self, policy)
        if result != 0:
            print("Failed to execute the 'nova' library's GPU POMDP solver.")
            raise Exception()
        return policy

    def get_policy(self):
        policy = pav.POMDPAlphaVectors()
        result = npp._nova.pomdp_pbvi_get_policy_gpu(self.pomdpPtr, self, policy)
        if result != 0:
            raise RuntimeError("pomdp_pbvi_get_policy_gpu failed with code %d" % result)
        return policy

    def __str__(self):
        return "currentHorizon: %i\n\nnumThreads: %i\n\n" % (self.currentHorizon, self.numThreads)


def solve_batched(pomdps, scoring=npp.SCORING_FP16, hostThreads=0, GammaInitials=None, graph=False,
                  persistent=False):
    """ Solve independent POMDPs (each already copied to the device with
    initialize_gpu) with pomdp_pbvi_execute_batched_gpu (graph=True:
    pomdp_pbvi_execute_batched_graph_gpu, horizon loops replayed as CUDA
    graphs; persistent=True: pomdp_pbvi_execute_batched_persistent_gpu,
    lock-step backups with one persistent scoring launch for the batch);
    returns one POMDPAlphaVectors per POMDP, as each POMDPPBVIGPU(p).solve()
    would. """
    from . import pomdp_alpha_vectors as pav
    count = len(pomdps)
    solvers, bufs = [], []
    for k, p in enumerate(pomdps):
        s = npp.NovaPOMDPPBVIGPU()
        buf = _initial_gamma(p, None if GammaInitials is None else GammaInitials[k])
        bufs.append(buf)
        s.GammaInitial = ct.cast(buf, ct.POINTER(ct.c_float))
        s.numThreads = 1024
        s.currentHorizon = 0
        solvers.append(s)
    policies = [pav.POMDPAlphaVectors() for _ in range(count)]
    P = (ct.POINTER(pomdp.POMDP) * count)(*[ct.pointer(p) for p in pomdps])
    G = (ct.POINTER(npp.NovaPOMDPPBVIGPU) * count)(*[ct.pointer(s) for s in solvers])
    A = (ct.POINTER(npp._npav.NovaPOMDPAlphaVectors) * count)(*[ct.cast(ct.pointer(a),
                                                                         ct.POINTER(npp._npav.NovaPOMDPAlphaVectors))
                                                                 for a in policies])
    entry = (npp._nova.pomdp_pbvi_execute_batched_persistent_gpu if persistent else
             npp._nova.pomdp_pbvi_execute_batched_graph_gpu if graph else npp._nova.pomdp_pbvi_execute_batched_gpu)
    result = entry(P, G, A, count, int(scoring), int(hostThreads))
    _ = bufs
    if result != 0:
        raise RuntimeError("batched solve failed with code %d" % result)
    return policies
