"""MDP model object (python/nova/mdp.py:40-305), without the file loader and
the legacy `solve` (use MDPValueIterationCPU / MDPValueIterationGPU; the
reference's `solve` calls mdp_vi_complete_* functions that its own library
does not export, and time.clock, which Python 3.8 removed)."""
import ctypes as ct

import numpy as np

from . import nova_mdp as nm
from .pomdp import _fill


class MDP(nm.NovaMDP):
    """ A Markov Decision Process (MDP) object. """

    def __init__(self):
        self.n = int(0)
        self.ns = int(0)
        self.m = int(0)
        self.gamma = float(0.9)
        self.horizon = int(1)
        self.epsilon = float(0.01)
        self.s0 = int(0)
        self.ng = int(0)
        self.goals = ct.POINTER(ct.c_uint)()
        self.S = ct.POINTER(ct.c_int)()
        self.T = ct.POINTER(ct.c_float)()
        self.R = ct.POINTER(ct.c_float)()
        self.d_goals = ct.POINTER(ct.c_uint)()
        self.d_S = ct.POINTER(ct.c_int)()
        self.d_T = ct.POINTER(ct.c_float)()
        self.d_R = ct.POINTER(ct.c_float)()
        self.Rmin = None
        self.Rmax = None
        self.cpuIsInitialized = False
        self.gpuIsInitialized = False

    def __del__(self):
        self.uninitialize_gpu()
        self.uninitialize()

    def __str__(self):
        """ The model's sizes and host arrays as text (arrays shown once allocated). """
        def arr(ptr, count, shape):
            return str(np.array([ptr[i] for i in range(count)]).reshape(shape)) if ptr else "(none)"
        n, m, ns = int(self.n), int(self.m), int(self.ns)
        goals = [int(self.goals[i]) for i in range(int(self.ng))] if self.goals else []
        result = "n:       %d\nm:       %d\nns:      %d\ns0:      %d\ngoals:   %s\nhorizon: %d\ngamma:   %s\n\n" % (
            n, m, ns, int(self.s0), str(goals), int(self.horizon), str(self.gamma))
        result += "S(s, a, s'):\n%s\n\n" % arr(self.S, n * m * ns, (n, m, ns))
        result += "T(s, a, s'):\n%s\n\n" % arr(self.T, n * m * ns, (n, m, ns))
        result += "R(s, a):\n%s\n\n" % arr(self.R, n * m, (n, m))
        return result

    def initialize(self, n, ns, m, gamma, horizon, epsilon, s0, ng):
        """ Allocate the MDP's arrays (mdp_initialize_cpu). """
        if self.cpuIsInitialized:
            return
        result = nm._nova.mdp_initialize_cpu(self, n, ns, m, gamma, horizon, epsilon, s0, ng)
        if result != 0:
            print("Failed to initialize the MDP.")
            raise Exception()
        self.cpuIsInitialized = True

    def uninitialize(self):
        if not self.cpuIsInitialized:
            return
        result = nm._nova.mdp_uninitialize_cpu(self)
        if result != 0:
            print("Failed to uninitialize the MDP.")
            raise Exception()
        self.cpuIsInitialized = False

    def initialize_gpu(self):
        """ Upload S, T, R (and goals) to the GPU (python/nova/mdp.py:119-136). """
        if self.gpuIsInitialized:
            return
        result = nm._nova.mdp_initialize_successors_gpu(self)
        result += nm._nova.mdp_initialize_state_transitions_gpu(self)
        result += nm._nova.mdp_initialize_rewards_gpu(self)
        if self.ng > 0:
            result += nm._nova.mdp_initialize_goals_gpu(self)
        if result != 0:
            print("Failed to initialize the 'nova' library's GPU variables for the MDP.")
            raise Exception()
        self.gpuIsInitialized = True

    def uninitialize_gpu(self):
        if not self.gpuIsInitialized:
            return
        result = nm._nova.mdp_uninitialize_successors_gpu(self)
        result += nm._nova.mdp_uninitialize_state_transitions_gpu(self)
        result += nm._nova.mdp_uninitialize_rewards_gpu(self)
        if self.ng > 0:
            result += nm._nova.mdp_uninitialize_goals_gpu(self)
        if result != 0:
            print("Failed to uninitialize the 'nova' library's GPU variables for the MDP.")
            raise Exception()
        self.gpuIsInitialized = False

    def set_arrays(self, S, T, R, goals=None):
        """ Copy numpy arrays (nova layouts) into the allocated C arrays. """
        _fill(self.S, S, np.int32)
        _fill(self.T, T, np.float32)
        _fill(self.R, R, np.float32)
        if goals is not None and self.ng > 0:
            _fill(self.goals, goals, np.uint32)
        R = np.asarray(R, dtype=np.float32)
        self.Rmin = float(R.min())
        self.Rmax = float(R.max())

    @classmethod
    def from_arrays(cls, model, epsilon=0.0001, s0=0, ng=0):
        p = cls()
        p.initialize(model["n"], model["ns"], model["m"], model["gamma"], model["horizon"], epsilon, s0, ng)
        p.set_arrays(model["S"], model["T"], model["R"], model.get("goals"))
        return p

    def load(self, filename, filetype='cassandra', scalarize=lambda x: x[0], rewardIndex=0):
        """ Load an MDP file (mdp.py of the reference). 'raw' files are parsed by
            nova_load_raw_mdp (C++), keeping reward function rewardIndex. """
        if filetype != 'raw':
            raise NotImplementedError("nova-gb300 parses raw files only; use set_arrays() for others")
        if self.S:
            raise RuntimeError("the MDP already holds arrays")
        result = nm._nova.nova_load_raw_mdp(str(filename).encode(), self, int(rewardIndex))
        if result != 0:
            print("Failed to load file '%s'." % (filename))
            raise Exception()
        R = np.ctypeslib.as_array(self.R, shape=(self.n * self.m,))
        self.Rmin = float(R.min())
        self.Rmax = float(R.max())
