"""POMDP model object (python/nova/pomdp.py:40-402).

Same class, fields and methods as the reference wrapper. Arrays are owned by
the C library (pomdp_initialize_cpu allocates them); `set_arrays` fills them
from numpy in one copy per array instead of the reference's element loop.
File loading is not part of this library; belief-set expansion and the sigma
approximation run on the GPU.
"""
import ctypes as ct

import numpy as np

from . import nova_pomdp as npm


def _fill(ptr, values, ctype):
    values = np.ascontiguousarray(values, dtype=ctype)
    ct.memmove(ptr, values.ctypes.data, values.nbytes)


class POMDP(npm.NovaPOMDP):
    """ A Partially Observable Markov Decision Process (POMDP) object. """

    def __init__(self):
        self.n = int(0)
        self.ns = int(0)
        self.m = int(0)
        self.z = int(0)
        self.r = int(0)
        self.rz = int(0)
        self.gamma = float(0.9)
        self.horizon = int(1)
        self.S = ct.POINTER(ct.c_int)()
        self.T = ct.POINTER(ct.c_float)()
        self.O = ct.POINTER(ct.c_float)()
        self.R = ct.POINTER(ct.c_float)()
        self.Z = ct.POINTER(ct.c_int)()
        self.B = ct.POINTER(ct.c_float)()
        self.d_S = ct.POINTER(ct.c_int)()
        self.d_T = ct.POINTER(ct.c_float)()
        self.d_O = ct.POINTER(ct.c_float)()
        self.d_R = ct.POINTER(ct.c_float)()
        self.d_Z = ct.POINTER(ct.c_int)()
        self.d_B = ct.POINTER(ct.c_float)()
        self.Rmin = None
        self.Rmax = None
        self.cpuIsInitialized = False
        self.gpuIsInitialized = False

    def __del__(self):
        self.uninitialize_gpu()
        self.uninitialize()

    def initialize(self, n, ns, m, z, r, rz, gamma, horizon):
        """ Allocate the POMDP's arrays (pomdp_initialize_cpu). """
        if self.cpuIsInitialized:
            return
        result = npm._nova.pomdp_initialize_cpu(self, n, ns, m, z, r, rz, gamma, horizon)
        if result != 0:
            print("Failed to initialize the POMDP.")
            raise Exception()
        self.cpuIsInitialized = True

    def uninitialize(self):
        """ Free the POMDP's arrays (pomdp_uninitialize_cpu). """
        if not self.cpuIsInitialized:
            return
        result = npm._nova.pomdp_uninitialize_cpu(self)
        if result != 0:
            print("Failed to uninitialize the POMDP.")
            raise Exception()
        self.cpuIsInitialized = False

    def initialize_gpu(self):
        """ Upload the arrays to the GPU (pomdp_initialize_gpu). """
        if self.gpuIsInitialized:
            return
        result = npm._nova.pomdp_initialize_gpu(self)
        if result != 0:
            print("Failed to initialize the 'nova' library's GPU variables for the POMDP.")
            raise Exception()
        self.gpuIsInitialized = True

    def uninitialize_gpu(self):
        """ Free the GPU copies (pomdp_uninitialize_gpu). """
        if not self.gpuIsInitialized:
            return
        result = npm._nova.pomdp_uninitialize_gpu(self)
        if result != 0:
            print("Failed to uninitialize the 'nova' library's GPU variables for the POMDP.")
            raise Exception()
        self.gpuIsInitialized = False

    def set_arrays(self, S, T, O, R, Z, B, Rmin=None, Rmax=None):
        """ Copy numpy arrays (nova layouts) into the allocated C arrays. """
        _fill(self.S, S, np.int32)
        _fill(self.T, T, np.float32)
        _fill(self.O, O, np.float32)
        _fill(self.R, R, np.float32)
        _fill(self.Z, Z, np.int32)
        _fill(self.B, B, np.float32)
        R = np.asarray(R, dtype=np.float32)
        self.Rmin = float(R.min()) if Rmin is None else Rmin
        self.Rmax = float(R.max()) if Rmax is None else Rmax

    @classmethod
    def from_arrays(cls, model):
        """ Build a POMDP from a dict with n, ns, m, z, r, rz, gamma, horizon, S, T, O, R, Z, B. """
        p = cls()
        p.initialize(model["n"], model["ns"], model["m"], model["z"], model["r"], model["rz"], model["gamma"],
                     model["horizon"])
        p.set_arrays(model["S"], model["T"], model["O"], model["R"], model["Z"], model["B"])
        return p

    def load(self, filename, filetype='cassandra', scalarize=lambda x: x[0], rewardIndex=0):
        """ Load a POMDP file (pomdp.py:149-200 of the reference). 'cassandra' files are
            parsed by nova_load_cassandra_pomdp (C++, the rules of file_loader.py:211-588);
            'raw' files by nova_load_raw_pomdp (C++), keeping reward function rewardIndex (the
            reference's default scalarisation keeps the first; other scalarisations are not
            supported). """
        if filetype not in ('cassandra', 'raw'):
            print("Invalid file type '%s'." % (filetype))
            raise Exception()
        if self.S:
            raise RuntimeError("the POMDP already holds arrays")
        if filetype == 'cassandra':
            rmin, rmax = ct.c_double(0.0), ct.c_double(0.0)
            result = npm._nova.nova_load_cassandra_pomdp(str(filename).encode(), self, ct.byref(rmin),
                                                         ct.byref(rmax))
            if result != 0:
                print("Failed to load file '%s'." % (filename))
                raise Exception()
            self.Rmin = rmin.value
            self.Rmax = rmax.value
            return
        result = npm._nova.nova_load_raw_pomdp(str(filename).encode(), self, int(rewardIndex))
        if result != 0:
            print("Failed to load file '%s'." % (filename))
            raise Exception()
        R = np.ctypeslib.as_array(self.R, shape=(self.n * self.m,))
        self.Rmin = float(R.min())
        self.Rmax = float(R.max())

    def expand(self, method='random', numBeliefsToAdd=1000, pemaPolicy=None, pemaAlgorithm=None):
        """ Expand the belief points (pomdp.py:202-229 of the reference): 'random' trajectories
            (pomdp_expand_random_cpu), 'distinct_beliefs' (pomdp_expand_distinct_beliefs_cpu) or
            'pema' (pomdp_expand_pema_cpu, with pemaPolicy or pemaAlgorithm.solve()). """
        if method not in ["random", "distinct_beliefs", "pema"]:
            print("Failed to expand. Method '%s' is not defined." % (method))
            raise Exception()
        if method == "random":
            result = npm._nova.pomdp_expand_random_cpu(self, numBeliefsToAdd)
        elif method == "distinct_beliefs":
            result = npm._nova.pomdp_expand_distinct_beliefs_cpu(self)
        else:
            if pemaPolicy is None:
                pemaPolicy = pemaAlgorithm.solve()
            result = npm._nova.pomdp_expand_pema_cpu(self, ct.cast(ct.pointer(pemaPolicy),
                                                                   ct.POINTER(npm._npav.NovaPOMDPAlphaVectors)))
        if result != 0:
            raise RuntimeError("belief expansion '%s' failed with code %d" % (method, result))

    def sigma_approximate(self, numDesiredNonZeroValues=1):
        """ Sigma approximation of the beliefs (pomdp_sigma_cpu); returns sigma = min_b sigma_b. """
        sigma = ct.c_float(0.0)
        result = npm._nova.pomdp_sigma_cpu(self, numDesiredNonZeroValues, ct.byref(sigma))
        if result != 0:
            print("Failed to perform sigma-approximation.")
            raise Exception()
        return sigma.value

    def arrays(self):
        """ The model and belief arrays as numpy copies (dict of synth.py's layout). """
        def get(ptr, count, dtype):
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype).copy() if count else \
                np.zeros(0, dtype)
        n, ns, m, z, r, rz = self.n, self.ns, self.m, self.z, self.r, self.rz
        return dict(n=n, ns=ns, m=m, z=z, r=r, rz=rz, gamma=float(self.gamma), horizon=int(self.horizon),
                    S=get(self.S, n * m * ns, np.int32).reshape(n, m, ns),
                    T=get(self.T, n * m * ns, np.float32).reshape(n, m, ns),
                    O=get(self.O, m * n * z, np.float32).reshape(m, n, z),
                    R=get(self.R, n * m, np.float32).reshape(n, m),
                    Z=get(self.Z, r * rz, np.int32).reshape(r, rz),
                    B=get(self.B, r * rz, np.float32).reshape(r, rz))

    def belief_update(self, b, a, o):
        """ Belief update b' = normalise(O(a,.,o) * T(.,a,.)^T b) (pomdp_belief_update_cpu). """
        b = (ct.c_float * self.n)(*np.asarray(b, dtype=np.float32).ravel())
        bp = ct.POINTER(ct.c_float)()
        result = npm._nova.pomdp_belief_update_cpu(self, b, int(a), int(o), ct.byref(bp))
        if result != 0:
            print("Failed to perform a belief update on the CPU.")
            raise Exception()
        out = np.array([bp[s] for s in range(self.n)], dtype=np.float32)
        return out

    def __str__(self):
        def arr(ptr, count, shape):
            return np.array([ptr[i] for i in range(count)]).reshape(shape)
        result = "n:       %d\nns:      %d\nm:       %d\nz:       %d\nr:       %d\nrz:      %d\n" \
                 "horizon: %d\ngamma:   %s\n" % (self.n, self.ns, self.m, self.z, self.r, self.rz, self.horizon,
                                                 str(self.gamma))
        result += "S(s, a, s'):\n%s\n\n" % str(arr(self.S, self.n * self.m * self.ns, (self.n, self.m, self.ns)))
        result += "T(s, a, s'):\n%s\n\n" % str(arr(self.T, self.n * self.m * self.ns, (self.n, self.m, self.ns)))
        result += "O(a, s', o):\n%s\n\n" % str(arr(self.O, self.m * self.n * self.z, (self.m, self.n, self.z)))
        result += "R(s, a):\n%s\n\n" % str(arr(self.R, self.n * self.m, (self.n, self.m)))
        result += "Z(i, s):\n%s\n\n" % str(arr(self.Z, self.r * self.rz, (self.r, self.rz)))
        result += "B(i, s):\n%s\n\n" % str(arr(self.B, self.r * self.rz, (self.r, self.rz)))
        return result
