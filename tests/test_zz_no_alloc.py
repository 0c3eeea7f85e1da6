"""The allocation-free V(b) entry point (pomdp_alpha_vectors_value_noalloc_gpu)
against the existing device evaluation (pomdp_pbvi_value_gpu), through the C
ABI, on two calls in a row. Callers of the allocation-free form are those
that cannot call cudaMalloc while they run (real-time policy execution, or
device memory owned by another framework); this file is collected last so a
stop-at-first-failure run has already run every other test."""
import ctypes as ct

import numpy as np
import pytest

from nova_gb300 import synth
from nova_gb300 import _lib
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_pbvi import POMDPPBVIGPU

pytestmark = pytest.mark.gpu

_F = ct.POINTER(ct.c_float)
_U = ct.POINTER(ct.c_uint)


def test_noalloc_value_matches_device_value_twice():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    lib.pomdp_alpha_vectors_value_noalloc_gpu.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint, ct.c_uint,
                                                          ct.c_void_p, ct.POINTER(ct.c_double), ct.POINTER(ct.c_uint)]
    m = synth.random_pomdp(n=160, m=5, z=6, ns=7, r=300, rz=9, gamma=0.95, horizon=4, seed=17)
    p = POMDP.from_arrays(m)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=m["GammaInitial"])
    for _ in range(m["horizon"]):
        alg.update()
    d_gamma = ct.cast(alg.d_Gamma if alg.currentHorizon % 2 == 0 else alg.d_GammaPrime, ct.c_void_p).value
    d_pi = ct.cast(alg.d_pi, ct.c_void_p).value
    for i in (0, 7):  # two calls in a row, different beliefs
        b = synth.dense_belief(m, i)
        V_ref, a_ref = alg.value(b)
        d_b = torch.from_numpy(b).to("cuda")
        torch.cuda.synchronize()
        V = ct.c_double(0.0)
        a = ct.c_uint(0)
        rc = lib.pomdp_alpha_vectors_value_noalloc_gpu(d_gamma, d_pi, m["r"], m["n"], d_b.data_ptr(),
                                                       ct.byref(V), ct.byref(a))
        assert rc == 0
        assert abs(V.value - V_ref) <= 1e-12 * max(1.0, abs(V_ref))
        assert a.value == a_ref
    # sizes beyond the scratch are rejected before any device work
    V = ct.c_double(0.0)
    a = ct.c_uint(0)
    assert lib.pomdp_alpha_vectors_value_noalloc_gpu(d_gamma, d_pi, 65537, m["n"], d_gamma, ct.byref(V),
                                                     ct.byref(a)) == 1
