"""The allocation-free V(b) entry point (pomdp_alpha_vectors_value_noalloc_gpu)
through the C ABI. Callers of the allocation-free form are those that cannot
call cudaMalloc while they run (real-time policy execution, or device memory
owned by another framework's pool), so besides agreeing with the existing
device evaluation (pomdp_pbvi_value_gpu) on two calls in a row, a call must
leave the device's free memory unchanged and must succeed while the next
device allocation of the library is armed to fail. Edge cases follow the
reference's evaluation (pomdp_alpha_vectors.cpp:52-79): the lowest index wins
ties, nothing above the -1e10 start gives V = -1e10 and action 0, and the
largest accepted alpha count works. This file is collected last so a
stop-at-first-failure run has already run every other test."""
import ctypes as ct

import numpy as np
import pytest

from nova_gb300 import synth
from nova_gb300 import _lib
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_pbvi import POMDPPBVIGPU

pytestmark = pytest.mark.gpu

MAX_ROWS = 65536


def _noalloc():
    lib = _lib.load()
    f = lib.pomdp_alpha_vectors_value_noalloc_gpu
    f.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint, ct.c_uint, ct.c_void_p, ct.POINTER(ct.c_double),
                  ct.POINTER(ct.c_uint)]
    lib.nova_gb300_inject_fault.argtypes = [ct.c_uint, ct.c_uint]
    return lib, f


def _call(f, d_gamma, d_pi, r, n, d_b):
    V = ct.c_double(0.0)
    a = ct.c_uint(0)
    rc = f(d_gamma, d_pi, r, n, d_b, ct.byref(V), ct.byref(a))
    return rc, V.value, a.value


def _fp64_value(G, pi, b):
    """V(b) in FP64 with the reference's rule: maximum from -1e10 with strict
    '>', lowest index on ties, action 0 when nothing beats the start."""
    vals = G.astype(np.float64) @ b.astype(np.float64)
    best, act = float(np.float32(-1e10)), 0
    for j, v in enumerate(vals):
        if v > best:
            best, act = float(v), int(pi[j])
    return best, act


def test_noalloc_value_matches_device_value_twice():
    torch = pytest.importorskip("torch")
    lib, f = _noalloc()
    m = synth.random_pomdp(n=160, m=5, z=6, ns=7, r=300, rz=9, gamma=0.95, horizon=4, seed=17)
    p = POMDP.from_arrays(m)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=m["GammaInitial"])
    for _ in range(m["horizon"]):
        alg.update()
    d_gamma = ct.cast(alg.d_Gamma if alg.currentHorizon % 2 == 0 else alg.d_GammaPrime, ct.c_void_p).value
    d_pi = ct.cast(alg.d_pi, ct.c_void_p).value
    beliefs = [torch.from_numpy(synth.dense_belief(m, i)).to("cuda") for i in (0, 7)]
    torch.cuda.synchronize()
    free0 = None
    for k, i in enumerate((0, 7)):  # two calls in a row, different beliefs
        V_ref, a_ref = alg.value(synth.dense_belief(m, i))
        torch.cuda.synchronize()
        if k == 1:
            # The first call resolved the scratch address. From here on a call
            # must not allocate: the library's next device allocation is armed
            # to fail, and the device's free memory must not move.
            free0 = torch.cuda.mem_get_info()[0]
            lib.nova_gb300_inject_fault(1, 1)
        try:
            rc, V, a = _call(f, d_gamma, d_pi, m["r"], m["n"], beliefs[k].data_ptr())
        finally:
            if k == 1:
                lib.nova_gb300_inject_fault(0, 0)
        assert rc == 0
        assert abs(V - V_ref) <= 1e-12 * max(1.0, abs(V_ref))
        assert a == a_ref
    for _ in range(5):
        assert _call(f, d_gamma, d_pi, m["r"], m["n"], beliefs[0].data_ptr())[0] == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    # sizes beyond the scratch are rejected before any device work
    assert _call(f, d_gamma, d_pi, MAX_ROWS + 1, m["n"], d_gamma)[0] == 1


def test_noalloc_ties_sentinel_and_largest_size():
    torch = pytest.importorskip("torch")
    _, f = _noalloc()
    rng = np.random.default_rng(5)
    n = 24
    b = rng.dirichlet(np.ones(n)).astype(np.float32)
    d_b = torch.from_numpy(b).to("cuda")
    # Ties: rows 3, 9 and 20 are the same alpha (the best one) with different
    # actions; the lowest index (3) must win.
    G = rng.uniform(-5.0, 0.0, size=(32, n)).astype(np.float32)
    G[3] = G[9] = G[20] = rng.uniform(1.0, 2.0, size=n).astype(np.float32)
    pi = np.arange(32, dtype=np.uint32) % 7
    pi[3], pi[9], pi[20] = 4, 5, 6
    d_G, d_pi = torch.from_numpy(G).to("cuda"), torch.from_numpy(pi.astype(np.int32)).to("cuda")
    torch.cuda.synchronize()
    rc, V, a = _call(f, d_G.data_ptr(), d_pi.data_ptr(), 32, n, d_b.data_ptr())
    V64, a64 = _fp64_value(G, pi, b)
    assert rc == 0 and a == a64 == 4
    assert abs(V - V64) <= 1e-12 * abs(V64)
    # Every alpha at or below the -1e10 start: V = -1e10 (as nova's FP32
    # sentinel) and action 0, whatever pi holds.
    Gs = np.full((40, n), -2e10, np.float32)
    Gs[11] = np.float32(-1.0001e10)  # just below the start
    pis = np.full(40, 3, np.uint32)
    d_Gs, d_pis = torch.from_numpy(Gs).to("cuda"), torch.from_numpy(pis.astype(np.int32)).to("cuda")
    torch.cuda.synchronize()
    rc, V, a = _call(f, d_Gs.data_ptr(), d_pis.data_ptr(), 40, n, d_b.data_ptr())
    V64, a64 = _fp64_value(Gs, pis, b)
    assert rc == 0 and a == a64 == 0
    assert V == V64 == float(np.float32(-1e10))
    # The largest accepted size, twice in a row.
    GL = rng.uniform(-1.0, 1.0, size=(MAX_ROWS, n)).astype(np.float32)
    piL = rng.integers(0, 9, size=MAX_ROWS).astype(np.uint32)
    d_GL, d_piL = torch.from_numpy(GL).to("cuda"), torch.from_numpy(piL.astype(np.int32)).to("cuda")
    V64, a64 = _fp64_value(GL, piL, b)
    torch.cuda.synchronize()
    for _ in range(2):
        rc, V, a = _call(f, d_GL.data_ptr(), d_piL.data_ptr(), MAX_ROWS, n, d_b.data_ptr())
        assert rc == 0 and a == a64
        assert abs(V - V64) <= 1e-12 * max(1.0, abs(V64))
