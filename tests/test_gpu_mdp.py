"""MDP value iteration on the GB300 through the C ABI."""
import ctypes as ct

import numpy as np
import pytest

from conftest import load_golden, bits, MDP_GOLDENS
from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300.mdp import MDP
from nova_gb300.mdp_vi import MDPValueIterationGPU, MDPValueIterationCPU
from nova_gb300 import nova_mdp_vi as nmvi

pytestmark = pytest.mark.gpu


def gpu_solve(model, VInitial=None):
    m = MDP.from_arrays(model)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=VInitial if VInitial is not None else np.zeros(model["n"], np.float32))
    pol = alg.solve()
    return pol.V_array(), pol.pi_array()


@pytest.mark.parametrize("name", MDP_GOLDENS)
def test_execute_gpu_matches_reference(name):
    g = load_golden(name)
    V, pi = gpu_solve(g, g.get("VInitial"))
    np.testing.assert_array_equal(bits(V), bits(g["out_V"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


@pytest.mark.parametrize("name", MDP_GOLDENS)
def test_execute_cpu_api_matches_reference(name):
    g = load_golden(name)
    m = MDP.from_arrays(g)
    alg = MDPValueIterationCPU(m, Vinitial=g.get("VInitial", np.zeros(g["n"], np.float32)))
    pol = alg.solve()
    np.testing.assert_array_equal(bits(pol.V_array()), bits(g["out_V"]))
    np.testing.assert_array_equal(pol.pi_array(), g["out_pi"])


def three_state():
    S = np.array([[[0, 1], [0, -1]], [[1, -1], [2, -1]], [[2, -1], [2, -1]]], np.int32)
    T = np.array([[[0.5, 0.5], [1.0, 0.0]], [[1.0, 0.0], [1.0, 0.0]], [[1.0, 0.0], [1.0, 0.0]]], np.float32)
    R = np.array([[-1.0, -2.0], [-1.0, -2.0], [0.0, 0.0]], np.float32)
    return dict(n=3, ns=2, m=2, gamma=0.9, horizon=5, S=S, T=T, R=R, goals=np.array([2], np.uint32))


def test_reference_unit_values_gpu():
    # mdp_vi_gpu_tests.cpp:226-228 (V = -3.303775, -2.0, 0.0; pi = 0, 1)
    V, pi = gpu_solve(three_state())
    np.testing.assert_allclose(V, [-3.303775, -2.0, 0.0], atol=1e-5)
    assert pi[0] == 0 and pi[1] == 1
    simple = dict(n=1, ns=1, m=1, gamma=0.9, horizon=3, S=np.array([[[0]]], np.int32),
                  T=np.array([[[1.0]]], np.float32), R=np.array([[1.0]], np.float32))
    V, pi = gpu_solve(simple)
    assert abs(V[0] - 2.71) < 1e-5


def test_update_cpu_per_step_host_arrays():
    """mdp_vi_cpu_tests.cpp:444-479: V and V' after each update, read from the struct."""
    mm = three_state()
    m = MDP.from_arrays(mm)
    alg = MDPValueIterationCPU(m, Vinitial=np.zeros(3, np.float32))
    f = nmvi._nova
    expect = [([0, 0, 0], [-1, -1, 0]), ([-1.9, -1.9, 0], [-1, -1, 0]), ([-1.9, -1.9, 0], [-2.71, -2.0, 0])]
    for h, (v, vp) in enumerate(expect):
        assert f.mdp_vi_update_cpu(alg.mdpPtr, alg) == 0
        assert alg.currentHorizon == h + 1
        np.testing.assert_allclose([alg.V[i] for i in range(3)], v, atol=1e-5)
        np.testing.assert_allclose([alg.Vprime[i] for i in range(3)], vp, atol=1e-5)


def test_update_gpu_matches_oracle_sweeps():
    md = synth.random_mdp(n=5000, m=7, ns=9, gamma=0.97, horizon=30, seed=4)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    V = np.zeros(md["n"], np.float32)
    for h in range(5):
        assert nmvi._nova.mdp_vi_update_gpu(alg.mdpPtr, alg) == 0
        Vn, pi = orc.mdp_vi_sweep(md, V)
        resid = ct.c_double(0)
        assert nmvi._nova.mdp_vi_residual_gpu(alg.mdpPtr, alg, ct.byref(resid)) == 0
        assert resid.value == np.max(np.abs(Vn.astype(np.float64) - V.astype(np.float64)))
        V = Vn
    from nova_gb300 import mdp_value_function as mvf
    pol = mvf.MDPValueFunction()
    assert nmvi._nova.mdp_vi_get_policy_gpu(alg.mdpPtr, alg, pol) == 0
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("m_actions", [1, 3, 8, 33])
def test_action_counts_and_until_converged(m_actions):
    md = synth.random_mdp(n=777, m=m_actions, ns=4, gamma=0.9, horizon=400, seed=m_actions)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    pol, sweeps, resid = alg.solve_until_converged(tol=1e-4, maxSweeps=400)
    assert resid < 1e-4 and 0 < sweeps < 400
    V, pi = orc.mdp_vi_solve(md, horizon=sweeps, VInitial=np.zeros(md["n"], np.float32))
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)
    Vprev, _ = orc.mdp_vi_solve(md, horizon=sweeps - 1, VInitial=np.zeros(md["n"], np.float32))
    assert resid == np.max(np.abs(V.astype(np.float64) - Vprev.astype(np.float64)))


# ---------------------------------------------------------------------------
# Column-tiled sweep (shared-memory V tiles; rows with ascending successors)
# ---------------------------------------------------------------------------

@pytest.fixture
def tiling():
    from nova_gb300 import mdp_vi
    yield mdp_vi
    mdp_vi.set_tiling(nmvi.TILING_AUTO, 0)


def ragged_sorted_mdp(n, m, ns, seed, gamma=0.95, horizon=10):
    """Random MDP whose rows keep ascending successors but stop early (-1),
    including rows with no successor at all."""
    md = synth.random_mdp(n=n, m=m, ns=ns, gamma=gamma, horizon=horizon, seed=seed)
    rng = np.random.default_rng(seed + 100)
    lens = rng.integers(0, ns + 1, size=(n, m))
    cut = np.arange(ns)[None, None, :] >= lens[:, :, None]
    md["S"] = np.where(cut, -1, md["S"]).astype(np.int32)
    md["T"] = np.where(cut, 0.0, md["T"]).astype(np.float32)
    return md


@pytest.mark.parametrize("n,m_actions,ns,tile", [(3000, 5, 12, 256), (1000, 1, 7, 64), (999, 33, 5, 100), (700, 3, 20, 0),
                                                 (4097, 8, 16, 0)])
def test_tiled_sweeps_match_oracle(tiling, n, m_actions, ns, tile):
    tiling.set_tiling(nmvi.TILING_ALWAYS, tile)
    md = ragged_sorted_mdp(n, m_actions, ns, seed=n + m_actions)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    V = np.zeros(md["n"], np.float32)
    for h in range(6):
        assert nmvi._nova.mdp_vi_update_gpu(alg.mdpPtr, alg) == 0
        assert tiling.tiling_status(alg) == 1
        Vn, pi = orc.mdp_vi_sweep(md, V)
        resid = ct.c_double(0)
        assert nmvi._nova.mdp_vi_residual_gpu(alg.mdpPtr, alg, ct.byref(resid)) == 0
        assert resid.value == np.max(np.abs(Vn.astype(np.float64) - V.astype(np.float64)))
        V = Vn
    from nova_gb300 import mdp_value_function as mvf
    pol = mvf.MDPValueFunction()
    assert nmvi._nova.mdp_vi_get_policy_gpu(alg.mdpPtr, alg, pol) == 0
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("mode", [nmvi.TILING_NEVER, nmvi.TILING_ALWAYS])
@pytest.mark.parametrize("n,m_actions,ns", [(1, 1, 1), (2, 3, 2), (5, 1, 5), (70, 2, 70)])
def test_degenerate_shapes_both_sweeps(tiling, mode, n, m_actions, ns):
    """One state, one action, one successor, and dense successor lists
    (ns = n), with the per-row and the column-tiled sweep (64-state tiles;
    a row with more than 31 successors inside one tile keeps the per-row
    sweep)."""
    tiling.set_tiling(mode, 64)
    md = synth.random_mdp(n=n, m=m_actions, ns=ns, gamma=0.9, horizon=7, seed=n)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    pol = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
    assert tiling.tiling_status() == (2 if mode == nmvi.TILING_NEVER or ns > 31 else 1)
    V, pi = orc.mdp_vi_solve(md, horizon=7, VInitial=np.zeros(md["n"], np.float32))
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)


def test_tiled_execute_until_converged_and_cpu_api(tiling):
    tiling.set_tiling(nmvi.TILING_ALWAYS, 512)
    md = ragged_sorted_mdp(2500, 4, 6, seed=9, gamma=0.9, horizon=40)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    V, pi = orc.mdp_vi_solve(md, horizon=40, VInitial=np.zeros(md["n"], np.float32))
    pol = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
    assert tiling.tiling_status() == 1
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)
    pol = MDPValueIterationCPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
    assert tiling.tiling_status() == 1
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)
    pol, sweeps, resid = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve_until_converged(
        tol=1e-4, maxSweeps=300)
    assert resid < 1e-4 and 0 < sweeps < 300
    V, pi = orc.mdp_vi_solve(md, horizon=sweeps, VInitial=np.zeros(md["n"], np.float32))
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)


def test_unsorted_rows_keep_gather_sweep(tiling):
    tiling.set_tiling(nmvi.TILING_ALWAYS, 256)
    md = synth.random_mdp(n=1500, m=3, ns=8, gamma=0.95, horizon=12, seed=21)
    rng = np.random.default_rng(5)
    perm = rng.permuted(np.broadcast_to(np.arange(8), md["S"].shape), axis=2)
    md["S"] = np.take_along_axis(md["S"], perm, axis=2).astype(np.int32)
    md["T"] = np.take_along_axis(md["T"], perm, axis=2).astype(np.float32)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    assert nmvi._nova.mdp_vi_update_gpu(alg.mdpPtr, alg) == 0
    assert tiling.tiling_status(alg) == 2
    pol = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
    V, pi = orc.mdp_vi_solve(md, horizon=12, VInitial=np.zeros(md["n"], np.float32))
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V))
    np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("n,m_actions,ns,tile", [(60000, 32, 4, 16384), (300000, 5, 6, 16384),
                                                 (100000, 16, 5, 16384), (500000, 3, 4, 16384),
                                                 (250000, 24, 4, 8192), (30000, 64, 3, 16384)])
def test_tiled_equals_gather_multi_wave(tiling, n, m_actions, ns, tile):
    """Models large enough for several source blocks per CTA at this tile
    size (more than one block of Q per SM's shared memory), so every CTA
    carries its V ring, R copies and scans across block boundaries; m covers
    the warp scan (powers of two up to 32) and the per-thread scan (5, 3, 24,
    64), and n = 30000 has fewer tiles than ring stages. Six tiled sweeps
    equal six per-row sweeps bit for bit."""
    md = synth.random_mdp(n=n, m=m_actions, ns=ns, gamma=0.95, horizon=6, seed=n + m_actions)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    out = {}
    for mode in (nmvi.TILING_ALWAYS, nmvi.TILING_NEVER):
        tiling.set_tiling(mode, tile)
        pol = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
        out[mode] = (pol.V_array().copy(), pol.pi_array().copy(), tiling.tiling_status())
    assert out[nmvi.TILING_ALWAYS][2] == 1 and out[nmvi.TILING_NEVER][2] == 2
    np.testing.assert_array_equal(bits(out[nmvi.TILING_ALWAYS][0]), bits(out[nmvi.TILING_NEVER][0]))
    np.testing.assert_array_equal(out[nmvi.TILING_ALWAYS][1], out[nmvi.TILING_NEVER][1])


def test_tiled_equals_gather_at_full_size(tiling):
    """n = 2^20, m = 8, ns = 16: the tiled sweep (chosen automatically) and the
    per-row sweep give the same bits after 12 sweeps, and the first sweep
    equals the oracle's."""
    cfg = synth.MDP_CONFIGS["vi_n1m"]
    md = synth.random_mdp(n=cfg["n"], m=cfg["m"], ns=cfg["ns"], gamma=cfg["gamma"], horizon=12, seed=0)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    out = {}
    for mode in (nmvi.TILING_AUTO, nmvi.TILING_NEVER):
        tiling.set_tiling(mode, 0)
        pol = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve()
        out[mode] = (pol.V_array().copy(), pol.pi_array().copy(), tiling.tiling_status())
    assert out[nmvi.TILING_AUTO][2] == 1 and out[nmvi.TILING_NEVER][2] == 2
    np.testing.assert_array_equal(bits(out[nmvi.TILING_AUTO][0]), bits(out[nmvi.TILING_NEVER][0]))
    np.testing.assert_array_equal(out[nmvi.TILING_AUTO][1], out[nmvi.TILING_NEVER][1])
    tiling.set_tiling(nmvi.TILING_AUTO, 0)
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    assert nmvi._nova.mdp_vi_update_gpu(alg.mdpPtr, alg) == 0
    from nova_gb300 import mdp_value_function as mvf
    pol = mvf.MDPValueFunction()
    assert nmvi._nova.mdp_vi_get_policy_gpu(alg.mdpPtr, alg, pol) == 0
    V1, pi1 = orc.mdp_vi_sweep(md, np.zeros(md["n"], np.float32))
    np.testing.assert_array_equal(bits(pol.V_array()), bits(V1))
    np.testing.assert_array_equal(pol.pi_array(), pi1)


@pytest.mark.parametrize("m_actions", [8, 5, 16])
def test_tiled_scan_nan_inf_and_ties(tiling, m_actions):
    """Rewards with NaN, +-inf and exact ties: the tiled sweep's action scan
    (rotated reads for power-of-two m, the reference's strict '>' in action
    order, a NaN at action 0 kept) and its residual (NaN differences skipped,
    as fmax skips them) equal the oracle's sweeps bit for bit."""
    tiling.set_tiling(nmvi.TILING_ALWAYS, 512)
    md = synth.random_mdp(n=3000, m=m_actions, ns=6, gamma=0.9, horizon=3, seed=31 + m_actions)
    R = md["R"].copy()
    rng = np.random.default_rng(m_actions)
    rows = rng.choice(md["n"], 60, replace=False)
    R[rows[:3], 0] = np.nan
    R[rows[15:30], rng.integers(1, m_actions, 15)] = np.nan
    R[rows[30:40], rng.integers(0, m_actions, 10)] = np.inf
    R[rows[40:50], rng.integers(0, m_actions, 10)] = -np.inf
    R[rows[50:], :] = 0.25  # every action ties before the successor terms
    md["R"] = R
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    alg = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
    V = np.zeros(md["n"], np.float32)
    for h in range(3):
        assert nmvi._nova.mdp_vi_update_gpu(alg.mdpPtr, alg) == 0
        assert tiling.tiling_status(alg) == 1
        Vn, pi = orc.mdp_vi_sweep(md, V)
        resid = ct.c_double(0)
        assert nmvi._nova.mdp_vi_residual_gpu(alg.mdpPtr, alg, ct.byref(resid)) == 0
        with np.errstate(invalid="ignore"):
            d = np.abs(Vn.astype(np.float64) - V.astype(np.float64))
        d = d[~np.isnan(d)]
        assert resid.value == (np.max(d) if d.size else 0.0)
        V = Vn
    from nova_gb300 import mdp_value_function as mvf
    pol = mvf.MDPValueFunction()
    assert nmvi._nova.mdp_vi_get_policy_gpu(alg.mdpPtr, alg, pol) == 0
    Vg = pol.V_array()
    # NaN payloads differ between the GPU (canonical NaN) and x86; NaN
    # positions and every other bit must match.
    nan = np.isnan(V)
    assert nan.any() and not nan.all()
    np.testing.assert_array_equal(np.isnan(Vg), nan)
    np.testing.assert_array_equal(bits(Vg[~nan]), bits(V[~nan]))
    np.testing.assert_array_equal(pol.pi_array(), pi)
