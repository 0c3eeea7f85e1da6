"""The oracle (oracle/nova_oracle.c) against the reference: golden fixtures
made by the reference's own CPU code, the reference's unit-test values, and
(where the reference library is built here) live cross-checks."""
import numpy as np
import pytest

from conftest import load_golden, bits, PBVI_GOLDENS, PERSEUS_GOLDENS, MDP_GOLDENS
from oracle import oracle as orc
from nova_gb300 import synth


@pytest.mark.parametrize("name", PBVI_GOLDENS)
def test_pbvi_loop_form_matches_reference(name):
    g = load_golden(name)
    if g["r"] * g["r"] * g["n"] * g["horizon"] > 2e8:
        pytest.skip("loop form too slow for this fixture; the factored form is checked below")
    G, pi = orc.pbvi_solve(g)
    np.testing.assert_array_equal(bits(G), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


@pytest.mark.parametrize("name", PBVI_GOLDENS)
def test_pbvi_factored_form_matches_reference(name):
    g = load_golden(name)
    G = g["GammaInitial"].copy()
    Gp = G.copy()
    pi = np.zeros(g["r"], np.uint32)
    for h in range(g["horizon"]):
        if h % 2 == 0:
            orc.pbvi_update(g, G, Gp, pi)
        else:
            orc.pbvi_update(g, Gp, G, pi)
    out = G if g["horizon"] % 2 == 0 else Gp
    np.testing.assert_array_equal(bits(out), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


@pytest.mark.parametrize("name", PERSEUS_GOLDENS)
def test_perseus_matches_reference(name):
    g = load_golden(name)
    G, pi = orc.perseus_solve(g, seed=g["out_srand"])
    np.testing.assert_array_equal(bits(G), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


@pytest.mark.parametrize("name", MDP_GOLDENS)
def test_mdp_vi_matches_reference(name):
    g = load_golden(name)
    V, pi = orc.mdp_vi_solve(g, VInitial=g.get("VInitial"))
    np.testing.assert_array_equal(bits(V), bits(g["out_V"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


def simple_mdp():
    """create_simple_mdp (tests/unit/mdp/mdp_tests.cpp:34-60)."""
    return dict(n=1, ns=1, m=1, gamma=float(np.float32(0.9)), horizon=3, S=np.array([[[0]]], np.int32),
                T=np.array([[[1.0]]], np.float32), R=np.array([[1.0]], np.float32))


def three_state_mdp():
    """create_three_state_mdp(false) (tests/unit/mdp/mdp_tests.cpp:63-153)."""
    S = np.array([[[0, 1], [0, -1]], [[1, -1], [2, -1]], [[2, -1], [2, -1]]], np.int32)
    T = np.array([[[0.5, 0.5], [1.0, 0.0]], [[1.0, 0.0], [1.0, 0.0]], [[1.0, 0.0], [1.0, 0.0]]], np.float32)
    R = np.array([[-1.0, -2.0], [-1.0, -2.0], [0.0, 0.0]], np.float32)
    return dict(n=3, ns=2, m=2, gamma=float(np.float32(0.9)), horizon=5, S=S, T=T, R=R)


def test_mdp_reference_unit_values():
    # mdp_vi_cpu_tests.cpp:171 and :229-237
    V, pi = orc.mdp_vi_solve(simple_mdp())
    assert abs(V[0] - 2.71) < 1e-5 and pi[0] == 0
    V, pi = orc.mdp_vi_solve(three_state_mdp())
    np.testing.assert_allclose(V, [-3.303775, -2.0, 0.0], atol=1e-5)
    assert pi[0] == 0 and pi[1] == 1
    # per-step values, mdp_vi_cpu_tests.cpp:398-415 (0 -> 1 -> 1.9 -> 2.71)
    m = simple_mdp()
    V = np.zeros(1, np.float32)
    for expect in (1.0, 1.9, 2.71):
        V, _ = orc.mdp_vi_sweep(m, V)
        assert abs(V[0] - expect) < 1e-5
    # three-state per-step values, mdp_vi_cpu_tests.cpp:444-479
    m = three_state_mdp()
    V = np.zeros(3, np.float32)
    for expect, epi in (([-1.0, -1.0, 0.0], [0, 0]), ([-1.9, -1.9, 0.0], [0, 0]), ([-2.71, -2.0, 0.0], [0, 1])):
        V, pi = orc.mdp_vi_sweep(m, V)
        np.testing.assert_allclose(V, expect, atol=1e-5)
        assert list(pi[:2]) == epi


def test_alpha_vector_reference_unit_values():
    # pomdp_alpha_vectors_tests.cpp:35-89
    G = np.array([[1.0, 0.0], [0.0, 1.0]], np.float32)
    pi = np.array([1, 0], np.uint32)
    for b, v, a in (([0.0, 1.0], 1.0, 0), ([1.0, 0.0], 1.0, 1), ([0.25, 0.75], 0.75, 0), ([0.67, 0.33], 0.67, 1)):
        V, act = orc.alpha_value(G, pi, np.array(b, np.float32))
        assert abs(V - v) < 1e-5 and act == a
    V, _ = orc.alpha_value(G, pi, np.array([0.5, 0.5], np.float32))
    assert abs(V - 0.5) < 1e-5


@pytest.mark.skipif(not orc.ref_available(), reason="reference sources not present on this machine")
@pytest.mark.parametrize("seed", [101, 102, 103])
def test_live_against_reference_library(seed):
    m = synth.random_pomdp(n=29, m=3, z=6, ns=5, r=31, rz=5, gamma=0.93, horizon=7, seed=seed)
    G1, p1 = orc.ref_pbvi_solve(m)
    G2, p2 = orc.pbvi_solve(m)
    np.testing.assert_array_equal(bits(G1), bits(G2))
    np.testing.assert_array_equal(p1, p2)
    G1, p1 = orc.ref_perseus_solve(m, seed=seed)
    G2, p2 = orc.perseus_solve(m, seed=seed)
    np.testing.assert_array_equal(bits(G1), bits(G2))
    np.testing.assert_array_equal(p1, p2)
    md = synth.random_mdp(n=200, m=5, ns=7, gamma=0.9, horizon=13, seed=seed)
    V1, q1 = orc.ref_mdp_vi_solve(md)
    V2, q2 = orc.mdp_vi_solve(md)
    np.testing.assert_array_equal(bits(V1), bits(V2))
    np.testing.assert_array_equal(q1, q2)


@pytest.mark.skipif(not orc.ref_available(), reason="reference sources not present on this machine")
def test_mdp_nan_inf_and_ties_against_reference_library():
    """Rewards with NaN (at action 0 and later actions), +-inf and exact ties:
    the oracle's VI keeps the reference's semantics (a NaN at action 0 stays,
    later NaNs lose every strict comparison), bit for bit with the payloads."""
    md = synth.random_mdp(n=400, m=6, ns=5, gamma=0.9, horizon=3, seed=77)
    R = md["R"].copy()
    rng = np.random.default_rng(77)
    rows = rng.choice(md["n"], 40, replace=False)
    R[rows[:2], 0] = np.nan
    R[rows[2:12], rng.integers(1, 6, 10)] = np.nan
    R[rows[12:20], rng.integers(0, 6, 8)] = np.inf
    R[rows[20:28], rng.integers(0, 6, 8)] = -np.inf
    R[rows[28:], :] = 0.25
    md["R"] = R
    V1, q1 = orc.ref_mdp_vi_solve(md)
    V2, q2 = orc.mdp_vi_solve(md)
    assert np.isnan(V1).any() and not np.isnan(V1).all()
    np.testing.assert_array_equal(bits(V1), bits(V2))
    np.testing.assert_array_equal(q1, q2)


def test_oracle_detects_a_planted_mistake():
    """A perturbed model must change the oracle's answer (the checker is not vacuous)."""
    g = load_golden("pbvi_n64_h5")
    bad = dict(g)
    bad["R"] = g["R"].copy()
    bad["R"][3, 1] += np.float32(1e-3)
    G, _ = orc.pbvi_solve(bad)
    assert not np.array_equal(bits(G), bits(g["out_Gamma"]))


def test_fixed_selection_reverse_matches_finite_differences():
    """The oracle's FP64 reverse mode of recorded PBVI backups against central
    finite differences (h = 1e-6) of its FP64 forward, on R, T and O."""
    model = synth.random_pomdp(n=24, m=3, z=4, ns=5, r=40, rz=6, gamma=0.95, horizon=8, seed=3)
    b0 = np.full(model["n"], 1.0 / model["n"])
    G_H, acts, sels = orc.pbvi_record(model, 8)
    V, dR, dT, dO, dG = orc.pbvi_fixed_reverse_f64(model, model["GammaInitial"], acts, sels, b0)
    V2, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0)
    assert V == V2
    # FP32 alphas of the recorded run against the same selections in FP64
    assert abs(np.max(G_H.astype(np.float64) @ b0) - V) < 1e-5
    rng = np.random.default_rng(0)
    h = 1e-6
    for name, grad in (("R", dR), ("T", dT), ("O", dO)):
        arr = model[name]
        for _ in range(6):
            idx = tuple(int(rng.integers(0, d)) for d in arr.shape)
            A = arr.astype(np.float64).copy()
            A[idx] += h
            Vp, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, **{name: A})
            A[idx] -= 2 * h
            Vm, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, **{name: A})
            fd = (Vp - Vm) / (2 * h)
            assert abs(fd - grad[idx]) <= 1e-6 * max(1.0, abs(fd)), (name, idx, fd, grad[idx])


def _model_of(g):
    return {k: g[k] for k in ("n", "ns", "m", "z", "r", "rz", "gamma", "horizon", "S", "T", "O", "R", "Z", "B")}


@pytest.mark.parametrize("name", ["expand_distinct", "expand_distinct_ragged"])
def test_expand_distinct_matches_reference(name):
    g = load_golden(name)
    m = _model_of(g)
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_distinct(m))
    np.testing.assert_array_equal(Z, g["out_Z"])
    np.testing.assert_array_equal(bits(B), bits(g["out_B"]))


def test_expand_random_matches_reference():
    g = load_golden("expand_random")
    m = _model_of(g)
    Bn = orc.expand_random(m, int(g["out_num"]), int(g["out_srand"]))
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], Bn)
    np.testing.assert_array_equal(Z, g["out_Z"])
    np.testing.assert_array_equal(bits(B), bits(g["out_B"]))
    g = load_golden("expand_random_b0")
    Bn, nz = orc.expand_random_from_b0(_model_of(g), int(g["out_num"]), int(g["out_srand"]))
    np.testing.assert_array_equal(bits(Bn), bits(g["out_Bnew"]))
    assert nz == int(g["out_maxNonZero"])


def test_expand_pema_and_sigma_match_reference():
    g = load_golden("expand_pema")
    m = _model_of(g)
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_pema(m, g["out_policyGamma"])[None, :])
    np.testing.assert_array_equal(Z, g["out_Z"])
    np.testing.assert_array_equal(bits(B), bits(g["out_B"]))
    g = load_golden("sigma_k3")
    Z, B, sigma = orc.sigma_approximate(_model_of(g), int(g["out_k"]))
    np.testing.assert_array_equal(Z, g["out_Z"])
    np.testing.assert_array_equal(bits(B), bits(g["out_B"]))
    assert np.float32(sigma) == g["out_sigma"]


def test_belief_update_matches_reference_when_present():
    if not orc.ref_available():
        pytest.skip("reference library not built")
    m = synth.random_pomdp(n=30, m=3, z=4, ns=5, r=8, rz=6, gamma=0.9, horizon=4, seed=8)
    b = synth.dense_belief(m, 2)
    L, p = orc._ref_pomdp_owned(m)
    import ctypes as ct
    L.pomdp_belief_update_cpu.argtypes = [ct.POINTER(orc._RefPOMDP), ct.POINTER(ct.c_float), ct.c_uint, ct.c_uint,
                                          ct.POINTER(ct.POINTER(ct.c_float))]
    for a, o in ((0, 0), (2, 3), (1, 1)):
        bp = ct.POINTER(ct.c_float)()
        rc = L.pomdp_belief_update_cpu(ct.byref(p), b.ctypes.data_as(ct.POINTER(ct.c_float)), a, o, ct.byref(bp))
        ref = np.ctypeslib.as_array(bp, shape=(m["n"],)).copy()
        ours, ok = orc.belief_update(m, b, a, o)
        assert ok == (rc == 0)
        np.testing.assert_array_equal(bits(ours), bits(ref))
    L.pomdp_uninitialize_cpu(ct.byref(p))
