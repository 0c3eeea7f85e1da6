"""PBVI on the GB300 through the C ABI (nova_gb300's ctypes wrapper):
bit-identical to the reference's outputs (golden fixtures) and to the oracle."""
import ctypes as ct

import numpy as np
import pytest

from conftest import load_golden, bits, PBVI_GOLDENS
from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_pbvi import POMDPPBVIGPU, POMDPPBVICPU
from nova_gb300 import nova_pomdp_pbvi as npp

pytestmark = pytest.mark.gpu

MODES = [npp.SCORING_EXACT, npp.SCORING_BF16, npp.SCORING_FP16]


def solve_gpu(model, mode, horizon=None):
    p = POMDP.from_arrays(dict(model, horizon=model["horizon"] if horizon is None else horizon))
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=model["GammaInitial"])
    alg.set_scoring(mode)
    pol = alg.solve()
    return pol.gamma_array(), pol.pi_array()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", PBVI_GOLDENS)
def test_execute_gpu_matches_reference(name, mode):
    g = load_golden(name)
    G, pi = solve_gpu(g, mode)
    np.testing.assert_array_equal(bits(G), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pi, g["out_pi"])


@pytest.mark.parametrize("name", ["pbvi_n64_h5", "pbvi_ragged", "pbvi_tiger"])
def test_execute_cpu_api_matches_reference(name):
    g = load_golden(name)
    p = POMDP.from_arrays(g)
    alg = POMDPPBVICPU(p, GammaInitial=g["GammaInitial"])
    pol = alg.solve()
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pol.pi_array(), g["out_pi"])


def test_stepwise_update_cpu_api_host_arrays():
    """update_cpu leaves valid host arrays after every call (the reference's contract)."""
    g = load_golden("pbvi_ragged")
    p = POMDP.from_arrays(g)
    alg = POMDPPBVICPU(p, GammaInitial=g["GammaInitial"])
    G = g["GammaInitial"].copy()
    Gp = G.copy()
    pi = np.zeros(g["r"], np.uint32)
    r, n = g["r"], g["n"]
    for h in range(4):
        alg.update()
        if h % 2 == 0:
            orc.pbvi_update(g, G, Gp, pi)
            host = np.ctypeslib.as_array(alg.GammaPrime, shape=(r * n,)).reshape(r, n)
            np.testing.assert_array_equal(bits(host), bits(Gp))
        else:
            orc.pbvi_update(g, Gp, G, pi)
            host = np.ctypeslib.as_array(alg.Gamma, shape=(r * n,)).reshape(r, n)
            np.testing.assert_array_equal(bits(host), bits(G))
        np.testing.assert_array_equal(np.ctypeslib.as_array(alg.pi, shape=(r,)), pi)
        assert alg.currentHorizon == h + 1


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("shape", [(1, 1, 1, 1, 40, 1), (2, 1, 3, 2, 50, 2), (33, 4, 1, 33, 64, 33),
                                   (7, 9, 2, 3, 1, 7), (64, 1, 64, 4, 130, 5), (129, 2, 2, 5, 257, 129),
                                   (50, 2, 1, 7, 300, 50)])
def test_degenerate_shapes_against_oracle(shape, mode):
    """One state, one action, one observation, one belief, full belief
    support (rz = n) and dense successor lists (ns = n), from a random
    initial set whose rows are all distinct (so the tensor-core modes score
    the first updates on the tensor cores whenever r >= 32)."""
    n, m, z, ns, r, rz = shape
    md = synth.random_pomdp(n=n, m=m, z=z, ns=ns, r=r, rz=rz, gamma=0.9, horizon=5, seed=n + r)
    md["GammaInitial"] = np.random.default_rng(n * r).normal(-3.0, 1.0, size=(r, n)).astype(np.float32)
    G, pi = solve_gpu(md, mode)
    Go, po = orc.pbvi_solve(md)
    np.testing.assert_array_equal(bits(G), bits(Go))
    np.testing.assert_array_equal(pi, po)


def kept_belief_model(seed=3):
    """Beliefs 0..39 live on states 0..29, whose rewards are -3e10, so no action
    of theirs beats the -1e10 sentinel and the update leaves their rows and
    actions as they were; states 30..59 lead only to themselves, so beliefs
    40..79 are backed up normally."""
    md = synth.random_pomdp(n=60, m=3, z=4, ns=6, r=80, rz=8, gamma=0.9, horizon=4, seed=seed)
    rng = np.random.default_rng(seed)
    for s in range(30, 60):
        for a in range(3):
            md["S"][s, a] = np.sort(rng.choice(np.arange(30, 60), 6, replace=False))
    md["R"][:30, :] = -3e10
    for i in range(80):
        pool = np.arange(0, 30) if i < 40 else np.arange(30, 60)
        md["Z"][i] = np.sort(rng.choice(pool, 8, replace=False))
    md["GammaInitial"] = rng.normal(size=(80, 60)).astype(np.float32)
    return md


def test_stepwise_update_cpu_api_keeps_rows_below_sentinel():
    """update_cpu uploads the host output set only when some belief keeps its
    row; both kinds of belief match nova's in-place update step by step."""
    md = kept_belief_model()
    p = POMDP.from_arrays(md)
    alg = POMDPPBVICPU(p, GammaInitial=md["GammaInitial"])
    G = md["GammaInitial"].copy()
    Gp = G.copy()
    pi = np.zeros(md["r"], np.uint32)
    r, n = md["r"], md["n"]
    for h in range(4):
        alg.update()
        src, dst = (G, Gp) if h % 2 == 0 else (Gp, G)
        orc.pbvi_update(md, src, dst, pi)
        host = np.ctypeslib.as_array(alg.GammaPrime if h % 2 == 0 else alg.Gamma, shape=(r * n,)).reshape(r, n)
        np.testing.assert_array_equal(bits(host), bits(dst))
        np.testing.assert_array_equal(np.ctypeslib.as_array(alg.pi, shape=(r,)), pi)
    assert np.array_equal(bits(Gp[:40]), bits(md["GammaInitial"][:40]))  # kept rows did survive
    assert not np.array_equal(bits(Gp[40:]), bits(md["GammaInitial"][40:]))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("seed", [7, 8])
def test_random_models_stepwise_against_oracle(seed, mode):
    """Uneven shapes (n, r, z not multiples of any tile) step by step."""
    m = synth.random_pomdp(n=173, m=5, z=11, ns=9, r=301, rz=13, gamma=0.93, horizon=6, seed=seed)
    p = POMDP.from_arrays(m)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=m["GammaInitial"])
    alg.set_scoring(mode)
    G = m["GammaInitial"].copy()
    Gp = G.copy()
    pi = np.zeros(m["r"], np.uint32)
    for h in range(m["horizon"]):
        alg.update()
        if h % 2 == 0:
            orc.pbvi_update(m, G, Gp, pi)
        else:
            orc.pbvi_update(m, Gp, G, pi)
        pol = alg.get_policy()
        ref = Gp if h % 2 == 0 else G
        np.testing.assert_array_equal(bits(pol.gamma_array()), bits(ref))
        np.testing.assert_array_equal(pol.pi_array(), pi)


def test_value_gpu_fp64():
    g = load_golden("pbvi_n64_h100")
    p = POMDP.from_arrays(g)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=g["GammaInitial"])
    for _ in range(g["horizon"]):
        alg.update()
    b0 = synth.dense_belief(g, 0)
    V, a = alg.value(b0)
    G = g["out_Gamma"].astype(np.float64)
    vals = G @ b0.astype(np.float64)
    assert abs(V - vals.max()) <= 1e-12 * max(1.0, abs(vals.max()))
    assert a == g["out_pi"][int(np.argmax(vals))]
    Vf, af = orc.alpha_value(g["out_Gamma"], g["out_pi"], b0)
    assert abs(V - Vf) < 1e-5 * max(1.0, abs(Vf))


def test_numthreads_must_be_multiple_of_32():
    g = load_golden("pbvi_tiger")
    p = POMDP.from_arrays(g)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, numThreads=33, GammaInitial=g["GammaInitial"])
    from nova_gb300 import pomdp_alpha_vectors as pav
    pol = pav.POMDPAlphaVectors()
    assert npp._nova.pomdp_pbvi_execute_gpu(alg.pomdpPtr, alg, pol) == 2  # NOVA_ERROR_INVALID_CUDA_PARAM


def _run_mode(model, mode, steps, table=npp.TABLE_AUTO):
    p = POMDP.from_arrays(model)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=model["GammaInitial"])
    alg.set_scoring(mode)
    alg.set_table(table)
    out, stats = [], []
    for _ in range(steps):
        alg.update()
        stats.append(alg.stats())
        pol = alg.get_policy()
        out.append((pol.gamma_array(), pol.pi_array()))
    return out, stats


@pytest.mark.parametrize("mode", [npp.SCORING_BF16, npp.SCORING_FP16])
def test_tensor_core_scoring_is_exact_and_runs(mode):
    """At a size where the tensor-core path engages (>= 32 distinct alphas),
    tensor-core scoring with the proven margin gives bit-identical alphas and
    actions to exact scoring at every step, and the tensor cores decide most
    rows (few fall back to the exact row scan)."""
    m = synth.random_pomdp(n=300, m=6, z=12, ns=12, r=700, rz=20, gamma=0.95, horizon=7, seed=5)
    exact, _ = _run_mode(m, npp.SCORING_EXACT, m["horizon"])
    tc, stats = _run_mode(m, mode, m["horizon"])
    for (Ge, pe), (Gt, pt) in zip(exact, tc):
        np.testing.assert_array_equal(bits(Gt), bits(Ge))
        np.testing.assert_array_equal(pt, pe)
    engaged = [s for s in stats if s["scoring"] == mode]
    assert len(engaged) >= 3, stats
    rows = m["r"] * m["m"] * m["z"]
    # BF16's proven margin (A rounded to 8 significant bits) is several
    # times wider than FP16's, so it may leave more rows to the exact scan.
    limit = 0.25 if mode == npp.SCORING_BF16 else 0.01
    for s in engaged:
        assert s["msGemm"] > 0
        assert s["rowsOverflow"] <= limit * rows, s


@pytest.mark.parametrize("mode", [npp.SCORING_BF16, npp.SCORING_FP16])
def test_tensor_core_scoring_many_unresolved_rows(mode):
    """n=512, r=1024, many near-tied alphas per row: every step must equal
    exact scoring bit for bit, whatever share of rows the margin leaves to
    the exact scan."""
    m = synth.random_pomdp(n=512, m=8, z=16, ns=16, r=1024, rz=32, gamma=0.95, horizon=5, seed=5)
    exact, _ = _run_mode(m, npp.SCORING_EXACT, m["horizon"])
    tc, stats = _run_mode(m, mode, m["horizon"])
    for (Ge, pe), (Gt, pt) in zip(exact, tc):
        np.testing.assert_array_equal(bits(Gt), bits(Ge))
        np.testing.assert_array_equal(pt, pe)
    assert any(s["scoring"] == mode for s in stats)


@pytest.mark.parametrize("mode", [npp.SCORING_BF16, npp.SCORING_FP16, npp.SCORING_EXACT])
@pytest.mark.parametrize("shape", [dict(n=300, m=6, z=12, ns=12, r=700, rz=20, horizon=6, seed=5),
                                   dict(n=512, m=8, z=16, ns=16, r=1024, rz=32, horizon=4, seed=5),
                                   dict(n=200, m=4, z=8, ns=40, r=512, rz=40, horizon=5, seed=7)])
def test_without_projection_table_same_bits(mode, shape):
    """NOVA_PBVI_TABLE_NEVER: tensor-core updates re-score their candidates,
    score their open rows' (belief, action) pairs and assemble straight from
    the alphas; the exact form scores every pair so. Every step equals the
    table-backed exact form bit for bit, and no projection time is spent
    (ns = 40 takes the re-score's path for more than 32 successors, rz = 40
    its support chunks past 32)."""
    m = synth.random_pomdp(gamma=0.95, **shape)
    ref, _ = _run_mode(m, npp.SCORING_EXACT, m["horizon"])
    out, stats = _run_mode(m, mode, m["horizon"], table=npp.TABLE_NEVER)
    for (Ge, pe), (Gt, pt) in zip(ref, out):
        np.testing.assert_array_equal(bits(Gt), bits(Ge))
        np.testing.assert_array_equal(pt, pe)
    assert stats[-1]["msProject"] < 0.1, stats  # (the first tensor-core step builds its operands there)
    if mode != npp.SCORING_EXACT:
        assert any(s["scoring"] == mode for s in stats), stats


def test_set_table_rejects_bad_arguments():
    m = synth.random_pomdp(n=40, m=3, z=4, ns=5, r=64, rz=8, gamma=0.9, horizon=2, seed=1)
    p = POMDP.from_arrays(m)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=m["GammaInitial"])
    assert npp._nova.pomdp_pbvi_set_table_gpu(alg, 7) != 0
    assert npp._nova.pomdp_pbvi_set_table_gpu(None, npp.TABLE_NEVER) != 0
    alg.set_table(npp.TABLE_NEVER)
    alg.set_table(npp.TABLE_AUTO)
