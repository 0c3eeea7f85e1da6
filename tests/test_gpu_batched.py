"""Batched PBVI solves (pomdp_pbvi_execute_batched_gpu) against nova's
per-POMDP results (the oracle), for every scoring mode."""
import numpy as np
import pytest

from conftest import bits
from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300 import nova_pomdp_pbvi as npp
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_pbvi import solve_batched

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [npp.SCORING_EXACT, npp.SCORING_BF16, npp.SCORING_FP16])
def test_batched_solves_equal_reference(mode):
    models = synth.batch_pomdps(count=12, seed=7, n_range=(8, 96), r_range=(16, 160), m_range=(2, 5),
                                z_range=(2, 6), horizon=6)
    pomdps = []
    for md in models:
        p = POMDP.from_arrays(md)
        p.initialize_gpu()
        pomdps.append(p)
    policies = solve_batched(pomdps, scoring=mode, hostThreads=4)
    for md, pol in zip(models, policies):
        G, pi = orc.pbvi_solve(md)
        np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
        np.testing.assert_array_equal(pol.pi_array(), pi)


def test_batched_rejects_repeated_solver():
    md = synth.random_pomdp(n=8, m=2, z=2, ns=3, r=8, rz=3, horizon=2, seed=1)
    p = POMDP.from_arrays(md)
    p.initialize_gpu()
    import ctypes as ct
    s = npp.NovaPOMDPPBVIGPU()
    P = (ct.POINTER(POMDP) * 2)(ct.pointer(p), ct.pointer(p))
    G = (ct.POINTER(npp.NovaPOMDPPBVIGPU) * 2)(ct.pointer(s), ct.pointer(s))
    from nova_gb300 import pomdp_alpha_vectors as pav
    a1, a2 = pav.POMDPAlphaVectors(), pav.POMDPAlphaVectors()
    A = (ct.POINTER(npp._npav.NovaPOMDPAlphaVectors) * 2)(
        ct.cast(ct.pointer(a1), ct.POINTER(npp._npav.NovaPOMDPAlphaVectors)),
        ct.cast(ct.pointer(a2), ct.POINTER(npp._npav.NovaPOMDPAlphaVectors)))
    assert npp._nova.pomdp_pbvi_execute_batched_gpu(P, G, A, 2, npp.SCORING_FP16, 2) != 0


def test_batched_graph_solves_equal_reference():
    """Graph mode (horizon loops replayed as CUDA graphs once the tensor-core
    schedule is tuned) gives nova's results."""
    models = synth.batch_pomdps(count=8, seed=11, n_range=(16, 96), r_range=(64, 200), m_range=(2, 4),
                                z_range=(2, 5), horizon=12)
    pomdps = []
    for md in models:
        p = POMDP.from_arrays(md)
        p.initialize_gpu()
        pomdps.append(p)
    policies = solve_batched(pomdps, scoring=npp.SCORING_FP16, hostThreads=4, graph=True)
    for md, pol in zip(models, policies):
        G, pi = orc.pbvi_solve(md)
        np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
        np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("n", [150, 2100])
def test_graph_updates_equal_reference(n):
    """Single solver in graph mode: updates after the schedule is fixed are
    graph replays (no per-update timings, kernels counted), with nova's
    results; n = 2100 uses the state-contiguous projection table."""
    from nova_gb300.pomdp_pbvi import POMDPPBVIGPU
    md = synth.random_pomdp(n=n, m=2, z=4, ns=8, r=256, rz=16, gamma=0.95, horizon=9, seed=21)
    p = POMDP.from_arrays(md)
    p.initialize_gpu()
    s = POMDPPBVIGPU(p)
    s.set_scoring(npp.SCORING_FP16)
    s.set_graph(True)
    replays = 0
    for _ in range(md["horizon"]):
        s.update()
        st = s.stats()
        if st["msTotal"] == 0.0 and st["launches"] > 0:
            replays += 1
    assert replays >= 2
    pol = s.get_policy()
    G, pi = orc.pbvi_solve(md)
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
    np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("n", [1100, 2100])
@pytest.mark.parametrize("mode", [npp.SCORING_FP16, npp.SCORING_BF16])
def test_large_state_layouts_equal_reference(mode, n):
    """n > 1024: FP16 updates use the state-contiguous projection table (while
    the exact scan stays small), BF16 the alpha-contiguous one; both give
    nova's results."""
    from nova_gb300.pomdp_pbvi import POMDPPBVIGPU
    md = synth.random_pomdp(n=n, m=3, z=5, ns=8, r=300, rz=16, gamma=0.95, horizon=6, seed=23)
    p = POMDP.from_arrays(md)
    p.initialize_gpu()
    s = POMDPPBVIGPU(p)
    s.set_scoring(mode)
    for _ in range(md["horizon"]):
        s.update()
    pol = s.get_policy()
    G, pi = orc.pbvi_solve(md)
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
    np.testing.assert_array_equal(pol.pi_array(), pi)


def test_graph_mode_survives_scoring_change():
    """Changing the scoring mode drops the captured updates; the next ones
    are captured (or run) in the new mode, with nova's results."""
    from nova_gb300.pomdp_pbvi import POMDPPBVIGPU
    md = synth.random_pomdp(n=150, m=2, z=4, ns=8, r=256, rz=16, gamma=0.95, horizon=12, seed=29)
    p = POMDP.from_arrays(md)
    p.initialize_gpu()
    s = POMDPPBVIGPU(p)
    s.set_scoring(npp.SCORING_FP16)
    s.set_graph(True)
    for _ in range(8):
        s.update()
    s.set_scoring(npp.SCORING_BF16)
    for _ in range(md["horizon"] - 8):
        s.update()
    pol = s.get_policy()
    G, pi = orc.pbvi_solve(md)
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
    np.testing.assert_array_equal(pol.pi_array(), pi)


@pytest.mark.parametrize("mode", [npp.SCORING_FP16, npp.SCORING_BF16, npp.SCORING_EXACT])
def test_persistent_batched_solves_equal_reference(mode):
    """Lock-step batched solve (pomdp_pbvi_execute_batched_persistent_gpu): after
    the warm-up that tunes each solver, every backup of the batch scores its
    tensor-core solvers in one persistent launch from a device work table;
    uneven n, r, m and z, one deep model (n = 2100: fixed schedule, the
    state-contiguous table) and horizons long enough for many lock-step
    backups. Every policy equals nova's."""
    models = synth.batch_pomdps(count=9, seed=23, n_range=(16, 180), r_range=(40, 260), m_range=(2, 5),
                                z_range=(2, 7), horizon=14)
    deep = synth.random_pomdp(n=2100, m=2, z=3, ns=5, r=72, rz=6, gamma=0.95, horizon=9, seed=29)
    deep["GammaInitial"] = np.random.default_rng(3).normal(-3.0, 1.0, size=(72, 2100)).astype(np.float32)
    models.append(deep)
    pomdps = []
    for md in models:
        p = POMDP.from_arrays(md)
        p.initialize_gpu()
        pomdps.append(p)
    inits = [md["GammaInitial"] for md in models]
    policies = solve_batched(pomdps, scoring=mode, hostThreads=4, GammaInitials=inits, persistent=True)
    for md, pol in zip(models, policies):
        G, pi = orc.pbvi_solve(md)
        np.testing.assert_array_equal(bits(pol.gamma_array()), bits(G))
        np.testing.assert_array_equal(pol.pi_array(), pi)
