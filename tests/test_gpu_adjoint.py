"""Reverse mode of recorded PBVI backups on the GB300 (pomdp_pbvi_adjoint_gpu)
against the oracle's FP64 reverse mode and FP64 central finite differences."""
import numpy as np
import pytest

from oracle import oracle as orc
from nova_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def small_model(seed=5, **kw):
    cfg = dict(n=48, m=3, z=4, ns=6, r=64, rz=8, gamma=0.95, horizon=12)
    cfg.update(kw)
    return synth.random_pomdp(**cfg, seed=seed)


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))


def fd_check(model, acts, sels, b0, grads, coords, istar, h=1e-6):
    """Central differences of the oracle's FP64 forward (selections and final
    argmax fixed) at `coords` [(name, index)]; returns the worst relative
    error against grads."""
    worst = 0.0
    for name, idx in coords:
        A = model[name].astype(np.float64).copy()
        A[idx] += h
        Vp, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar, **{name: A})
        A[idx] -= 2 * h
        Vm, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar, **{name: A})
        fd = (Vp - Vm) / (2 * h)
        g = grads[name][idx]
        worst = max(worst, abs(g - fd) / max(abs(fd), 1e-3))
    return worst


def random_coords(model, count, rng):
    out = []
    for k in range(count):
        name = ("R", "T", "O")[k % 3]
        out.append((name, tuple(int(rng.integers(0, d)) for d in model[name].shape)))
    return out


def test_recorded_selections_equal_reference_backups():
    from nova_gb300.pomdp_adjoint import pbvi_record_and_adjoint
    model = small_model()
    b0 = synth.dense_belief(model, 0)
    V, istar, dR, dT, dO, dG, acts, sels = pbvi_record_and_adjoint(model, b0, 12, 5)
    G_H, acts_o, sels_o = orc.pbvi_record(model, 12)
    np.testing.assert_array_equal(acts, acts_o)
    np.testing.assert_array_equal(sels, sels_o)
    # V of the GPU's FP32 alphas, reduced in FP64, equals the same reduction of nova's alphas
    vals = G_H.astype(np.float64) @ b0.astype(np.float64)
    assert istar == int(np.argmax(vals))
    assert abs(V - vals[istar]) <= 1e-12 * max(1.0, abs(V))


@pytest.mark.parametrize("k", [1, 3, 12, 20])
def test_adjoint_matches_oracle_reverse(k):
    from nova_gb300.pomdp_adjoint import pbvi_record_and_adjoint
    model = small_model(seed=k)
    b0 = np.full(model["n"], 1.0 / model["n"], np.float32)
    V, istar, dR, dT, dO, dG, acts, sels = pbvi_record_and_adjoint(model, b0, 12, k)
    V64, dR64, dT64, dO64, dG64 = orc.pbvi_fixed_reverse_f64(model, model["GammaInitial"], acts, sels, b0,
                                                              istar=istar)
    # FP32 alphas vs FP64 with the same selections
    assert abs(V - V64) <= 1e-4
    for a, b in ((dR, dR64), (dT, dT64), (dO, dO64), (dG, dG64)):
        assert rel_err(a, b) < 1e-5


def test_adjoint_matches_finite_differences():
    from nova_gb300.pomdp_adjoint import pbvi_record_and_adjoint
    model = small_model(seed=11)
    b0 = synth.dense_belief(model, 0)
    V, istar, dR, dT, dO, dG, acts, sels = pbvi_record_and_adjoint(model, b0, 12, 4)
    coords = random_coords(model, 64, np.random.default_rng(3))
    assert fd_check(model, acts, sels, b0, {"R": dR, "T": dT, "O": dO}, coords, istar) < 1e-3


def test_autograd_function():
    from nova_gb300.pomdp_adjoint import PBVIGradSpec, pbvi_value, pbvi_record_and_adjoint
    model = small_model(seed=2)
    b0 = np.full(model["n"], 1.0 / model["n"], np.float32)
    spec = PBVIGradSpec(model=model, b0=b0, horizon=12, checkpoint_every=5)
    R = torch.tensor(model["R"], requires_grad=True)
    T = torch.tensor(model["T"], requires_grad=True)
    O = torch.tensor(model["O"], requires_grad=True)
    V = pbvi_value(R, T, O, spec)
    (2.0 * V).backward()
    V2, _, dR, dT, dO, _, _, _ = pbvi_record_and_adjoint(model, b0, 12, 5)
    assert float(V.detach()) == V2
    np.testing.assert_allclose(R.grad.numpy(), (2.0 * dR).astype(np.float32), rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(T.grad.numpy(), (2.0 * dT).astype(np.float32), rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(O.grad.numpy(), (2.0 * dO).astype(np.float32), rtol=1e-6, atol=1e-12)


def test_adjoint_full_size_gradient_workload():
    """n=1024, m=8, z=16, ns=16, r=2048, rz=32, H=50, b0 uniform, checkpoints
    every 10 steps: the GPU gradient against the oracle's FP64 reverse mode
    and against central differences on 6 coordinates."""
    from nova_gb300.pomdp_adjoint import pbvi_record_and_adjoint
    cfg = dict(synth.POMDP_CONFIGS["grad_n1024"])
    model = synth.random_pomdp(**cfg, seed=0)
    b0 = np.full(model["n"], 1.0 / model["n"], np.float32)
    V, istar, dR, dT, dO, dG, acts, sels = pbvi_record_and_adjoint(model, b0, cfg["horizon"], 10)
    V64, dR64, dT64, dO64, _ = orc.pbvi_fixed_reverse_f64(model, model["GammaInitial"], acts, sels, b0,
                                                           istar=istar)
    assert abs(V - V64) <= 1e-4
    for a, b in ((dR, dR64), (dT, dT64), (dO, dO64)):
        assert rel_err(a, b) < 1e-5
    coords = random_coords(model, 6, np.random.default_rng(1))
    assert fd_check(model, acts, sels, b0, {"R": dR, "T": dT, "O": dO}, coords, istar) < 1e-3


@pytest.mark.parametrize("kw", [dict(), dict(n=70, m=4, z=5, ns=9, r=90, rz=11, horizon=15)])
def test_fp64_replay_value_matches_oracle(kw):
    """pomdp_pbvi_value_replay_f64_gpu against the oracle's FP64 forward of the
    same recorded selections (pomdp_pbvi_cpu.cpp:37-162 with its argmax
    results fixed), at the FP32 run's maximising row."""
    from nova_gb300.pomdp_adjoint import pbvi_value_vs_fp64
    model = small_model(seed=9, **kw)
    b0 = synth.dense_belief(model, 0)
    H = model["horizon"]
    V, V64, istar, acts, sels = pbvi_value_vs_fp64(model, b0, H)
    Vo, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar)
    assert abs(V64 - Vo) <= 1e-12 * max(1.0, abs(Vo))
    assert abs(V - V64) <= 1e-4
