"""Batched V(b) and action (pomdp_alpha_vectors_value_and_action_batched,
pomdp_alpha_vectors_value_batched_gpu) against nova's one-belief evaluation
(the oracle), bit for bit."""
import ctypes as ct

import numpy as np
import pytest

from conftest import bits
from oracle import oracle as orc
from nova_gb300 import nova_pomdp_alpha_vectors as npav
from nova_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def policy(G, pi):
    from nova_gb300.pomdp_alpha_vectors import POMDPAlphaVectors
    p = POMDPAlphaVectors()
    G = np.ascontiguousarray(G, np.float32)
    pi = np.ascontiguousarray(pi, np.uint32)
    assert npav._nova.pomdp_alpha_vectors_initialize(p, G.shape[1], int(pi.max()) + 1, G.shape[0]) == 0
    ct.memmove(p.Gamma, G.ctypes.data, G.nbytes)
    ct.memmove(p.pi, pi.ctypes.data, pi.nbytes)
    return p


def reference(G, pi, B):
    out = [orc.alpha_value(G, pi, b) for b in B]
    return np.array([v for v, _ in out], np.float32), np.array([a for _, a in out], np.uint32)


@pytest.mark.parametrize("r,n,count", [(300, 200, 500), (64, 33, 7), (1, 1, 1), (129, 517, 65)])
def test_batched_values_equal_reference(r, n, count):
    rng = np.random.default_rng(r + n)
    G = rng.uniform(-5, 5, size=(r, n)).astype(np.float32)
    pi = rng.integers(0, 7, size=r).astype(np.uint32)
    if r > 3:
        G[r // 2] = G[1]          # an exact tie: the lower index (1) must win
        pi[r // 2] = 6
    B = rng.dirichlet(np.ones(n), size=count).astype(np.float32)
    B[:, ::3] = 0.0               # zero states are added like the reference adds them
    p = policy(G, pi)
    V, a = p.value_and_action_batched(B)
    Vr, ar = reference(G, pi, B)
    np.testing.assert_array_equal(bits(V), bits(Vr))
    np.testing.assert_array_equal(a, ar)


def test_sentinel_and_device_entry_point():
    n, r, count = 40, 10, 5
    G = np.full((r, n), -3e10, np.float32)   # every value below -1e10: V = -1e10, action 0
    pi = np.arange(r, dtype=np.uint32) + 1
    B = np.full((count, n), 1.0 / n, np.float32)
    dG, dPi, dB = (torch.as_tensor(x, device="cuda") for x in (G, pi.astype(np.int32), B))
    dV = torch.empty(count, dtype=torch.float32, device="cuda")
    dA = torch.empty(count, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert npav._nova.pomdp_alpha_vectors_value_batched_gpu(dG.data_ptr(), dPi.data_ptr(), r, n, dB.data_ptr(),
                                                            count, dV.data_ptr(), dA.data_ptr()) == 0
    Vr, ar = reference(G, pi, B)
    np.testing.assert_array_equal(bits(dV.cpu().numpy()), bits(Vr))
    np.testing.assert_array_equal(dA.cpu().numpy().astype(np.uint32), ar)


def test_policy_of_a_solve():
    model = synth.random_pomdp(n=64, m=4, z=8, ns=8, r=256, rz=8, gamma=0.95, horizon=10, seed=3)
    G, pi = orc.pbvi_solve(model)
    B = np.stack([synth.dense_belief(model, i) for i in range(model["r"])])
    V, a = policy(G, pi).value_and_action_batched(B)
    Vr, ar = reference(G, pi, B)
    np.testing.assert_array_equal(bits(V), bits(Vr))
    np.testing.assert_array_equal(a, ar)
