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
