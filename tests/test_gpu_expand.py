"""Belief-set expansion and sigma approximation on the GB300 (nova's
pomdp_expand_* / pomdp_sigma_cpu entry points) against the reference's
outputs (golden fixtures) and the oracle."""
import ctypes as ct

import numpy as np
import pytest

from conftest import load_golden, bits
from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300 import nova_pomdp as npm
from nova_gb300 import nova_pomdp_alpha_vectors as npav
from nova_gb300.pomdp import POMDP

pytestmark = pytest.mark.gpu

KEYS = ("n", "ns", "m", "z", "r", "rz", "gamma", "horizon", "S", "T", "O", "R", "Z", "B")


@pytest.fixture
def seeded():
    def set_seed(seed):
        assert npm._nova.nova_gb300_expand_seed(1, seed) == 0
    yield set_seed
    npm._nova.nova_gb300_expand_seed(0, 0)


def model_of(g):
    return {k: g[k] for k in KEYS}


def policy_struct(G, pi, n, m):
    G = np.ascontiguousarray(G, np.float32)
    pi = np.ascontiguousarray(pi, np.uint32)
    pol = npav.NovaPOMDPAlphaVectors()
    pol.n, pol.m, pol.r = n, m, G.shape[0]
    pol.Gamma = G.ctypes.data_as(ct.POINTER(ct.c_float))
    pol.pi = pi.ctypes.data_as(ct.POINTER(ct.c_uint))
    return pol, (G, pi)


@pytest.mark.parametrize("name", ["expand_distinct", "expand_distinct_ragged"])
def test_distinct_matches_reference(name):
    g = load_golden(name)
    p = POMDP.from_arrays(model_of(g))
    p.expand(method="distinct_beliefs")
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], g["out_Z"])
    np.testing.assert_array_equal(bits(out["B"]), bits(g["out_B"]))


def test_random_matches_reference(seeded):
    g = load_golden("expand_random")
    seeded(int(g["out_srand"]))
    p = POMDP.from_arrays(model_of(g))
    p.expand(method="random", numBeliefsToAdd=int(g["out_num"]))
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], g["out_Z"])
    np.testing.assert_array_equal(bits(out["B"]), bits(g["out_B"]))


def test_random_from_b0_matches_reference(seeded):
    g = load_golden("expand_random_b0")
    seeded(int(g["out_srand"]))
    p = POMDP.from_arrays(model_of(g))
    nz = ct.c_uint(0)
    Bn = ct.POINTER(ct.c_float)()
    num = int(g["out_num"])
    assert npm._nova.pomdp_expand_random_gpu(p, 32, num, ct.byref(nz), ct.byref(Bn)) == 0
    out = np.ctypeslib.as_array(Bn, shape=(num * p.n,)).reshape(num, p.n).copy()
    np.testing.assert_array_equal(bits(out), bits(g["out_Bnew"]))
    assert nz.value == int(g["out_maxNonZero"])


def test_pema_matches_reference():
    g = load_golden("expand_pema")
    p = POMDP.from_arrays(model_of(g))
    pol, keep = policy_struct(g["out_policyGamma"], g["out_policyPi"], p.n, p.m)
    assert npm._nova.pomdp_expand_pema_cpu(p, ct.byref(pol)) == 0
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], g["out_Z"])
    np.testing.assert_array_equal(bits(out["B"]), bits(g["out_B"]))


def test_sigma_matches_reference():
    g = load_golden("sigma_k3")
    p = POMDP.from_arrays(model_of(g))
    sigma = p.sigma_approximate(int(g["out_k"]))
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], g["out_Z"])
    np.testing.assert_array_equal(bits(out["B"]), bits(g["out_B"]))
    assert np.float32(sigma) == g["out_sigma"]


def larger_model(seed):
    return synth.random_pomdp(n=128, m=4, z=8, ns=8, r=200, rz=16, gamma=0.95, horizon=12, seed=seed)


def test_larger_models_match_oracle(seeded):
    m = larger_model(5)
    # distinct
    p = POMDP.from_arrays(m)
    p.expand(method="distinct_beliefs")
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_distinct(m))
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], Z)
    np.testing.assert_array_equal(bits(out["B"]), bits(B))
    # random, seeded
    seeded(1234)
    p = POMDP.from_arrays(m)
    p.expand(method="random", numBeliefsToAdd=300)
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_random(m, 300, 1234))
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], Z)
    np.testing.assert_array_equal(bits(out["B"]), bits(B))
    # PEMA with a policy from a few backups
    G, pi = orc.pbvi_solve(m, horizon=3)
    p = POMDP.from_arrays(m)
    pol, keep = policy_struct(G, pi, m["n"], m["m"])
    assert npm._nova.pomdp_expand_pema_cpu(p, ct.byref(pol)) == 0
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_pema(m, G)[None, :])
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], Z)
    np.testing.assert_array_equal(bits(out["B"]), bits(B))
    # sigma
    p = POMDP.from_arrays(m)
    sigma = p.sigma_approximate(5)
    Z, B, s = orc.sigma_approximate(m, 5)
    out = p.arrays()
    np.testing.assert_array_equal(out["Z"], Z)
    np.testing.assert_array_equal(bits(out["B"]), bits(B))
    assert np.float32(sigma) == np.float32(s)


def test_distinct_with_empty_belief_adds_a_zero_row():
    m = synth.random_pomdp(n=16, m=2, z=3, ns=4, r=10, rz=4, gamma=0.9, horizon=4, seed=2)
    m["Z"][3] = -1
    m["B"][3] = 0.0
    p = POMDP.from_arrays(m)
    p.expand(method="distinct_beliefs")
    out = p.arrays()
    assert (out["Z"][m["r"] + 3] == -1).all()
    Z, B = orc.merge_raw_beliefs(m["Z"], m["B"], orc.expand_distinct(m))
    np.testing.assert_array_equal(out["Z"], Z)
    np.testing.assert_array_equal(bits(out["B"]), bits(B))
