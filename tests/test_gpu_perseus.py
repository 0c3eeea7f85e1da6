"""Perseus on the GB300 (host-buffer and device-buffer entry points) against
the reference's outputs with the same srand() seed."""
import numpy as np
import pytest

from conftest import load_golden, bits, PERSEUS_GOLDENS
from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_perseus import POMDPPerseusCPU, POMDPPerseusGPU

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", PERSEUS_GOLDENS)
@pytest.mark.parametrize("api", ["cpu", "gpu"])
def test_perseus_matches_reference(name, api):
    g = load_golden(name)
    p = POMDP.from_arrays(g)
    if api == "gpu":
        p.initialize_gpu()
        alg = POMDPPerseusGPU(p, GammaInitial=g["GammaInitial"])
    else:
        alg = POMDPPerseusCPU(p, GammaInitial=g["GammaInitial"])
    orc.lib().oracle_srand(g["out_srand"])  # libc rand() is shared by the process
    pol = alg.solve()
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(g["out_Gamma"]))
    np.testing.assert_array_equal(pol.pi_array(), g["out_pi"])


@pytest.mark.parametrize("seed", [3, 4])
def test_perseus_random_models_against_oracle(seed):
    m = synth.random_pomdp(n=61, m=4, z=7, ns=6, r=150, rz=9, gamma=0.92, horizon=6, seed=seed)
    Go, po = orc.perseus_solve(m, seed=seed)
    p = POMDP.from_arrays(m)
    p.initialize_gpu()
    alg = POMDPPerseusGPU(p, GammaInitial=m["GammaInitial"])
    orc.lib().oracle_srand(seed)
    pol = alg.solve()
    np.testing.assert_array_equal(bits(pol.gamma_array()), bits(Go))
    np.testing.assert_array_equal(pol.pi_array(), po)
