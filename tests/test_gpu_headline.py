"""PBVI parity at the benchmarked size: the pbvi_n4096 workload (n=4096,
m=16, z=32, ns=32, r=8192, rz=64, gamma=0.95, seed 0). After three
tensor-core updates, one more update in each tensor-core scoring mode is
compared bit for bit, for 16 sampled beliefs, with nova's loop-form backup
(the oracle's restatement of pomdp_pbvi_cpu.cpp:106-162) over all m actions
against the full alpha set. The sample holds the beliefs with rows sent to
the exact scan, those with the most alphas re-scored exactly in the merge, and
random ones (pomdp_pbvi_row_detail_gpu says which)."""
import numpy as np
import pytest

from oracle import oracle as orc
from nova_gb300 import synth
from nova_gb300 import nova_pomdp_pbvi as npp
from nova_gb300.pomdp import POMDP
from nova_gb300.pomdp_pbvi import POMDPPBVIGPU

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline():
    cfg = dict(synth.POMDP_CONFIGS["pbvi_n4096"])
    model = synth.random_pomdp(**cfg, seed=0)
    p = POMDP.from_arrays(model)
    p.initialize_gpu()
    return model, p


@pytest.mark.parametrize("mode", [npp.SCORING_FP16, npp.SCORING_BF16])
def test_headline_sampled_beliefs_match_oracle(headline, mode):
    model, p = headline
    alg = POMDPPBVIGPU(p, GammaInitial=model["GammaInitial"])
    alg.set_scoring(mode)
    for _ in range(3):
        alg.update()
    before = alg.get_policy()
    G = before.gamma_array()
    del before
    alg.update()
    st = alg.stats()
    assert st["scoring"] == mode and st["msGemm"] > 0, st
    cand, exact = alg.row_detail()
    assert int(cand.sum()) == st["candidates"]
    assert int(exact.sum()) == st["rowsOverflow"]
    after = alg.get_policy()
    Gp, pi = after.gamma_array(), after.pi_array()
    del after
    del alg
    beliefs = orc.choose_parity_beliefs(cand, exact, k=16, seed=mode)
    assert len(beliefs) == 16
    assert cand[beliefs[0]] > 0 or exact[beliefs[0]] > 0
    bad = orc.sampled_backup_parity(model, G, Gp, pi, beliefs)
    assert bad == [], "beliefs %s differ from the oracle (mode %d)" % (bad, mode)
