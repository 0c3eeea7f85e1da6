import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (run with -m gpu)")


def _ensure_library():
    from nova_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()


_ensure_library()


def load_golden(name):
    """A golden fixture as a dict (model arrays, scalars, and out_* outputs)."""
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        d = {k: f[k] for k in f.files}
    for k in ("n", "ns", "m", "z", "r", "rz", "horizon", "seed", "out_srand"):
        if k in d:
            d[k] = int(d[k])
    d["gamma"] = float(d["gamma"])
    return d


PBVI_GOLDENS = ["pbvi_n64_h5", "pbvi_n64_h100", "pbvi_tiger", "pbvi_ragged", "pbvi_two_state_h3",
                "pbvi_two_state_h10"]
PERSEUS_GOLDENS = ["perseus_tiger", "perseus_small"]
MDP_GOLDENS = ["mdp_vi_ragged", "mdp_vi_vinit"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
