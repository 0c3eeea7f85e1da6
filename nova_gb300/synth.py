"""Seeded synthetic POMDP / MDP generators for the benchmark workloads.

Every model uses nova's array layouts (S,T [n][m][ns]; O [m][n][z]; R [n][m];
Z,B [r][rz]) and the workload definitions of the benchmark configurations:

* successors: ns distinct states per (s, a), uniform without replacement,
  stored in increasing order; T over them ~ Dirichlet(1);
* O(a, s', .) ~ Dirichlet(1) over the z observations;
* R ~ Uniform[-1, 1];
* beliefs: rz distinct support states (uniform), weights ~ Dirichlet(1);
* initial alpha set: every entry min(R) / (1 - gamma) (nova's default,
  pomdp_pbvi.py:59-65).

Dirichlet(1) is drawn as normalised Exp(1) variates. Generation is numpy
(PCG64) and deterministic for a given seed on a given platform.
"""
import numpy as np

# Named workloads (sizes of the benchmark configurations).
POMDP_CONFIGS = {
    "pbvi_n64": dict(n=64, m=4, z=8, ns=8, r=256, rz=8, gamma=0.95, horizon=100),
    "pbvi_n4096": dict(n=4096, m=16, z=32, ns=32, r=8192, rz=64, gamma=0.95, horizon=200),
    "pbvi_n512": dict(n=512, m=8, z=16, ns=16, r=1024, rz=32, gamma=0.95, horizon=50),
    "pbvi_n4096_small": dict(n=4096, m=2, z=4, ns=32, r=4096, rz=64, gamma=0.95, horizon=10),
    "pbvi_n4096_r256": dict(n=4096, m=16, z=32, ns=32, r=256, rz=64, gamma=0.95, horizon=4),
    "expand_n512": dict(n=512, m=8, z=16, ns=16, r=1024, rz=32, gamma=0.95, horizon=50),
    "pbvi_n4096_prof": dict(n=4096, m=2, z=32, ns=32, r=2048, rz=64, gamma=0.95, horizon=10),
    "pbvi_n4096_m4z8": dict(n=4096, m=4, z=8, ns=32, r=8192, rz=64, gamma=0.95, horizon=10),
    "grad_n1024": dict(n=1024, m=8, z=16, ns=16, r=2048, rz=32, gamma=0.95, horizon=50),
    "pbvi_n59_r3725": dict(n=59, m=7, z=29, ns=16, r=3725, rz=32, gamma=0.95, horizon=10),
}
MDP_CONFIGS = {
    "vi_n1m": dict(n=1 << 20, m=8, ns=16, gamma=0.99, horizon=2000),
}


def _distinct_rows(rng, rows, n, k):
    """rows x k distinct integers in [0, n) per row, each row sorted."""
    if k > n:
        raise ValueError("cannot draw %d distinct states out of %d" % (k, n))
    if rows * n <= 1 << 25 or 2 * k > n:
        keys = rng.random((rows, n), dtype=np.float32)
        out = np.argpartition(keys, k - 1, axis=1)[:, :k]
        return np.sort(out, axis=1).astype(np.int32)
    out = rng.integers(0, n, size=(rows, k), dtype=np.int64)
    while True:
        srt = np.sort(out, axis=1)
        dup = (np.diff(srt, axis=1) == 0).any(axis=1)
        if not dup.any():
            return srt.astype(np.int32)
        out[dup] = rng.integers(0, n, size=(int(dup.sum()), k), dtype=np.int64)


def _dirichlet1(rng, shape):
    w = rng.standard_exponential(size=shape, dtype=np.float64)
    w /= w.sum(axis=-1, keepdims=True)
    return w.astype(np.float32)


def random_pomdp(n, m, z, ns, r, rz, gamma=0.95, horizon=100, seed=0):
    """Seeded random sparse POMDP as a dict of numpy arrays and scalars."""
    rng = np.random.Generator(np.random.PCG64(seed))
    S = _distinct_rows(rng, n * m, n, ns).reshape(n, m, ns)
    T = _dirichlet1(rng, (n, m, ns))
    O = _dirichlet1(rng, (m, n, z))
    R = rng.uniform(-1.0, 1.0, size=(n, m)).astype(np.float32)
    Z = _distinct_rows(rng, r, n, rz)
    B = _dirichlet1(rng, (r, rz))
    gamma = np.float32(gamma)
    g0 = np.float32(np.float32(R.min()) / (np.float32(1.0) - gamma))
    return dict(n=n, ns=ns, m=m, z=z, r=r, rz=rz, gamma=float(gamma), horizon=horizon, S=S, T=T, O=O, R=R,
                Z=Z, B=B, GammaInitial=np.full((r, n), g0, dtype=np.float32), seed=seed)


def random_mdp(n, m, ns, gamma=0.99, horizon=100, seed=0):
    """Seeded random sparse MDP as a dict of numpy arrays and scalars."""
    rng = np.random.Generator(np.random.PCG64(seed))
    S = _distinct_rows(rng, n * m, n, ns).reshape(n, m, ns)
    T = _dirichlet1(rng, (n, m, ns))
    R = rng.uniform(-1.0, 1.0, size=(n, m)).astype(np.float32)
    return dict(n=n, ns=ns, m=m, gamma=float(np.float32(gamma)), horizon=horizon, S=S, T=T, R=R, seed=seed)


def dense_belief(model, i):
    """Row i of (Z, B) as a dense n-vector (b0 of the benchmarks is row 0)."""
    b = np.zeros(model["n"], dtype=np.float32)
    for s, p in zip(model["Z"][i], model["B"][i]):
        if s < 0:
            break
        b[s] = p
    return b


def batch_shapes(count=256, seed=0, n_range=(32, 2048), r_range=(128, 4096), m_range=(2, 16), z_range=(2, 32),
                 horizon=100):
    """Shapes of a batch of independent POMDPs: n and r log-uniform, m and z
    uniform integers, ns = min(16, n), rz = min(32, n), gamma = 0.95."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        r = int(round(np.exp(rng.uniform(np.log(r_range[0]), np.log(r_range[1])))))
        m = int(rng.integers(m_range[0], m_range[1] + 1))
        z = int(rng.integers(z_range[0], z_range[1] + 1))
        out.append(dict(n=n, m=m, z=z, ns=min(16, n), r=r, rz=min(32, n), gamma=0.95, horizon=horizon,
                        seed=seed * 100003 + k + 1))
    return out


def batch_pomdps(count=256, seed=0, **kw):
    """The seeded batch of random POMDPs of batch_shapes (config of the
    batched-solve benchmark: 256 POMDPs, horizon 100)."""
    return [random_pomdp(**s) for s in batch_shapes(count, seed, **kw)]
