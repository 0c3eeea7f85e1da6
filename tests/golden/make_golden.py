"""Generate the golden fixtures in tests/golden/ by running the REFERENCE.

Each fixture holds a model (inputs) and the outputs of nova's own CPU code
(its sources compiled by `make -C oracle ref` into oracle/_ref), called
through nova's C API: pomdp_pbvi_execute_cpu, pomdp_perseus_execute_cpu,
mdp_vi_execute_cpu. The tiger model is read with the reference's own raw
file loader (python/nova/file_loader.py). Run here, where the reference is
present:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from nova_gb300 import synth  # noqa: E402

REF_DIR = orc.REF_DIR


def save(name, model, **outputs):
    data = {k: v for k, v in model.items() if isinstance(v, np.ndarray)}
    for k in ("n", "ns", "m", "z", "r", "rz", "horizon", "seed"):
        if k in model:
            data[k] = np.int64(model[k])
    data["gamma"] = np.float32(model["gamma"])
    for k, v in outputs.items():
        data["out_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
    print("wrote", name, {k: getattr(v, "shape", v) for k, v in outputs.items()})


def ragged(model, seed):
    """Truncate successor rows and belief rows at random lengths with -1,
    leaving non-negative garbage after some terminators (nova stops at the
    first negative entry), and give one belief an empty support."""
    rng = np.random.Generator(np.random.PCG64(seed))
    S, T, Z, B = model["S"].copy(), model["T"].copy(), model["Z"].copy(), model["B"].copy()
    n, m, ns = S.shape
    for s in range(n):
        for a in range(m):
            L = int(rng.integers(1, ns + 1))
            if L < ns:
                S[s, a, L] = -1
                T[s, a, L] = 0.0
                if L + 1 < ns and rng.random() < 0.5:
                    S[s, a, L + 1] = int(rng.integers(0, n))  # garbage after the terminator
                    T[s, a, L + 1] = 0.25
                else:
                    S[s, a, L + 1:] = -1
                    T[s, a, L + 1:] = 0.0
    r, rz = Z.shape
    for i in range(r):
        L = int(rng.integers(1, rz + 1))
        if L < rz:
            Z[i, L:] = -1
            B[i, L:] = 0.0
    Z[r // 2, :] = -1
    B[r // 2, :] = 0.0
    out = dict(model)
    out.update(S=S, T=T, Z=Z, B=B)
    return out


def tiger():
    sys.path.insert(0, os.path.join(REF_DIR, "python", "nova"))
    import file_loader  # the reference's loader
    fl = file_loader.FileLoader()
    fl.load_raw_pomdp(os.path.join(REF_DIR, "tests", "tiger", "tiger_pomdp.raw"))
    gamma = np.float32(fl.gamma)
    model = dict(n=fl.n, ns=fl.ns, m=fl.m, z=fl.z, r=fl.r, rz=fl.rz, gamma=float(gamma), horizon=fl.horizon,
                 S=np.asarray(fl.S, np.int32), T=np.asarray(fl.T, np.float32), O=np.asarray(fl.O, np.float32),
                 R=np.asarray(fl.R, np.float32), Z=np.asarray(fl.Z, np.int32), B=np.asarray(fl.B, np.float32),
                 seed=0)
    g0 = np.float32(np.float32(fl.Rmin) / (np.float32(1.0) - gamma))
    model["GammaInitial"] = np.full((fl.r, fl.n), g0, np.float32)
    return model


def two_state():
    """create_two_state_pomdp of tests/unit/pomdp/pomdp_tests.cpp:69-135."""
    S = np.array([[[0, 1], [0, 1]], [[0, 1], [0, 1]]], np.int32)
    T = np.array([[[0.8, 0.2], [0.2, 0.8]], [[0.8, 0.2], [0.2, 0.8]]], np.float32)
    O = np.array([[[0.8, 0.2], [0.2, 0.8]], [[0.8, 0.2], [0.2, 0.8]]], np.float32)
    R = np.array([[-1.0, 1.0], [1.0, -1.0]], np.float32)
    Z = np.array([[0]], np.int32)
    B = np.array([[1.0]], np.float32)
    model = dict(n=2, ns=2, m=2, z=2, r=1, rz=1, gamma=float(np.float32(0.9)), horizon=3, S=S, T=T, O=O, R=R,
                 Z=Z, B=B, seed=0)
    model["GammaInitial"] = np.full((1, 2), np.float32(-1.0) / (np.float32(1.0) - np.float32(0.9)), np.float32)
    return model


def reference_loader():
    sys.path.insert(0, os.path.join(REF_DIR, "python", "nova"))
    import file_loader  # the reference's loader
    return file_loader.FileLoader()


def loader_fixtures():
    import raw_files
    mp = ragged(synth.random_pomdp(n=12, m=3, z=4, ns=3, r=6, rz=4, gamma=0.9, horizon=7, seed=51), seed=52)
    path = os.path.join(HERE, "loader_pomdp.raw")
    raw_files.write_raw_pomdp(mp, path, k=2)
    fl = reference_loader()
    fl.load_raw_pomdp(path)
    np.savez_compressed(os.path.join(HERE, "loader_pomdp.npz"), n=fl.n, ns=fl.ns, m=fl.m, z=fl.z, r=fl.r, rz=fl.rz,
                        horizon=fl.horizon, gamma=np.float32(fl.gamma), S=np.asarray(fl.S, np.int32),
                        T=np.asarray(fl.T, np.float32), O=np.asarray(fl.O, np.float32),
                        R=np.asarray(fl.R, np.float32), Z=np.asarray(fl.Z, np.int32), B=np.asarray(fl.B, np.float32))
    md = synth.random_mdp(n=15, m=2, ns=4, gamma=0.95, horizon=9, seed=53)
    path = os.path.join(HERE, "loader_mdp.raw")
    raw_files.write_raw_mdp(md, path, k=3, s0=2, goals=(4, 11))
    fl = reference_loader()
    fl.load_raw_mdp(path)
    np.savez_compressed(os.path.join(HERE, "loader_mdp.npz"), n=fl.n, ns=fl.ns, m=fl.m, horizon=fl.horizon,
                        gamma=np.float32(fl.gamma), s0=fl.s0, goals=np.asarray(fl.goals, np.uint32),
                        S=np.asarray(fl.S, np.int32), T=np.asarray(fl.T, np.float32),
                        R=np.asarray(fl.R, np.float32), epsilon=np.float32(fl.epsilon))
    print("wrote loader fixtures")


def cassandra_fixtures():
    """Synthetic Cassandra-format files (cassandra_files.py) read by the
    reference's FileLoader.load_cassandra; numpy's removed np.float alias,
    which its reward statements call, is provided as Python's float."""
    import cassandra_files
    if not hasattr(np, "float"):
        np.float = float
    for name, writer in cassandra_files.WRITERS.items():
        path = os.path.join(HERE, name + ".pomdp")
        writer(path)
        fl = reference_loader()
        try:
            fl.load_cassandra(path)
            # POMDP.load (pomdp.py:149-200) then needs every array and passes
            # the sizes to pomdp_initialize_cpu, whose checks
            # (pomdp_model_cpu.cpp:37-43) are applied here.
            ok = all(getattr(fl, k) is not None for k in ("S", "T", "O", "R", "Z", "B")) and \
                fl.n >= fl.ns >= 1 and min(fl.m, fl.z, fl.r, fl.rz) >= 1 and \
                0.0 <= np.float32(fl.gamma) <= 1.0 and 1 <= fl.horizon < 2 ** 32
        except Exception:
            ok = False
        if not ok:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), ok=np.int64(0))
            print("wrote", name, "(the reference fails to load it)")
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), ok=np.int64(1), n=fl.n, ns=fl.ns, m=fl.m, z=fl.z,
                            r=fl.r, rz=fl.rz, horizon=fl.horizon, gamma=np.float64(fl.gamma),
                            Rmin=np.float64(fl.Rmin), Rmax=np.float64(fl.Rmax), S=np.asarray(fl.S, np.int32),
                            T=np.asarray(fl.T, np.float32), O=np.asarray(fl.O, np.float32),
                            R=np.asarray(fl.R, np.float32), Z=np.asarray(fl.Z, np.int32),
                            B=np.asarray(fl.B, np.float32))
        print("wrote", name, "n=%d ns=%d m=%d z=%d rz=%d horizon=%d" % (fl.n, fl.ns, fl.m, fl.z, fl.rz, fl.horizon))


def main():
    if not orc.ref_available():
        raise SystemExit("the reference library is not available (needs %s)" % REF_DIR)

    m = synth.random_pomdp(**synth.POMDP_CONFIGS["pbvi_n64"], seed=0)
    G, pi = orc.ref_pbvi_solve(m, horizon=5)
    save("pbvi_n64_h5", dict(m, horizon=5), Gamma=G, pi=pi)
    G, pi = orc.ref_pbvi_solve(m)  # full horizon 100 (about 20 s)
    save("pbvi_n64_h100", m, Gamma=G, pi=pi)

    t = tiger()
    G, pi = orc.ref_pbvi_solve(t)
    save("pbvi_tiger", t, Gamma=G, pi=pi)
    G, pi = orc.ref_perseus_solve(t, seed=1, horizon=50)
    save("perseus_tiger", dict(t, horizon=50), Gamma=G, pi=pi, srand=np.int64(1))

    rg = ragged(synth.random_pomdp(n=37, m=3, z=5, ns=6, r=53, rz=7, gamma=0.9, horizon=20, seed=11), seed=12)
    G, pi = orc.ref_pbvi_solve(rg)
    save("pbvi_ragged", rg, Gamma=G, pi=pi)

    ts = two_state()
    G, pi = orc.ref_pbvi_solve(ts)
    save("pbvi_two_state_h3", ts, Gamma=G, pi=pi)
    ts10 = dict(ts, horizon=10)
    G, pi = orc.ref_pbvi_solve(ts10)
    save("pbvi_two_state_h10", ts10, Gamma=G, pi=pi)

    mp = synth.random_pomdp(n=32, m=3, z=4, ns=5, r=64, rz=6, gamma=0.9, horizon=8, seed=21)
    G, pi = orc.ref_perseus_solve(mp, seed=42)
    save("perseus_small", mp, Gamma=G, pi=pi, srand=np.int64(42))

    # Belief expansion and sigma approximation (the random forms seed from
    # the clock; the seed of a call that stayed within one second is stored).
    me = synth.random_pomdp(n=24, m=3, z=4, ns=5, r=30, rz=6, gamma=0.9, horizon=8, seed=3)
    Z, B = orc.ref_expand_distinct(me)
    save("expand_distinct", me, Z=Z, B=B)
    mr = ragged(synth.random_pomdp(n=20, m=2, z=3, ns=4, r=25, rz=5, gamma=0.9, horizon=6, seed=41), seed=42)
    # No empty belief here: for one the reference copies an uninitialised buffer.
    base = synth.random_pomdp(n=20, m=2, z=3, ns=4, r=25, rz=5, gamma=0.9, horizon=6, seed=41)
    mr["Z"][12], mr["B"][12] = base["Z"][12], base["B"][12]
    Z, B = orc.ref_expand_distinct(mr)
    save("expand_distinct_ragged", mr, Z=Z, B=B)
    Z, B, seed = orc.ref_expand_random(me, 40)
    save("expand_random", me, Z=Z, B=B, num=np.int64(40), srand=np.int64(seed))
    Bn, nz, seed = orc.ref_expand_random_from_b0(me, 25)
    save("expand_random_b0", me, Bnew=Bn, maxNonZero=np.int64(nz), num=np.int64(25), srand=np.int64(seed))
    G, pi = orc.ref_pbvi_solve(me, horizon=5)
    Z, B = orc.ref_expand_pema(me, G, pi)
    save("expand_pema", me, Z=Z, B=B, policyGamma=G, policyPi=pi)
    Z, B, sigma = orc.ref_sigma(me, 3)
    save("sigma_k3", me, Z=Z, B=B, sigma=np.float32(sigma), k=np.int64(3))

    # Raw-file loaders: files written by raw_files.py, parsed by the
    # reference's FileLoader; the parsed arrays are the fixture.
    loader_fixtures()
    cassandra_fixtures()

    md = synth.random_mdp(n=1000, m=4, ns=8, gamma=0.95, horizon=50, seed=31)
    rmd = ragged(dict(md, Z=np.zeros((2, 2), np.int32), B=np.zeros((2, 2), np.float32)), seed=32)
    md.update(S=rmd["S"], T=rmd["T"])
    V, pi = orc.ref_mdp_vi_solve(md)
    save("mdp_vi_ragged", md, V=V, pi=pi)
    V0 = np.random.Generator(np.random.PCG64(33)).uniform(-5, 5, size=md["n"]).astype(np.float32)
    V, pi = orc.ref_mdp_vi_solve(dict(md, horizon=7), VInitial=V0)
    save("mdp_vi_vinit", dict(md, horizon=7, VInitial=V0), V=V, pi=pi)


if __name__ == "__main__":
    main()
