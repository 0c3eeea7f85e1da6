"""Host-side behaviour of the C library that needs no GPU: model allocation,
argument validation and error codes, policy containers, belief update,
fault injection wiring."""
import ctypes as ct
import os

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as orc
from nova_gb300 import _lib
from nova_gb300.pomdp import POMDP
from nova_gb300.mdp import MDP
from nova_gb300 import nova_pomdp as npm, nova_pomdp_pbvi as npp, nova_mdp_vi as nmvi
from nova_gb300 import pomdp_alpha_vectors as pav, mdp_value_function as mvf
from nova_gb300 import nova_pomdp_perseus as npper

L = _lib.load()
NOVA_SUCCESS, INVALID_DATA, INVALID_CUDA_PARAM, DEVICE_MALLOC = 0, 1, 2, 3


def test_pomdp_initialize_validation_and_defaults():
    p = npm.NovaPOMDP()
    assert L.pomdp_initialize_cpu(ct.byref(p), 0, 1, 1, 1, 1, 1, 0.9, 1) == INVALID_DATA
    assert L.pomdp_initialize_cpu(ct.byref(p), 2, 3, 1, 1, 1, 1, 0.9, 1) == INVALID_DATA  # n < ns
    assert L.pomdp_initialize_cpu(ct.byref(p), 3, 2, 2, 2, 4, 2, 1.5, 1) == INVALID_DATA  # gamma > 1
    assert L.pomdp_initialize_cpu(ct.byref(p), 3, 2, 2, 2, 4, 2, 0.9, 10) == NOVA_SUCCESS
    assert (p.n, p.ns, p.m, p.z, p.r, p.rz, p.horizon) == (3, 2, 2, 2, 4, 2, 10)
    assert all(p.S[i] == -1 for i in range(3 * 2 * 2)) and all(p.T[i] == 0.0 for i in range(12))
    assert all(p.Z[i] == 0 for i in range(8))
    assert not p.d_S and not p.d_B
    # a second initialize on allocated arrays is rejected (pomdp_model_cpu.cpp:37-38)
    assert L.pomdp_initialize_cpu(ct.byref(p), 3, 2, 2, 2, 4, 2, 0.9, 10) == INVALID_DATA
    assert L.pomdp_uninitialize_cpu(ct.byref(p)) == NOVA_SUCCESS
    assert not p.S and p.n == 0


def test_mdp_initialize_validation():
    m = nmvi.mdp.MDP()
    assert L.mdp_initialize_cpu(ct.byref(m), 4, 2, 2, 0.9, 5, 0.001, 4, 0) == INVALID_DATA  # s0 >= n
    assert L.mdp_initialize_cpu(ct.byref(m), 4, 2, 2, 0.9, 5, 0.001, 0, 1) == NOVA_SUCCESS
    assert m.goals and m.goals[0] == 0
    assert L.mdp_uninitialize_cpu(ct.byref(m)) == NOVA_SUCCESS


def test_alpha_vectors_reference_values_through_library():
    # pomdp_alpha_vectors_tests.cpp:35-89, through pomdp_alpha_vectors_value_and_action
    pol = pav.POMDPAlphaVectors()
    assert L.pomdp_alpha_vectors_initialize(pol, 2, 2, 2) == NOVA_SUCCESS
    for k, v in enumerate([1.0, 0.0, 0.0, 1.0]):
        pol.Gamma[k] = v
    pol.pi[0], pol.pi[1] = 1, 0
    for b, v, a in (([0.0, 1.0], 1.0, 0), ([1.0, 0.0], 1.0, 1), ([0.25, 0.75], 0.75, 0), ([0.67, 0.33], 0.67, 1)):
        V, act = pol.value_and_action(np.array(b, np.float32))
        assert abs(V - v) < 1e-5 and act == a
    # initialize refuses a policy that already holds arrays
    assert L.pomdp_alpha_vectors_initialize(pol, 2, 2, 2) == INVALID_DATA


def test_alpha_value_matches_oracle_on_fixture():
    g = load_golden("pbvi_n64_h100")
    pol = pav.POMDPAlphaVectors()
    assert L.pomdp_alpha_vectors_initialize(pol, g["n"], g["m"], g["r"]) == NOVA_SUCCESS
    G = np.ascontiguousarray(g["out_Gamma"])
    ct.memmove(pol.Gamma, G.ctypes.data, G.nbytes)
    ct.memmove(pol.pi, g["out_pi"].ctypes.data, g["out_pi"].nbytes)
    for i in range(5):
        b = np.zeros(g["n"], np.float32)
        b[g["Z"][i]] = g["B"][i]
        assert pol.value_and_action(b) == orc.alpha_value(G, g["out_pi"], b)


def test_value_function_dense_and_sparse():
    vf = mvf.MDPValueFunction()
    assert L.mdp_value_function_initialize(vf, 5, 2, 0) == NOVA_SUCCESS
    assert not vf.S and vf.V and vf.pi
    vf2 = mvf.MDPValueFunction()
    assert L.mdp_value_function_initialize(vf2, 5, 2, 3) == NOVA_SUCCESS
    assert vf2.S and vf2.r == 3
    assert L.mdp_value_function_initialize(vf2, 5, 2, 3) == INVALID_DATA


def test_belief_update_and_raw_beliefs():
    g = load_golden("pbvi_tiger")
    p = POMDP.from_arrays(g)
    b = np.array([0.5, 0.5], np.float32)
    bp = p.belief_update(b, 0, 0)
    # numpy restatement of pomdp_model_cpu.cpp:89-137 for the tiger 'listen' action
    expect = np.zeros(2, np.float32)
    for s in range(2):
        for l in range(g["ns"]):
            sp = g["S"][s, 0, l]
            if sp < 0:
                break
            expect[sp] += g["T"][s, 0, l] * b[s]
    expect *= g["O"][0, :, 0]
    expect /= expect.sum()
    np.testing.assert_allclose(bp, expect, rtol=1e-6)
    r0, rz0 = p.r, p.rz
    Bnew = np.array([[0.3, 0.7], [1.0, 0.0]], np.float32)
    assert L.pomdp_add_new_raw_beliefs_cpu(p, 2, Bnew.ctypes.data_as(ct.POINTER(ct.c_float))) == NOVA_SUCCESS
    assert p.r == r0 + 2 and p.rz == max(rz0, 2)
    assert [p.Z[(r0) * p.rz + k] for k in range(2)] == [0, 1]
    assert p.Z[(r0 + 1) * p.rz + 1] == -1


def test_execute_validation_before_any_device_work():
    g = load_golden("pbvi_tiger")
    p = POMDP.from_arrays(g)
    pol = pav.POMDPAlphaVectors()
    alg = npp.NovaPOMDPPBVIGPU()
    # no device model: invalid data
    assert L.pomdp_pbvi_execute_gpu(p, ct.byref(alg), pol) == INVALID_DATA
    # with (never dereferenced) device pointers and a bad numThreads: invalid CUDA parameter
    fake = ct.cast(ct.c_void_p(0x1000), ct.POINTER(ct.c_int))
    fakef = ct.cast(ct.c_void_p(0x1000), ct.POINTER(ct.c_float))
    p.d_S, p.d_Z = fake, fake
    p.d_T, p.d_O, p.d_R, p.d_B = fakef, fakef, fakef, fakef
    G0 = (ct.c_float * (g["r"] * g["n"]))()
    alg.GammaInitial = ct.cast(G0, ct.POINTER(ct.c_float))
    alg.numThreads = 48
    assert L.pomdp_pbvi_execute_gpu(p, ct.byref(alg), pol) == INVALID_CUDA_PARAM
    p.d_S = p.d_Z = ct.POINTER(ct.c_int)()
    p.d_T = p.d_O = p.d_R = p.d_B = ct.POINTER(ct.c_float)()
    # CPU-buffer entry points validate too
    cpu = npp.NovaPOMDPPBVICPU()
    assert L.pomdp_pbvi_execute_cpu(p, ct.byref(cpu), pol) == INVALID_DATA  # no GammaInitial
    per = npper.NovaPOMDPPerseusCPU()
    assert L.pomdp_perseus_execute_cpu(p, ct.byref(per), pol) == INVALID_DATA
    assert L.pomdp_pbvi_update_gpu(p, ct.byref(alg)) == INVALID_DATA
    assert L.mdp_vi_execute_gpu(None, None, None) == INVALID_DATA
    # solver settings reject a null or uninitialized solver and unknown modes
    # before any device work
    assert L.pomdp_pbvi_set_table_gpu(None, npp.TABLE_NEVER) == INVALID_DATA
    assert L.pomdp_pbvi_set_table_gpu(ct.byref(alg), npp.TABLE_NEVER) == INVALID_DATA
    assert L.pomdp_pbvi_set_table_gpu(ct.byref(alg), 7) == INVALID_DATA
    assert L.pomdp_pbvi_set_scoring_gpu(ct.byref(alg), npp.SCORING_FP16) == INVALID_DATA
    assert L.pomdp_pbvi_set_scoring_gpu(ct.byref(alg), 9) == INVALID_DATA


def test_fault_injection_hook_is_wired():
    """An armed allocation fault fails the next device allocation on the host,
    before CUDA is called, with the reference's error code."""
    g = load_golden("pbvi_tiger")
    p = POMDP.from_arrays(g)
    L.nova_gb300_inject_fault(1, 1)
    assert L.pomdp_initialize_successors_gpu(p) == DEVICE_MALLOC
    assert not p.d_S
    L.nova_gb300_inject_fault(0, 0)


# ---------------------------------------------------------------------------
# Raw-file loaders (host code; no GPU)
# ---------------------------------------------------------------------------

def test_raw_pomdp_loader_matches_reference_loader():
    from conftest import GOLDEN
    from nova_gb300.pomdp import POMDP
    g = np.load(os.path.join(GOLDEN, "loader_pomdp.npz"))
    p = POMDP()
    p.load(os.path.join(GOLDEN, "loader_pomdp.raw"), filetype="raw")
    out = p.arrays()
    for k in ("n", "ns", "m", "z", "r", "rz", "horizon"):
        assert out[k] == int(g[k])
    assert np.float32(out["gamma"]) == g["gamma"]
    for k in ("S", "Z"):
        np.testing.assert_array_equal(out[k], g[k])
    for k in ("T", "O", "R", "B"):
        np.testing.assert_array_equal(out[k].view(np.uint32), g[k].view(np.uint32))
    assert p.Rmin == float(g["R"].min())


def test_raw_mdp_loader_matches_reference_loader():
    from conftest import GOLDEN
    from nova_gb300.mdp import MDP
    g = np.load(os.path.join(GOLDEN, "loader_mdp.npz"))
    m = MDP()
    m.load(os.path.join(GOLDEN, "loader_mdp.raw"), filetype="raw")
    assert (m.n, m.ns, m.m, m.horizon, m.s0, m.ng) == (int(g["n"]), int(g["ns"]), int(g["m"]), int(g["horizon"]),
                                                      int(g["s0"]), len(g["goals"]))
    assert np.float32(m.gamma) == g["gamma"] and np.float32(m.epsilon) == g["epsilon"]
    S = np.ctypeslib.as_array(m.S, shape=(m.n * m.m * m.ns,)).reshape(m.n, m.m, m.ns)
    T = np.ctypeslib.as_array(m.T, shape=(m.n * m.m * m.ns,)).reshape(m.n, m.m, m.ns)
    R = np.ctypeslib.as_array(m.R, shape=(m.n * m.m,)).reshape(m.n, m.m)
    goals = np.ctypeslib.as_array(m.goals, shape=(m.ng,))
    np.testing.assert_array_equal(S, g["S"])
    np.testing.assert_array_equal(T.view(np.uint32), g["T"].view(np.uint32))
    np.testing.assert_array_equal(R.view(np.uint32), g["R"].view(np.uint32))
    np.testing.assert_array_equal(goals, g["goals"])


def test_raw_loader_rejects_bad_files(tmp_path):
    from nova_gb300.pomdp import POMDP
    bad = tmp_path / "bad.raw"
    bad.write_text("3,2,2,2,1,1,1,0,5,0.9\n0,1\n")
    p = POMDP()
    with pytest.raises(Exception):
        p.load(str(bad), filetype="raw")
    with pytest.raises(Exception):
        POMDP().load(str(tmp_path / "missing.raw"), filetype="raw")


@pytest.mark.skipif(not os.path.isfile(os.path.join(orc.REF_DIR, "tests", "tiger", "tiger_pomdp.raw")),
                    reason="reference fixtures not present")
def test_raw_loader_on_reference_tiger_file():
    import sys
    from nova_gb300.pomdp import POMDP
    sys.path.insert(0, os.path.join(orc.REF_DIR, "python", "nova"))
    import file_loader
    path = os.path.join(orc.REF_DIR, "tests", "tiger", "tiger_pomdp.raw")
    fl = file_loader.FileLoader()
    fl.load_raw_pomdp(path)
    p = POMDP()
    p.load(path, filetype="raw")
    out = p.arrays()
    for k, t in (("S", np.int32), ("T", np.float32), ("O", np.float32), ("R", np.float32), ("Z", np.int32),
                 ("B", np.float32)):
        np.testing.assert_array_equal(out[k], np.asarray(getattr(fl, k), t))


# ---------------------------------------------------------------------------
# Cassandra-format loader (host code; no GPU)
# ---------------------------------------------------------------------------

CASSANDRA_FIXTURES = ["cass_named", "cass_counts", "cass_exclude", "cass_single_start", "cass_start_uniform",
                      "cass_no_reward", "cass_long_rows"]


def _check_cassandra(p, g):
    out = p.arrays()
    for k in ("n", "ns", "m", "z", "r", "rz", "horizon"):
        assert out[k] == int(g[k]), k
    assert np.float32(out["gamma"]) == np.float32(g["gamma"])
    for k in ("S", "Z"):
        np.testing.assert_array_equal(out[k], np.asarray(g[k], np.int32).reshape(out[k].shape))
    for k in ("T", "O", "R", "B"):
        np.testing.assert_array_equal(out[k].view(np.uint32),
                                      np.asarray(g[k], np.float32).reshape(out[k].shape).view(np.uint32))
    assert p.Rmin == float(g["Rmin"]) and p.Rmax == float(g["Rmax"])


@pytest.mark.parametrize("name", CASSANDRA_FIXTURES)
def test_cassandra_loader_matches_reference_loader(name):
    """Synthetic files (tests/golden/cassandra_files.py) against the arrays the
    reference's FileLoader.load_cassandra produced for them; files the
    reference fails to load must fail here too."""
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = POMDP()
    path = os.path.join(GOLDEN, name + ".pomdp")
    if int(g["ok"]) == 0:
        with pytest.raises(Exception):
            p.load(path, filetype="cassandra")
        assert not p.S
        return
    p.load(path, filetype="cassandra")
    _check_cassandra(p, g)


def test_cassandra_loader_rejects_missing_file(tmp_path):
    with pytest.raises(Exception):
        POMDP().load(str(tmp_path / "missing.pomdp"), filetype="cassandra")
    with pytest.raises(Exception):
        POMDP().load(str(tmp_path / "missing.pomdp"), filetype="xml")


_REF_DOMAINS = os.path.join(orc.REF_DIR, "tests", "benchmarks", "algorithms", "domains")


@pytest.mark.skipif(not os.path.isdir(_REF_DOMAINS), reason="reference domain files not present")
@pytest.mark.parametrize("name", ["4x3_95", "aloha_10", "drive_san_francisco", "hallway2", "mit", "paint_95",
                                  "shuttle_95", "tag", "tiger_95", "tiger_grid"])
def test_cassandra_loader_on_reference_domains(name):
    """The reference's own benchmark domains, loaded by its Python loader
    (numpy's removed np.float alias provided as float) and by ours."""
    import importlib.util
    if not hasattr(np, "float"):
        np.float = float
    spec = importlib.util.spec_from_file_location("ref_file_loader",
                                                  os.path.join(orc.REF_DIR, "python", "nova", "file_loader.py"))
    fl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fl)
    path = os.path.join(_REF_DOMAINS, name + ".pomdp")
    L = fl.FileLoader()
    L.load_cassandra(path)
    p = POMDP()
    p.load(path, filetype="cassandra")
    g = dict(n=L.n, ns=L.ns, m=L.m, z=L.z, r=L.r, rz=L.rz, horizon=L.horizon, gamma=L.gamma, S=L.S, T=L.T, O=L.O,
             R=L.R, Z=L.Z, B=L.B, Rmin=L.Rmin, Rmax=L.Rmax)
    _check_cassandra(p, g)


def test_text_forms_of_models_and_solvers():
    """__str__ of the MDP and of the VI and Perseus solver objects, as the
    reference's wrapper offers, built without device work (the solver objects
    are made with their fields set directly)."""
    from nova_gb300 import synth
    from nova_gb300.mdp import MDP
    from nova_gb300.mdp_vi import MDPValueIterationCPU, MDPValueIterationGPU
    from nova_gb300.pomdp_perseus import POMDPPerseusCPU, POMDPPerseusGPU
    md = synth.random_mdp(n=3, m=2, ns=2, gamma=0.9, horizon=4, seed=3)
    m = MDP.from_arrays(md)
    text = str(m)
    assert "n:       3" in text and "horizon: 4" in text and "S(s, a, s'):" in text and "R(s, a):" in text
    V0 = (ct.c_float * 3)(1.0, 2.0, 3.0)
    def bare(cls):
        # An instance without __init__ (no device work) and nothing to free.
        sub = type("Bare" + cls.__name__, (cls,), {"__del__": lambda self: None})
        return sub.__new__(sub)

    for cls in (MDPValueIterationCPU, MDPValueIterationGPU):
        vi = bare(cls)
        vi.mdp = m
        vi.Vinitial = ct.cast(V0, ct.POINTER(ct.c_float))
        vi.currentHorizon = 2
        if issubclass(type(vi), MDPValueIterationCPU):
            vi.V, vi.Vprime, vi.pi = ct.POINTER(ct.c_float)(), ct.POINTER(ct.c_float)(), ct.POINTER(ct.c_uint)()
            t = str(vi)
            assert "currentHorizon: 2" in t and "[1. 2. 3.]" in t and "V:\n(none)" in t
        else:
            vi.numThreads = 64
            t = str(vi)
            assert "numThreads: 64" in t and "[1. 2. 3.]" in t
    pm = synth.random_pomdp(n=2, m=2, z=2, ns=2, r=2, rz=2, gamma=0.9, horizon=2, seed=3)
    p = POMDP.from_arrays(pm)
    G0 = (ct.c_float * 4)(1.0, 2.0, 3.0, 4.0)
    for cls in (POMDPPerseusCPU, POMDPPerseusGPU):
        per = bare(cls)
        per.pomdp = p
        per.GammaInitial = ct.cast(G0, ct.POINTER(ct.c_float))
        per.currentHorizon, per.rGamma, per.rGammaPrime, per.rTilde = 1, 2, 0, 2
        per.numThreads = 32
        t = str(per)
        assert "rGamma: 2" in t and "rTilde: 2" in t and "[[1. 2.]\n [3. 4.]]" in t
        assert ("numThreads: 32" in t) == issubclass(type(per), POMDPPerseusGPU)
