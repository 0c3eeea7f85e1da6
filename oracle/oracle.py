"""ORACLE -- test infrastructure only (tests/, __graft_entry__.smoke(), the CPU
baseline leg of bench.py). The product library never imports this module.

Two CPU implementations of nova's hot-path algorithms, behind one numpy API:

* the C restatement in oracle/nova_oracle.c (`liboracle`), built by
  oracle/Makefile wherever the tests run (x86 here, Arm on the GPU machine);
* the reference itself: nova's own CPU sources compiled by `make -C oracle ref`
  into oracle/_ref/libnova_ref.so, called through nova's own C API
  (pomdp_pbvi_execute_cpu, mdp_vi_execute_cpu, ...). It exists only where the
  reference sources are present; `ref_available()` says whether it loaded.

The restatement is pinned bit for bit to the reference by tests/test_oracle.py
and by the fixtures in tests/golden/ (made by tests/golden/make_golden.py from
the reference).
"""
import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnova_ref.so")
# The one setting for where the reference project lies: NOVA_REFERENCE_DIR,
# else the place it is mounted read-only in the build container. Where neither
# holds its sources (the GPU host), everything that needs them is skipped.
REF_DIR = os.environ.get("NOVA_REFERENCE_DIR", "/root/reference")

_F = ct.POINTER(ct.c_float)
_I = ct.POINTER(ct.c_int)
_U = ct.POINTER(ct.c_uint)
_D = ct.POINTER(ct.c_double)

_oracle = None
_ref = None


def build(with_ref=None):
    """Build liboracle.so (and the reference library when its sources exist)."""
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REF_DIR, "src"))
    target = "ref" if with_ref else "all"
    subprocess.run(["make", "-s", "-C", HERE, target, "REF_DIR=" + REF_DIR], check=True,
                   stdout=subprocess.DEVNULL)


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
                os.path.join(HERE, "nova_oracle.c")):
            build(with_ref=False)
        _oracle = ct.CDLL(ORACLE_SO)
        L = _oracle
        L.oracle_pbvi_update_range.argtypes = [ct.c_uint] * 6 + [ct.c_float, _I, _F, _F, _F, _I, _F, _F, _F, _U,
                                                                 ct.c_uint, ct.c_uint]
        L.oracle_pbvi_update.argtypes = [ct.c_uint] * 6 + [ct.c_float, _I, _F, _F, _F, _I, _F, _F, _F, _U]
        L.oracle_pbvi_solve.argtypes = [ct.c_uint] * 6 + [ct.c_float, ct.c_uint, _I, _F, _F, _F, _I, _F, _F, _F, _U]
        L.oracle_pbvi_update_factored.argtypes = [ct.c_uint] * 6 + [ct.c_float, _I, _F, _F, _F, _I, _F, _F, _F, _U,
                                                                    ct.c_uint, ct.c_uint, _U]
        L.oracle_pbvi_update_f64.argtypes = [ct.c_uint] * 6 + [ct.c_double, _I, _D, _D, _D, _I, _D, _D, _D, _U]
        L.oracle_alpha_value.argtypes = [ct.c_uint, ct.c_uint, _F, _U, _F, _F, _U]
        L.oracle_mdp_vi_sweep.argtypes = [ct.c_uint, ct.c_uint, ct.c_uint, ct.c_float, _I, _F, _F, _F, _F, _U]
        L.oracle_mdp_vi_solve.argtypes = [ct.c_uint, ct.c_uint, ct.c_uint, ct.c_float, ct.c_uint, _I, _F, _F, _F,
                                          _F, _U]
        L.oracle_perseus_solve.argtypes = [ct.c_uint] * 6 + [ct.c_float, ct.c_uint, _I, _F, _F, _F, _I, _F, _F,
                                                             _F, _U]
        L.oracle_perseus_solve.restype = ct.c_int
        L.oracle_srand.argtypes = [ct.c_uint]
        L.oracle_pbvi_belief_action.argtypes = [ct.c_uint] * 6 + [ct.c_float, _I, _F, _F, _F, _I, _F, _F, ct.c_uint,
                                                                  ct.c_uint, _F]
        L.oracle_pbvi_belief_action.restype = ct.c_float
        fixed = [ct.c_uint] * 5 + [ct.c_double, _I, _D, _D, _D, _D, ct.c_uint, _U, _U, _D]
        L.oracle_pbvi_fixed_forward_f64.argtypes = fixed + [_U, _D]
        L.oracle_pbvi_fixed_forward_f64.restype = ct.c_double
        L.oracle_pbvi_fixed_reverse_f64.argtypes = fixed + [ct.c_uint, _D, _D, _D, _D]
        L.oracle_pbvi_fixed_reverse_f64.restype = ct.c_double
    return _oracle


def ref_available():
    return ref_lib() is not None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO) and os.path.isdir(os.path.join(REF_DIR, "src")):
            try:
                build(with_ref=True)
            except Exception:
                return None
        if not os.path.exists(REF_SO):
            return None
        _ref = ct.CDLL(REF_SO)
    return _ref


def _p(a, t):
    return a.ctypes.data_as(t)


def _arrays(model):
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    T = np.ascontiguousarray(model["T"], dtype=np.float32)
    O = np.ascontiguousarray(model["O"], dtype=np.float32)
    R = np.ascontiguousarray(model["R"], dtype=np.float32)
    Z = np.ascontiguousarray(model["Z"], dtype=np.int32)
    B = np.ascontiguousarray(model["B"], dtype=np.float32)
    return S, T, O, R, Z, B


def _dims(model):
    return (model["n"], model["ns"], model["m"], model["z"], model["r"], model["rz"])


# ---------------------------------------------------------------------------
# Restatement (liboracle)
# ---------------------------------------------------------------------------

def pbvi_solve(model, horizon=None, GammaInitial=None):
    """nova's PBVI CPU solve (loop form); returns (Gamma [r,n], pi [r])."""
    L = lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    G0 = np.ascontiguousarray(model["GammaInitial"] if GammaInitial is None else GammaInitial, dtype=np.float32)
    Gout = np.empty((r, n), np.float32)
    pi = np.empty(r, np.uint32)
    L.oracle_pbvi_solve(n, ns, m, z, r, rz, model["gamma"], model["horizon"] if horizon is None else horizon,
                        _p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F), _p(Z, _I), _p(B, _F), _p(G0, _F),
                        _p(Gout, _F), _p(pi, _U))
    return Gout, pi


def pbvi_update(model, Gamma, GammaPrime, pi, i0=0, i1=None, factored=True, jstar=None):
    """One backup of beliefs [i0, i1) in place into GammaPrime/pi (bit-identical forms)."""
    L = lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    i1 = r if i1 is None else i1
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    assert GammaPrime.dtype == np.float32 and GammaPrime.flags.c_contiguous
    assert pi.dtype == np.uint32 and pi.flags.c_contiguous
    if factored:
        js = _p(jstar, _U) if jstar is not None else None
        L.oracle_pbvi_update_factored(n, ns, m, z, r, rz, model["gamma"], _p(S, _I), _p(T, _F), _p(O, _F),
                                      _p(R, _F), _p(Z, _I), _p(B, _F), _p(G, _F), _p(GammaPrime, _F), _p(pi, _U),
                                      i0, i1, js)
    else:
        L.oracle_pbvi_update_range(n, ns, m, z, r, rz, model["gamma"], _p(S, _I), _p(T, _F), _p(O, _F),
                                   _p(R, _F), _p(Z, _I), _p(B, _F), _p(G, _F), _p(GammaPrime, _F), _p(pi, _U),
                                   i0, i1)


def pbvi_update_f64(model, Gamma):
    """FP64 backup of every belief; returns (GammaPrime [r,n] float64, pi)."""
    L = lib()
    n, ns, m, z, r, rz = _dims(model)
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    Z = np.ascontiguousarray(model["Z"], dtype=np.int32)
    T, O, R, B = (np.ascontiguousarray(model[k], dtype=np.float64) for k in ("T", "O", "R", "B"))
    G = np.ascontiguousarray(Gamma, dtype=np.float64)
    Gp = G.copy()
    pi = np.zeros(r, np.uint32)
    L.oracle_pbvi_update_f64(n, ns, m, z, r, rz, float(model["gamma"]), _p(S, _I), _p(T, _D), _p(O, _D),
                             _p(R, _D), _p(Z, _I), _p(B, _D), _p(G, _D), _p(Gp, _D), _p(pi, _U))
    return Gp, pi


def pbvi_belief_action_sampler(model, Gamma):
    """A callable (i, a) -> value running one (belief, action) pair of nova's
    loop-form backup against Gamma (the unit the CPU baseline times). The
    ctypes call releases the GIL, so threads run in parallel."""
    L = lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    keep = (S, T, O, R, Z, B, G)
    ptrs = (_p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F), _p(Z, _I), _p(B, _F), _p(G, _F))

    def run(i, a):
        out = np.empty(n, np.float32)
        _ = keep
        return L.oracle_pbvi_belief_action(n, ns, m, z, G.shape[0], rz, model["gamma"], *ptrs, i, a,
                                           _p(out, _F))
    return run


def pbvi_backup_beliefs(model, Gamma, beliefs, threads=None):
    """nova's loop-form backup (pomdp_pbvi_cpu.cpp:106-162) of the listed
    beliefs only, against the full alpha set Gamma: returns (rows [k, n],
    pi [k], kept [k]) where rows[t] / pi[t] are what the update writes for
    belief beliefs[t] and kept[t] says no action beat the -1e10 sentinel (the
    update then leaves that belief's row and action untouched; rows[t] is
    undefined). The (belief, action) pairs run on `threads` host threads
    (default: all), as each ctypes call releases the GIL."""
    import threading
    L = lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    beliefs = [int(i) for i in beliefs]
    k = len(beliefs)
    alphas = np.empty((k, m, n), np.float32)
    values = np.empty((k, m), np.float32)
    ptrs = (_p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F), _p(Z, _I), _p(B, _F), _p(G, _F))
    jobs = [(t, a) for t in range(k) for a in range(m)]
    lock = threading.Lock()
    nxt = [0]

    def worker():
        while True:
            with lock:
                if nxt[0] >= len(jobs):
                    return
                t, a = jobs[nxt[0]]
                nxt[0] += 1
            out = alphas[t, a]
            values[t, a] = L.oracle_pbvi_belief_action(n, ns, m, z, G.shape[0], rz, model["gamma"], *ptrs,
                                                       beliefs[t], a, _p(out, _F))
    if threads is None:
        try:
            threads = len(os.sched_getaffinity(0))
        except Exception:
            threads = os.cpu_count() or 1
    ts = [threading.Thread(target=worker) for _ in range(max(1, min(threads, len(jobs))))]
    for th in ts:
        th.start()
    for th in ts:
        th.join()
    rows = np.zeros((k, n), np.float32)
    pi = np.zeros(k, np.uint32)
    kept = np.ones(k, bool)
    for t in range(k):
        best = np.float32(-1e10)
        for a in range(m):   # strict '>' from nova's -1e10 start: the lowest action wins ties
            if values[t, a] > best:
                best = values[t, a]
                rows[t] = alphas[t, a]
                pi[t] = a
                kept[t] = False
    return rows, pi, kept


def choose_parity_beliefs(candidates, exactRows, k=16, seed=0):
    """k beliefs for a sampled parity check of one tensor-core update: up to
    k/4 with rows sent to the exact scan (most such rows first), then those
    with the most alphas re-scored in the merge up to 3k/4, then random ones."""
    candidates = np.asarray(candidates).astype(np.int64)
    exactRows = np.asarray(exactRows).astype(np.int64)
    r = len(candidates)
    chosen = [int(i) for i in np.argsort(-exactRows, kind="stable")[:k // 4] if exactRows[i] > 0]
    for i in np.argsort(-candidates, kind="stable"):
        if len(chosen) >= (3 * k) // 4:
            break
        if int(i) not in chosen:
            chosen.append(int(i))
    rng = np.random.default_rng(seed)
    while len(chosen) < min(k, r):
        i = int(rng.integers(0, r))
        if i not in chosen:
            chosen.append(i)
    return chosen


def sampled_backup_parity(model, Gamma, GammaPrime, pi, beliefs, threads=None):
    """Bits of GammaPrime rows and pi for the listed beliefs against nova's
    loop-form backup of Gamma (pbvi_backup_beliefs). Returns the list of
    beliefs whose row or action differ (beliefs that no action improves must
    keep their row, which the caller checks)."""
    rows, p, kept = pbvi_backup_beliefs(model, Gamma, beliefs, threads)
    bad = []
    for t, i in enumerate(beliefs):
        if kept[t]:
            continue
        if not (np.array_equal(rows[t].view(np.uint32), np.ascontiguousarray(GammaPrime[i], np.float32)
                               .view(np.uint32)) and int(p[t]) == int(pi[i])):
            bad.append(int(i))
    return bad


def alpha_value(Gamma, pi, b):
    """nova's V(b) (FP32, strict '<'); returns (V, action)."""
    L = lib()
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    p = np.ascontiguousarray(pi, dtype=np.uint32)
    bb = np.ascontiguousarray(b, dtype=np.float32)
    V = ct.c_float(0)
    a = ct.c_uint(0)
    L.oracle_alpha_value(G.shape[1], G.shape[0], _p(G, _F), _p(p, _U), _p(bb, _F), ct.byref(V), ct.byref(a))
    return V.value, a.value


def mdp_vi_solve(model, horizon=None, VInitial=None):
    """nova's VI CPU solve; returns (V [n], pi [n])."""
    L = lib()
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    T = np.ascontiguousarray(model["T"], dtype=np.float32)
    R = np.ascontiguousarray(model["R"], dtype=np.float32)
    n = model["n"]
    V = np.empty(n, np.float32)
    pi = np.empty(n, np.uint32)
    V0 = None if VInitial is None else np.ascontiguousarray(VInitial, dtype=np.float32)
    L.oracle_mdp_vi_solve(n, model["ns"], model["m"], model["gamma"],
                          model["horizon"] if horizon is None else horizon, _p(S, _I), _p(T, _F), _p(R, _F),
                          _p(V0, _F) if V0 is not None else None, _p(V, _F), _p(pi, _U))
    return V, pi


def mdp_vi_sweep(model, V):
    """One Bellman sweep; returns (V', pi)."""
    L = lib()
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    T = np.ascontiguousarray(model["T"], dtype=np.float32)
    R = np.ascontiguousarray(model["R"], dtype=np.float32)
    Vin = np.ascontiguousarray(V, dtype=np.float32)
    n = model["n"]
    Vp = np.empty(n, np.float32)
    pi = np.empty(n, np.uint32)
    L.oracle_mdp_vi_sweep(n, model["ns"], model["m"], model["gamma"], _p(S, _I), _p(T, _F), _p(R, _F),
                          _p(Vin, _F), _p(Vp, _F), _p(pi, _U))
    return Vp, pi


def perseus_solve(model, seed, horizon=None, GammaInitial=None):
    """nova's Perseus CPU solve after srand(seed); returns (Gamma rows, pi)."""
    L = lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    G0 = np.ascontiguousarray(model["GammaInitial"] if GammaInitial is None else GammaInitial, dtype=np.float32)
    Gout = np.zeros((r, n), np.float32)
    pi = np.zeros(r, np.uint32)
    L.oracle_srand(seed)
    rows = L.oracle_perseus_solve(n, ns, m, z, r, rz, model["gamma"], model["horizon"] if horizon is None else horizon,
                                  _p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F), _p(Z, _I), _p(B, _F), _p(G0, _F),
                                  _p(Gout, _F), _p(pi, _U))
    if rows < 0:
        raise RuntimeError("oracle Perseus failed")
    return Gout[:rows].copy(), pi[:rows].copy()


# ---------------------------------------------------------------------------
# The reference itself (oracle/_ref/libnova_ref.so), through nova's C API
# ---------------------------------------------------------------------------

class _RefPOMDP(ct.Structure):
    _fields_ = [("n", ct.c_uint), ("ns", ct.c_uint), ("m", ct.c_uint), ("z", ct.c_uint), ("r", ct.c_uint),
                ("rz", ct.c_uint), ("gamma", ct.c_float), ("horizon", ct.c_uint),
                ("S", _I), ("T", _F), ("O", _F), ("R", _F), ("Z", _I), ("B", _F),
                ("d_S", _I), ("d_T", _F), ("d_O", _F), ("d_R", _F), ("d_Z", _I), ("d_B", _F)]


class _RefMDP(ct.Structure):
    _fields_ = [("n", ct.c_uint), ("ns", ct.c_uint), ("m", ct.c_uint), ("gamma", ct.c_float),
                ("horizon", ct.c_uint), ("epsilon", ct.c_float), ("s0", ct.c_uint), ("ng", ct.c_uint),
                ("goals", _U), ("S", _I), ("T", _F), ("R", _F), ("d_goals", _U), ("d_S", _I), ("d_T", _F),
                ("d_R", _F)]


class _RefAlpha(ct.Structure):
    _fields_ = [("n", ct.c_uint), ("m", ct.c_uint), ("r", ct.c_uint), ("Gamma", _F), ("pi", _U)]


class _RefVF(ct.Structure):
    _fields_ = [("n", ct.c_uint), ("m", ct.c_uint), ("r", ct.c_uint), ("S", _U), ("V", _F), ("pi", _U)]


class _RefPBVI(ct.Structure):
    _fields_ = [("GammaInitial", _F), ("currentHorizon", ct.c_uint), ("Gamma", _F), ("GammaPrime", _F), ("pi", _U)]


class _RefPerseus(ct.Structure):
    _fields_ = [("GammaInitial", _F), ("currentHorizon", ct.c_uint), ("rGamma", ct.c_uint),
                ("rGammaPrime", ct.c_uint), ("rTilde", ct.c_uint), ("BTilde", _U), ("Gamma", _F),
                ("GammaPrime", _F), ("pi", _U), ("piPrime", _U)]


class _RefVI(ct.Structure):
    _fields_ = [("VInitial", _F), ("currentHorizon", ct.c_uint), ("V", _F), ("VPrime", _F), ("pi", _U)]


def _ref_pomdp(model, keep):
    S, T, O, R, Z, B = _arrays(model)
    keep.extend([S, T, O, R, Z, B])
    p = _RefPOMDP()
    p.n, p.ns, p.m, p.z, p.r, p.rz = _dims(model)
    p.gamma = model["gamma"]
    p.horizon = model["horizon"]
    p.S, p.T, p.O, p.R, p.Z, p.B = _p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F), _p(Z, _I), _p(B, _F)
    return p


def ref_pbvi_solve(model, horizon=None):
    """Reference pomdp_pbvi_execute_cpu; returns (Gamma, pi)."""
    L = ref_lib()
    keep = []
    p = _ref_pomdp(model, keep)
    if horizon is not None:
        p.horizon = horizon
    G0 = np.ascontiguousarray(model["GammaInitial"], dtype=np.float32)
    alg = _RefPBVI()
    alg.GammaInitial = _p(G0, _F)
    pol = _RefAlpha()
    rc = L.pomdp_pbvi_execute_cpu(ct.byref(p), ct.byref(alg), ct.byref(pol))
    if rc != 0:
        raise RuntimeError("reference pomdp_pbvi_execute_cpu failed: %d" % rc)
    G = np.ctypeslib.as_array(pol.Gamma, shape=(pol.r * pol.n,)).reshape(pol.r, pol.n).copy()
    pi = np.ctypeslib.as_array(pol.pi, shape=(pol.r,)).copy().astype(np.uint32)
    L.pomdp_alpha_vectors_uninitialize(ct.byref(pol))
    return G, pi


def ref_perseus_solve(model, seed, horizon=None):
    """Reference pomdp_perseus_execute_cpu after srand(seed); returns (Gamma, pi)."""
    L = ref_lib()
    keep = []
    p = _ref_pomdp(model, keep)
    if horizon is not None:
        p.horizon = horizon
    G0 = np.ascontiguousarray(model["GammaInitial"], dtype=np.float32)
    alg = _RefPerseus()
    alg.GammaInitial = _p(G0, _F)
    pol = _RefAlpha()
    lib().oracle_srand(seed)  # same libc rand() state as the reference library
    rc = L.pomdp_perseus_execute_cpu(ct.byref(p), ct.byref(alg), ct.byref(pol))
    if rc != 0:
        raise RuntimeError("reference pomdp_perseus_execute_cpu failed: %d" % rc)
    G = np.ctypeslib.as_array(pol.Gamma, shape=(pol.r * pol.n,)).reshape(pol.r, pol.n).copy()
    pi = np.ctypeslib.as_array(pol.pi, shape=(pol.r,)).copy().astype(np.uint32)
    L.pomdp_alpha_vectors_uninitialize(ct.byref(pol))
    return G, pi


def ref_mdp_vi_solve(model, horizon=None, VInitial=None):
    """Reference mdp_vi_execute_cpu; returns (V, pi)."""
    L = ref_lib()
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    T = np.ascontiguousarray(model["T"], dtype=np.float32)
    R = np.ascontiguousarray(model["R"], dtype=np.float32)
    mdp = _RefMDP()
    mdp.n, mdp.ns, mdp.m = model["n"], model["ns"], model["m"]
    mdp.gamma = model["gamma"]
    mdp.horizon = model["horizon"] if horizon is None else horizon
    mdp.S, mdp.T, mdp.R = _p(S, _I), _p(T, _F), _p(R, _F)
    alg = _RefVI()
    V0 = None
    if VInitial is not None:
        V0 = np.ascontiguousarray(VInitial, dtype=np.float32)
        alg.VInitial = _p(V0, _F)
    pol = _RefVF()
    rc = L.mdp_vi_execute_cpu(ct.byref(mdp), ct.byref(alg), ct.byref(pol))
    if rc != 0:
        raise RuntimeError("reference mdp_vi_execute_cpu failed: %d" % rc)
    V = np.ctypeslib.as_array(pol.V, shape=(pol.n,)).copy()
    pi = np.ctypeslib.as_array(pol.pi, shape=(pol.n,)).copy().astype(np.uint32)
    L.mdp_value_function_uninitialize(ct.byref(pol))
    return V, pi


def ref_alpha_value(Gamma, pi, b):
    """Reference pomdp_alpha_vectors_value_and_action; returns (V, action)."""
    L = ref_lib()
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    p = np.ascontiguousarray(pi, dtype=np.uint32)
    bb = np.ascontiguousarray(b, dtype=np.float32)
    pol = _RefAlpha()
    pol.n, pol.m, pol.r = G.shape[1], int(p.max()) + 1, G.shape[0]
    pol.Gamma, pol.pi = _p(G, _F), _p(p, _U)
    V = ct.c_float(0)
    a = ct.c_uint(0)
    rc = L.pomdp_alpha_vectors_value_and_action(ct.byref(pol), _p(bb, _F), ct.byref(V), ct.byref(a))
    if rc != 0:
        raise RuntimeError("reference value_and_action failed: %d" % rc)
    return V.value, a.value


# ---------------------------------------------------------------------------
# PBVI with recorded selections (FP64): reference for the GPU adjoint
# ---------------------------------------------------------------------------

def pbvi_record(model, horizon, GammaInitial=None):
    """nova's PBVI (FP32, the factored restatement) for `horizon` backups,
    recording the selections: actions [H][r] (pi after each backup) and
    selects [H][r][z] (the alpha chosen per observation under that action).
    Returns (Gamma_H float32 [r,n], actions, selects)."""
    n, ns, m, z, r, rz = _dims(model)
    G = np.ascontiguousarray(model["GammaInitial"] if GammaInitial is None else GammaInitial, dtype=np.float32)
    acts = np.zeros((horizon, r), np.uint32)
    sels = np.zeros((horizon, r, z), np.uint32)
    for t in range(horizon):
        Gp = np.empty_like(G)
        pi = np.zeros(r, np.uint32)
        js = np.zeros((r, m, z), np.uint32)
        pbvi_update(model, G, Gp, pi, jstar=js)
        acts[t] = pi
        sels[t] = js[np.arange(r), pi]
        G = Gp
    return G, acts, sels


def _fixed_args(model, Gamma0, actions, selects, b, T=None, O=None, R=None):
    n, ns, m, z, r, rz = _dims(model)
    S = np.ascontiguousarray(model["S"], dtype=np.int32)
    T = np.ascontiguousarray(model["T"] if T is None else T, dtype=np.float64)
    O = np.ascontiguousarray(model["O"] if O is None else O, dtype=np.float64)
    R = np.ascontiguousarray(model["R"] if R is None else R, dtype=np.float64)
    G0 = np.ascontiguousarray(Gamma0, dtype=np.float64)
    A = np.ascontiguousarray(actions, dtype=np.uint32)
    Se = np.ascontiguousarray(selects, dtype=np.uint32)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    keep = (S, T, O, R, G0, A, Se, bb)
    args = [n, ns, m, z, r, float(model["gamma"]), _p(S, _I), _p(T, _D), _p(O, _D), _p(R, _D), _p(G0, _D),
            A.shape[0], _p(A, _U), _p(Se, _U), _p(bb, _D)]
    return args, keep


def pbvi_fixed_forward_f64(model, Gamma0, actions, selects, b, T=None, O=None, R=None, istar=None):
    """V(b) = max_i b . Gamma_H[i] in FP64 with the recorded selections
    (optionally with T, O, R replaced, and the final argmax fixed to row
    `istar`); returns (V, i*)."""
    n, ns, m, z, r, rz = _dims(model)
    args, keep = _fixed_args(model, Gamma0, actions, selects, b, T, O, R)
    H = args[11]
    GammaAll = np.empty((H + 1) * r * n, np.float64)
    istar = ct.c_uint(0xFFFFFFFF if istar is None else int(istar))
    V = lib().oracle_pbvi_fixed_forward_f64(*args, ct.byref(istar), _p(GammaAll, _D))
    _ = keep
    return V, istar.value


def pbvi_fixed_reverse_f64(model, Gamma0, actions, selects, b, istar=None):
    """FP64 reverse mode (direct form) of the recorded backups (final argmax
    fixed to row `istar` when given); returns
    (V, dR [n,m], dT [n,m,ns], dO [m,n,z], dGamma0 [r,n])."""
    n, ns, m, z, r, rz = _dims(model)
    args, keep = _fixed_args(model, Gamma0, actions, selects, b)
    dR = np.zeros((n, m)); dT = np.zeros((n, m, ns)); dO = np.zeros((m, n, z)); dG = np.zeros((r, n))
    V = lib().oracle_pbvi_fixed_reverse_f64(*args, 0xFFFFFFFF if istar is None else int(istar), _p(dR, _D),
                                            _p(dT, _D), _p(dO, _D), _p(dG, _D))
    _ = keep
    return V, dR, dT, dO, dG


# ---------------------------------------------------------------------------
# Belief expansion and sigma approximation
# ---------------------------------------------------------------------------

def _exp_lib():
    L = lib()
    if not getattr(L, "_exp_bound", False):
        L.oracle_belief_update.argtypes = [ct.c_uint] * 4 + [_I, _F, _F, _F, ct.c_uint, ct.c_uint, _F]
        L.oracle_belief_update.restype = ct.c_int
        L.oracle_expand_random.argtypes = [ct.c_uint] * 7 + [_I, _F, _F, _I, _F, ct.c_uint, ct.c_uint, _F]
        L.oracle_expand_random_from_b0.argtypes = [ct.c_uint] * 6 + [_I, _F, _F, _I, _F, ct.c_uint, ct.c_uint, _F]
        L.oracle_expand_random_from_b0.restype = ct.c_uint
        L.oracle_expand_distinct.argtypes = [ct.c_uint] * 6 + [_I, _F, _F, _I, _F, _F]
        L.oracle_expand_distinct_range.argtypes = [ct.c_uint] * 6 + [_I, _F, _F, _I, _F, ct.c_uint, ct.c_uint, _F]
        L.oracle_expand_pema.argtypes = [ct.c_uint] * 6 + [ct.c_float, _I, _F, _F, _F, _I, _F, ct.c_uint, _F, _F]
        L._exp_bound = True
    return L


def belief_update(model, b, a, o):
    """nova's belief update (FP32); returns (b', valid)."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    bb = np.ascontiguousarray(b, dtype=np.float32)
    bp = np.empty(n, np.float32)
    rc = L.oracle_belief_update(n, ns, m, z, _p(S, _I), _p(T, _F), _p(O, _F), _p(bb, _F), a, o, _p(bp, _F))
    return bp, rc == 0


def expand_random(model, num, seed):
    """pomdp_expand_random_cpu after srand(seed); returns Bnew [num, n]."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    out = np.empty((num, n), np.float32)
    L.oracle_expand_random(n, ns, m, z, r, rz, model["horizon"], _p(S, _I), _p(T, _F), _p(O, _F), _p(Z, _I),
                           _p(B, _F), num, seed, _p(out, _F))
    return out


def expand_random_from_b0(model, num, seed):
    """pomdp_expand_random_gpu after srand(seed); returns (Bnew [num, n], maxNonZeroValues)."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    out = np.empty((num, n), np.float32)
    nz = L.oracle_expand_random_from_b0(n, ns, m, z, rz, model["horizon"], _p(S, _I), _p(T, _F), _p(O, _F),
                                        _p(Z, _I), _p(B, _F), num, seed, _p(out, _F))
    return out, nz


def expand_distinct(model):
    """pomdp_expand_distinct_beliefs_cpu's new beliefs Bnew [r, n]."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    out = np.empty((r, n), np.float32)
    L.oracle_expand_distinct(n, ns, m, z, r, rz, _p(S, _I), _p(T, _F), _p(O, _F), _p(Z, _I), _p(B, _F),
                             _p(out, _F))
    return out


def expand_distinct_rows(model, i0, i1):
    """Rows [i0, i1) of pomdp_expand_distinct_beliefs_cpu's new beliefs (the
    unit the CPU baseline times)."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    out = np.zeros((r, n), np.float32)
    L.oracle_expand_distinct_range(n, ns, m, z, r, rz, _p(S, _I), _p(T, _F), _p(O, _F), _p(Z, _I), _p(B, _F),
                                   i0, i1, _p(out, _F))
    return out[i0:i1]


def expand_pema(model, Gamma):
    """pomdp_expand_pema_cpu's new belief [n] for the policy's Gamma [pr, n]."""
    L = _exp_lib()
    S, T, O, R, Z, B = _arrays(model)
    n, ns, m, z, r, rz = _dims(model)
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    out = np.empty(n, np.float32)
    L.oracle_expand_pema(n, ns, m, z, r, rz, model["gamma"], _p(S, _I), _p(T, _F), _p(O, _F), _p(R, _F),
                         _p(Z, _I), _p(B, _F), G.shape[0], _p(G, _F), _p(out, _F))
    return out


def merge_raw_beliefs(Z, B, Bnew):
    """pomdp_add_new_raw_beliefs_cpu (pomdp_model_cpu.cpp:157-227) on arrays:
    appends the positive entries of each row of Bnew; returns (Z, B)."""
    r, rz = Z.shape
    nz = [(row > 0.0).sum() for row in Bnew]
    rz2 = max([rz] + [int(v) for v in nz])
    Zf = np.full((r + len(Bnew), rz2), -1, np.int32)
    Bf = np.zeros((r + len(Bnew), rz2), np.float32)
    Zf[:r, :rz] = Z
    Bf[:r, :rz] = B
    for i, row in enumerate(Bnew):
        idx = np.nonzero(row > 0.0)[0]
        Zf[r + i, :len(idx)] = idx
        Bf[r + i, :len(idx)] = row[idx]
    return Zf, Bf


def _ref_bind_expand(L):
    if not getattr(L, "_exp_bound", False):
        P = ct.POINTER(_RefPOMDP)
        L.pomdp_initialize_cpu.argtypes = [P] + [ct.c_uint] * 6 + [ct.c_float, ct.c_uint]
        L.pomdp_uninitialize_cpu.argtypes = [P]
        L.pomdp_expand_random_cpu.argtypes = [P, ct.c_uint]
        L.pomdp_expand_distinct_beliefs_cpu.argtypes = [P]
        L.pomdp_expand_pema_cpu.argtypes = [P, ct.POINTER(_RefAlpha)]
        L.pomdp_sigma_cpu.argtypes = [P, ct.c_uint, ct.POINTER(ct.c_float)]
        L.pomdp_expand_random_gpu.argtypes = [P, ct.c_uint, ct.c_uint, ct.POINTER(ct.c_uint), ct.POINTER(_F)]
        L._exp_bound = True


def _ref_pomdp_owned(model):
    """A reference POMDP whose arrays the reference allocated (its expansion
    frees and reallocates Z and B)."""
    L = ref_lib()
    _ref_bind_expand(L)
    n, ns, m, z, r, rz = _dims(model)
    p = _RefPOMDP()
    if L.pomdp_initialize_cpu(ct.byref(p), n, ns, m, z, r, rz, model["gamma"], model["horizon"]) != 0:
        raise RuntimeError("reference pomdp_initialize_cpu failed")
    for name, arr, t in zip(("S", "T", "O", "R", "Z", "B"), _arrays(model), (_I, _F, _F, _F, _I, _F)):
        ct.memmove(getattr(p, name), arr.ctypes.data, arr.nbytes)
    return L, p


def _ref_beliefs(p):
    Z = np.ctypeslib.as_array(p.Z, shape=(p.r * p.rz,)).reshape(p.r, p.rz).copy()
    B = np.ctypeslib.as_array(p.B, shape=(p.r * p.rz,)).reshape(p.r, p.rz).copy()
    return Z, B


def ref_expand_distinct(model):
    L, p = _ref_pomdp_owned(model)
    if L.pomdp_expand_distinct_beliefs_cpu(ct.byref(p)) != 0:
        raise RuntimeError("reference distinct expansion failed")
    out = _ref_beliefs(p)
    L.pomdp_uninitialize_cpu(ct.byref(p))
    return out


def ref_expand_pema(model, Gamma, pi):
    L, p = _ref_pomdp_owned(model)
    G = np.ascontiguousarray(Gamma, dtype=np.float32)
    P = np.ascontiguousarray(pi, dtype=np.uint32)
    pol = _RefAlpha()
    pol.n, pol.m, pol.r = model["n"], model["m"], G.shape[0]
    pol.Gamma, pol.pi = _p(G, _F), _p(P, _U)
    if L.pomdp_expand_pema_cpu(ct.byref(p), ct.byref(pol)) != 0:
        raise RuntimeError("reference PEMA expansion failed")
    out = _ref_beliefs(p)
    L.pomdp_uninitialize_cpu(ct.byref(p))
    return out


def ref_sigma(model, k):
    L, p = _ref_pomdp_owned(model)
    sigma = ct.c_float(0.0)
    if L.pomdp_sigma_cpu(ct.byref(p), k, ct.byref(sigma)) != 0:
        raise RuntimeError("reference sigma approximation failed")
    out = _ref_beliefs(p)
    L.pomdp_uninitialize_cpu(ct.byref(p))
    return out + (sigma.value,)


def ref_expand_random(model, num, tries=20):
    """The reference's random expansion seeds with time(nullptr): a call that
    starts and ends within one clock second used that second as its seed.
    Returns (Z, B, seed)."""
    import time
    for _ in range(tries):
        L, p = _ref_pomdp_owned(model)
        t0 = int(time.time())
        rc = L.pomdp_expand_random_cpu(ct.byref(p), num)
        t1 = int(time.time())
        if rc != 0:
            raise RuntimeError("reference random expansion failed")
        out = _ref_beliefs(p)
        L.pomdp_uninitialize_cpu(ct.byref(p))
        if t0 == t1:
            return out + (t0,)
    raise RuntimeError("could not pin the reference's clock seed")


def ref_expand_random_from_b0(model, num, tries=20):
    """pomdp_expand_random_gpu of the reference (host code); returns (Bnew, maxNonZeroValues, seed)."""
    import time
    for _ in range(tries):
        L, p = _ref_pomdp_owned(model)
        nz = ct.c_uint(0)
        Bn = _F()
        t0 = int(time.time())
        rc = L.pomdp_expand_random_gpu(ct.byref(p), 32, num, ct.byref(nz), ct.byref(Bn))
        t1 = int(time.time())
        if rc != 0:
            raise RuntimeError("reference random expansion (b0 form) failed")
        out = np.ctypeslib.as_array(Bn, shape=(num * model["n"],)).reshape(num, model["n"]).copy()
        L.pomdp_uninitialize_cpu(ct.byref(p))
        if t0 == t1:
            return out, nz.value, t0
    raise RuntimeError("could not pin the reference's clock seed")


def sigma_approximate(model, k):
    """pomdp_sigma_cpu (pomdp_sigma_cpu.cpp:49-118) on arrays: each belief
    keeps its k largest values (equal values in support order), divided by
    their FP32 sum; returns (Z, B, sigma)."""
    Z, B = model["Z"], model["B"]
    r, rz = Z.shape
    Zn = np.full((r, k), -1, np.int32)
    Bn = np.zeros((r, k), np.float32)
    sigma = np.float32(1.0)
    for i in range(r):
        order = sorted(range(rz), key=lambda q: -float(B[i, q]))  # stable: ties keep support order
        sb = np.float32(0.0)
        for q in order[:k]:
            sb = np.float32(sb + B[i, q])
        if sb < sigma:
            sigma = sb
        for t, q in enumerate(order[:k]):
            if B[i, q] > 0.0:
                Bn[i, t] = np.float32(B[i, q] / sb)
                Zn[i, t] = Z[i, q]
    return Zn, Bn, float(sigma)
