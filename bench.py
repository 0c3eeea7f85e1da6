"""nova-gb300 benchmark: PBVI belief-backups/s on one GB300 per rank.

Workload (default `pbvi_n4096`): seeded random sparse POMDP with n=4096
states, m=16 actions, z=32 observations, ns=32 successors per (s, a),
r=8192 beliefs with rz=64 support states, gamma=0.95 (nova's PBVI update,
|Gamma| = r). A step is one PBVI backup of every belief
(pomdp_pbvi_update_gpu); the metric is beliefs backed up per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]

Our arm prints one JSON line with: value (device-resident, tensor-core
scoring), the plain FP32 exact-scoring form on the same state, e2e through
the host-buffer entry point pomdp_pbvi_update_cpu (host<->device copies
inside the timed region), the roofline of the scoring kernel, the CPU
baseline (the oracle's port of nova's CPU loop, timed on a bounded sample on
this host's cores), clocks sampled during the timed region, and the MDP
Bellman sweep on n=2^20. The reference arm (--impl reference) times nova's
CPU algorithm on this host's cores (the oracle port; nova's own CPU sources
are not present on the GPU host) on the same workload.

Multi-GPU: every rank runs an independent replica of the workload (PBVI
beliefs of one POMDP need the full alpha set each step, and the library has
no collective); value is the sum over ranks of beliefs backed up divided by
the maximum time over ranks.
"""
import argparse
import ctypes as ct
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PBVI belief-backups/s at n=4096: BF16-TC vs plain FP32, |ΔV(b0)|≤1e-4 vs FP64"
UNIT = "belief-backups/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="pbvi_n4096")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--table-free-steps", type=int, default=2,
                    help="FP16 updates timed without the projection table (NOVA_PBVI_TABLE_NEVER)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-mdp", action="store_true")
    ap.add_argument("--bf16-steps", type=int, default=2)
    ap.add_argument("--precision-steps", type=int, default=3)
    ap.add_argument("--precision-horizon", type=int, default=12)
    ap.add_argument("--parity-beliefs", type=int, default=16)
    ap.add_argument("--batch-horizon", type=int, default=100)
    ap.add_argument("--batch-threads", type=int, default=16)
    return ap.parse_args()


def workload(args):
    from nova_gb300 import synth
    cfg = dict(synth.POMDP_CONFIGS[args.config])
    return synth.random_pomdp(**cfg, seed=args.seed), cfg


def workload_name(cfg, args):
    return "%s (n=%d,m=%d,z=%d,ns=%d,r=%d,rz=%d,gamma=%g,seed=%d)" % (
        args.config, cfg["n"], cfg["m"], cfg["z"], cfg["ns"], cfg["r"], cfg["rz"], cfg["gamma"], args.seed)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_sample(model, Gamma, seconds, threads):
    """Time nova's loop-form backup (the oracle port) on (belief, action)
    pairs against the full alpha set, on `threads` host threads, for about
    `seconds`. Returns (belief-backups/s, pairs done, wall seconds)."""
    from oracle import oracle as orc
    run = orc.pbvi_belief_action_sampler(model, Gamma)
    m = model["m"]
    lock = threading.Lock()
    counter = [0]
    done = [0]
    deadline = [None]

    def worker():
        while True:
            with lock:
                k = counter[0]
                if deadline[0] is not None and time.perf_counter() > deadline[0]:
                    return
                counter[0] += 1
            i, a = (k // m) % model["r"], k % m
            run(i, a)
            with lock:
                done[0] += 1

    t0 = time.perf_counter()
    deadline[0] = t0 + seconds
    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    wall = time.perf_counter() - t0
    return done[0] / m / wall, done[0], wall


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.reader.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nme, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nme)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    """(HBM GB/s, dense BF16 TFLOP/s, source). The tensor peak is the sustained
    figure: the scoring GEMM is timed inside steps of a multi-second loop,
    under the power cap."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d.get("bf16_tflops_sustained", d["bf16_tflops"]), "measured (bf16 sustained)"
    except Exception:
        return 6800.0, 1700.0, "fallback (sustained)"


def gemm_traffic(units, split):
    """DRAM bytes per launch of the scoring GEMM: an ncu capture of a smaller
    launch of the same kernel (profiles/tc_score_gemm_traffic.json: its DRAM
    read and write bytes and its work units, one unit being one (a,o) pair x
    128-row tile x alpha group) scaled to `units` units, since each unit
    streams one A tile and writes one candidate set. None when no capture of
    this operand form is recorded."""
    try:
        with open(os.path.join(ROOT, "profiles", "tc_score_gemm_traffic.json")) as f:
            d = json.load(f)["bf16_split" if split else "fp16"]
        per_unit = (float(d["dram_bytes_read"]) + float(d["dram_bytes_write"])) / float(d["units"])
        return per_unit * units, ("DRAM bytes per launch: ncu capture of a %d-unit launch (%s) scaled to %d units"
                                  % (d["units"], d["workload"], units))
    except Exception:
        return None, "no ncu capture recorded for this operand form"


def sampled_parity(alg, model, k, seed, backup0):
    """One more (untimed) update on `alg` (whose alpha set is that after
    backup0 backups from GammaInitial plus alg's own updates), then its rows and actions for k
    sampled beliefs (those with rows sent to the exact scan, those with the
    most alphas re-scored, random ones) against nova's loop-form backup (the
    oracle, as the checker) over all actions and the full alpha set."""
    from oracle import oracle as orc
    pol = alg.get_policy()
    G = pol.gamma_array()
    del pol
    alg.update()
    st = alg.stats()
    cand, exact = alg.row_detail()
    pol = alg.get_policy()
    Gp, pi = pol.gamma_array(), pol.pi_array()
    del pol
    beliefs = orc.choose_parity_beliefs(cand, exact, k=k, seed=seed)
    t0 = time.perf_counter()
    bad = orc.sampled_backup_parity(model, G, Gp, pi, beliefs, threads=host_cores())
    return {"matched": "%d of %d" % (len(beliefs) - len(bad), len(beliefs)), "beliefs": beliefs,
            "mismatched": bad, "backup": backup0 + st["horizon"], "scoring": st["scoring"],
            "rows_exact_scan": st["rowsOverflow"], "candidates_rescored": st["candidates"],
            "max_candidates_one_belief": int(cand.max()), "oracle_seconds": time.perf_counter() - t0}


def run_reference(args, rank):
    if rank != 0:
        return
    model, cfg = workload(args)
    cores = host_cores()
    per_step = max(1.0, args.cpu_seconds / 3.0)
    for _ in range(args.warmup):
        cpu_sample(model, model["GammaInitial"], min(per_step, 2.0), cores)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, pairs, wall = cpu_sample(model, model["GammaInitial"], per_step, cores)
        vals.append((v, pairs, wall))
    total = time.perf_counter() - t0
    pairs = sum(p for _, p, _ in vals)
    value = pairs / model["m"] / sum(w for _, _, w in vals)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(cfg, args), "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "per step: (belief, action) pairs of nova's loop-form backup against the full "
                                   "alpha set (r=%d) for %.1f s on %d threads; %d pairs in total"
                                   % (cfg["r"], per_step, cores, pairs)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_precision(args):
    """|V(b0) - V_FP64(b0)| after H backups with the default (FP16 tensor-core)
    scoring. Two FP64 references from the oracle, on the same GammaInitial:
    `dV_b0` re-evaluates the GPU run's own selections (recorded actions,
    per-observation alphas and final argmax) in FP64, which isolates the
    arithmetic error; `dV_b0_free_fp64_run` is an independent FP64 PBVI run,
    whose own argmax choices can part from the FP32 ones at near-ties. Two
    workloads: pbvi_n64 over its full horizon, and the n=4096 shapes (m=16,
    z=32, ns=32, rz=64) with r=256 beliefs."""
    from nova_gb300 import synth
    from nova_gb300.pomdp_adjoint import pbvi_record_and_adjoint
    from oracle import oracle as orc
    out = {}
    for name, horizon in (("pbvi_n64", None), ("pbvi_n4096_r256", args.precision_steps)):
        cfg = dict(synth.POMDP_CONFIGS[name])
        model = synth.random_pomdp(**cfg, seed=args.seed)
        H = cfg["horizon"] if horizon is None else horizon
        b0 = synth.dense_belief(model, 0)
        Vg, istar, _, _, _, _, acts, sels = pbvi_record_and_adjoint(model, b0, H, 10)
        t0 = time.perf_counter()
        Vfix, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar)
        G = model["GammaInitial"].astype(np.float64)
        for _ in range(H):
            G, _ = orc.pbvi_update_f64(model, G)
        Vfree = float(np.max(G @ b0.astype(np.float64)))
        out[name] = {"horizon": H, "r": cfg["r"], "V_b0": Vg, "V_b0_fp64_same_selections": Vfix,
                     "dV_b0": abs(Vg - Vfix), "V_b0_free_fp64_run": Vfree, "dV_b0_free_fp64_run": abs(Vg - Vfree),
                     "oracle_seconds": time.perf_counter() - t0}
    out["max_dV_b0"] = max(v["dV_b0"] for v in out.values())
    out["note"] = ("tensor-core alphas are bit-identical to the plain FP32 path's; dV_b0 is their FP32 rounding "
                   "against FP64 on the same selections, dV_b0_free_fp64_run the gap to an FP64 solve that made "
                   "different argmax choices at near-ties")
    return out


def run_precision_headline(args, model, pomdp):
    """|V(b0) - V_FP64(b0)| on the full pbvi_n4096 workload (r=8192): H
    backups from GammaInitial with the library's default (FP16 tensor-core)
    scoring, their selections recorded, then the same H backups recomputed
    in FP64 on the GPU with those selections held fixed
    (pomdp_pbvi_value_replay_f64_gpu); b0 = belief 0. The difference is the
    arithmetic error of the FP32 backups (the tensor-core alphas equal the
    plain FP32 path's bit for bit)."""
    from nova_gb300 import synth
    from nova_gb300.pomdp_adjoint import pbvi_value_vs_fp64
    H = args.precision_horizon
    b0 = synth.dense_belief(model, 0)
    t0 = time.perf_counter()
    V, V64, istar, _, _ = pbvi_value_vs_fp64(model, b0, H, pomdp=pomdp)
    return {"horizon": H, "r": model["r"], "n": model["n"], "V_b0": V, "V_b0_fp64_same_selections": V64,
            "dV_b0": abs(V - V64), "alpha": istar, "seconds": time.perf_counter() - t0,
            "fp64": "GPU FP64 replay of the recorded selections (checked against the oracle's FP64 forward on "
                    "small models in the tests)"}


def run_margins(args):
    """Candidates within proven margins at n=4096 (pbvi_n4096, seed 0): after
    --warmup FP16 backups, for 2048 random (belief, action, observation) rows,
    the exact scores (FP64, from a dense A row and the distinct alphas) of all
    alphas, and how many lie within 2E of the best for the error bound E of
    each operand form: E = a1 (U gmax + gN Gmax) with U the sum of both
    operands' unit roundoffs (FP16 2^-11, BF16 2^-8, E4M3 2^-4), the FP32
    build of A and the accumulation; the split forms carry one operand as a
    hi + lo pair (2^-16). Worst-case operand rounding is used for both
    operands here (the library bounds A's rounding by its measured value,
    which is tighter). This is the design input for the operand precision
    of the scoring GEMM."""
    import torch
    from nova_gb300 import synth
    from nova_gb300 import nova_pomdp_pbvi as npp
    from nova_gb300.pomdp import POMDP
    from nova_gb300.pomdp_pbvi import POMDPPBVIGPU
    cfg = dict(synth.POMDP_CONFIGS["pbvi_n4096"])
    model = synth.random_pomdp(**cfg, seed=args.seed)
    n, m, z, ns, r, rz = (cfg[k] for k in ("n", "m", "z", "ns", "r", "rz"))
    p = POMDP.from_arrays(model)
    p.initialize_gpu()
    alg = POMDPPBVIGPU(p, GammaInitial=model["GammaInitial"])
    alg.set_scoring(npp.SCORING_FP16)
    for _ in range(args.warmup):
        alg.update()
    pol = alg.get_policy()
    G = pol.gamma_array()
    del pol
    del alg
    dev = "cuda"
    S = torch.tensor(model["S"].astype(np.int64), device=dev)
    T = torch.tensor(model["T"].astype(np.float64), device=dev)
    O = torch.tensor(model["O"].astype(np.float64), device=dev)
    rng = np.random.default_rng(args.seed + 1)
    NS = 2048
    ri, ra, ro = rng.integers(0, r, NS), rng.integers(0, m, NS), rng.integers(0, z, NS)
    A = torch.zeros((NS, n), dtype=torch.float64, device=dev)
    for t in range(NS):
        i, a, o = int(ri[t]), int(ra[t]), int(ro[t])
        sk = torch.tensor(model["Z"][i].astype(np.int64), device=dev)
        w = torch.tensor(model["B"][i].astype(np.float64), device=dev)[:, None] * T[sk, a, :]
        W = torch.zeros(n, dtype=torch.float64, device=dev)
        W.index_add_(0, S[sk, a, :].reshape(-1), w.reshape(-1))
        A[t] = float(np.float32(cfg["gamma"])) * W * O[a, :, o]
    Gu = torch.tensor(np.unique(G, axis=0).astype(np.float64), device=dev)
    h = 0.5 * (Gu.max(0).values - Gu.min(0).values)
    gmax, Gmax = float(h.max()), float(Gu.abs().max())
    sc = A @ Gu.T
    best = sc.max(1).values
    a1 = A.abs().sum(1)
    u24 = 2.0 ** -24
    epsA = (rz * ns + 4) * u24
    gN = (ns + rz + 3) * u24 * 1.01

    def bound(uA, uG, ksplit=1):
        acc = (ksplit * n / 16 + 2) / 4194304.0
        return a1 * ((epsA + (1 + uA) * (uG + 2 * u24) + uA + acc) * gmax + gN * Gmax)
    forms = {"fp16": bound(2 ** -11, 2 ** -11), "bf16": bound(2 ** -8, 2 ** -8),
             "bf16_alphas_split": bound(2 ** -8, 2 ** -16, 2), "bf16_both_split": bound(2 ** -16, 2 ** -16, 3),
             "e4m3": bound(2 ** -4, 2 ** -4), "reference_rounding_only": a1 * gN * Gmax}
    out = {"workload": "pbvi_n4096 (seed %d) after %d FP16 backups; %d sampled rows" % (args.seed, args.warmup, NS),
           "distinct_alphas": int(Gu.shape[0]), "gmax": gmax, "Gmax": Gmax}
    for name, E in forms.items():
        cnt = (sc >= (best - 2 * E)[:, None]).sum(1).cpu().numpy()
        out[name] = {"mean": float(cnt.mean()), "p50": float(np.percentile(cnt, 50)),
                     "p90": float(np.percentile(cnt, 90)), "p99": float(np.percentile(cnt, 99)),
                     "max": int(cnt.max()), "rows_over_128": float((cnt > 128).mean()),
                     "E_over_a1_gmax_median": float(torch.median(E / (a1 * gmax)))}
    return out


def run_gradient(args):
    """Gradient of V(b0) after H=50 PBVI backups w.r.t. R, T, O (n=1024, m=8,
    z=16, ns=16, r=2048, rz=32, b0 uniform, checkpoints every 10 steps):
    GPU time of the recorded forward and of the reverse pass, and the
    gradient's error against the oracle's FP64 reverse mode and against FP64
    central differences (h=1e-6) on 64 random coordinates."""
    import torch
    from nova_gb300 import synth
    from nova_gb300.pomdp_adjoint import PBVIGradSpec, pbvi_value, pbvi_record_and_adjoint
    from oracle import oracle as orc
    cfg = dict(synth.POMDP_CONFIGS["grad_n1024"])
    model = synth.random_pomdp(**cfg, seed=args.seed)
    H = cfg["horizon"]
    b0 = np.full(model["n"], 1.0 / model["n"], np.float32)
    spec = PBVIGradSpec(model=model, b0=b0, horizon=H, checkpoint_every=10)
    times = []
    for it in range(args.warmup + args.steps):
        R = torch.tensor(model["R"], device="cuda", requires_grad=True)
        T = torch.tensor(model["T"], device="cuda", requires_grad=True)
        O = torch.tensor(model["O"], device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        V = pbvi_value(R, T, O, spec)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        V.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if it >= args.warmup:
            times.append((t1 - t0, t2 - t1))
    fwd = float(np.median([a for a, _ in times]))
    bwd = float(np.median([b for _, b in times]))
    Vg, istar, dR, dT, dO, dG, acts, sels = pbvi_record_and_adjoint(model, b0, H, 10)
    t0 = time.perf_counter()
    V64, dR64, dT64, dO64, _ = orc.pbvi_fixed_reverse_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar)
    t_rev = time.perf_counter() - t0

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(1e-30, np.max(np.abs(b))))
    rng = np.random.default_rng(args.seed + 1)
    grads = {"R": dR, "T": dT, "O": dO}
    worst, h = 0.0, 1e-6
    t0 = time.perf_counter()
    for k in range(64):
        name = ("R", "T", "O")[k % 3]
        idx = tuple(int(rng.integers(0, d)) for d in model[name].shape)
        A = model[name].astype(np.float64).copy()
        A[idx] += h
        Vp, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar, **{name: A})
        A[idx] -= 2 * h
        Vm, _ = orc.pbvi_fixed_forward_f64(model, model["GammaInitial"], acts, sels, b0, istar=istar, **{name: A})
        fd = (Vp - Vm) / (2 * h)
        worst = max(worst, abs(grads[name][idx] - fd) / max(abs(fd), 1e-3))
    t_fd = time.perf_counter() - t0
    return {"metric": "gradients of V(b0) per second (H=50 PBVI backups, forward + reverse)",
            "value": 1.0 / (fwd + bwd), "unit": "gradients/s", "steps": args.steps, "warmup": args.warmup,
            "forward_s": fwd, "reverse_s": bwd, "higher_is_better": True,
            "config": {"workload": "grad_n1024 (n=1024,m=8,z=16,ns=16,r=2048,rz=32,gamma=0.95,H=50,b0 uniform,"
                                   "checkpoint every 10,seed=%d)" % args.seed},
            "V_b0": Vg, "V_b0_fp64_same_selections": V64, "dV_b0": abs(Vg - V64),
            "rel_err_vs_fp64_reverse": {"R": rel(dR, dR64), "T": rel(dT, dT64), "O": rel(dO, dO64)},
            "fd_max_rel_err_64_coords": worst, "fd_step": h,
            "oracle_reverse_seconds": t_rev, "fd_seconds": t_fd, "host_cores": host_cores()}


def run_batch(args):
    """256 independent random POMDPs (n, r log-uniform in [32, 2048] and
    [128, 4096], m in 2..16, z in 2..32, ns = min(16, n), rz = min(32, n),
    gamma 0.95) for --batch-horizon backups each: belief-backups/s summed over
    the batch for the batched solve (host-thread pool, per-thread streams) with
    FP16 and BF16 tensor-core scoring, against solving them one after another
    with plain FP32 scoring; every batched policy is checked bit for bit
    against the sequential plain one."""
    import torch
    from nova_gb300 import synth
    from nova_gb300 import nova_pomdp_pbvi as npp
    from nova_gb300.pomdp import POMDP
    from nova_gb300.pomdp_pbvi import solve_batched
    H = args.batch_horizon
    t0 = time.perf_counter()
    models = synth.batch_pomdps(256, seed=args.seed, horizon=H)
    gen_s = time.perf_counter() - t0
    pomdps = []
    for md in models:
        p = POMDP.from_arrays(md)
        p.initialize_gpu()
        pomdps.append(p)
    total = float(sum(md["r"] for md in models) * H)

    def timed(mode, threads, horizon=H, graph=False, persistent=False):
        for p in pomdps:
            p.horizon = horizon
        torch.cuda.synchronize()
        t = time.perf_counter()
        pols = solve_batched(pomdps, scoring=mode, hostThreads=threads, graph=graph, persistent=persistent)
        torch.cuda.synchronize()
        return time.perf_counter() - t, [(p.gamma_array(), p.pi_array()) for p in pols]

    timed(npp.SCORING_FP16, args.batch_threads, horizon=1)  # warm-up: builds and first launches
    t_per16, g_per16 = timed(npp.SCORING_FP16, args.batch_threads, persistent=True)
    t_fp16, g16 = timed(npp.SCORING_FP16, args.batch_threads)
    t_graph, g_gr = timed(npp.SCORING_FP16, args.batch_threads, graph=True)
    t_perbf, g_perbf = timed(npp.SCORING_BF16, args.batch_threads, persistent=True)
    t_bf16, g_bf = timed(npp.SCORING_BF16, args.batch_threads)
    t_plain, g_plain = timed(npp.SCORING_EXACT, 1)
    identical = 0
    for k, (G, pi) in enumerate(g_plain):
        identical += int(all(np.array_equal(g[k][0].view(np.uint32), G.view(np.uint32)) and
                             np.array_equal(g[k][1], pi) for g in (g_per16, g16, g_gr, g_perbf, g_bf)))
    return {"metric": "belief-backups/s summed over a batch of 256 random POMDPs", "unit": "belief-backups/s",
            "value": total / t_per16, "horizon": H, "host_threads": args.batch_threads,
            "fp16_persistent": {"value": total / t_per16, "seconds": t_per16,
                                "note": "lock-step backups after a tuning warm-up; one persistent tcgen05 launch "
                                        "per backup scores the work units of every tensor-core solver from a "
                                        "device work table (pomdp_pbvi_execute_batched_persistent_gpu)"},
            "bf16_persistent": {"value": total / t_perbf, "seconds": t_perbf},
            "fp16_thread_pool": {"value": total / t_fp16, "seconds": t_fp16,
                                 "note": "one ordinary solve per POMDP on a pool of host threads"},
            "bf16_thread_pool": {"value": total / t_bf16, "seconds": t_bf16},
            "fp16_thread_pool_graph": {"value": total / t_graph, "seconds": t_graph,
                                       "note": "horizon loops replayed as CUDA graphs after schedule tuning"},
            "plain_fp32_one_by_one": {"value": total / t_plain, "seconds": t_plain},
            "policies_bit_identical": "%d of 256 (every form against the one-by-one plain FP32 solves)" % identical,
            "belief_backups": total, "generation_s": gen_s,
            "config": {"workload": "batch256 (n~logU[32,2048], r~logU[128,4096], m~U{2..16}, z~U{2..32}, "
                                   "ns=min(16,n), rz=min(32,n), gamma=0.95, H=%d, seed=%d)" % (H, args.seed)}}


def run_expand(args):
    """Belief-set expansion on n=512, m=8, z=16, ns=16, r=1024, rz=32:
    pomdp_expand_distinct_beliefs_cpu (1024 new beliefs; about m*z*r*n =
    6.7e7 L1 terms per belief) and pomdp_expand_random_cpu (2048 beliefs from
    seeded random trajectories), timed on the GPU through the C API with host
    arrays; beside them nova's CPU algorithm (the oracle port) on a bounded
    sample of beliefs on one host thread; the GPU rows are checked bit for bit
    against the sampled oracle rows."""
    import torch
    from nova_gb300 import synth
    from nova_gb300 import nova_pomdp as npm
    from nova_gb300.pomdp import POMDP
    from oracle import oracle as orc
    cfg = dict(synth.POMDP_CONFIGS["expand_n512"])
    model = synth.random_pomdp(**cfg, seed=args.seed)
    n, r = cfg["n"], cfg["r"]

    def distinct_once():
        p = POMDP.from_arrays(model)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.expand(method="distinct_beliefs")
        torch.cuda.synchronize()
        return time.perf_counter() - t0, p.arrays()

    distinct_once()
    times, out = [], None
    for _ in range(max(1, args.steps)):
        t, out = distinct_once()
        times.append(t)
    t_gpu = float(np.median(times))
    sample = 16
    t0 = time.perf_counter()
    rows = orc.expand_distinct_rows(model, 0, sample)
    t_cpu = time.perf_counter() - t0
    ok = 0
    for i in range(sample):
        dense = np.zeros(n, np.float32)
        for zz, bb in zip(out["Z"][r + i], out["B"][r + i]):
            if zz >= 0:
                dense[zz] = bb
        ok += int(np.array_equal(dense.view(np.uint32), np.where(rows[i] > 0, rows[i], 0).astype(np.float32)
                                 .view(np.uint32)))
    npm._nova.nova_gb300_expand_seed(1, 77)
    p = POMDP.from_arrays(model)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p.expand(method="random", numBeliefsToAdd=2048)
    torch.cuda.synchronize()
    t_rand = time.perf_counter() - t0
    t0 = time.perf_counter()
    orc.expand_random(model, 512, 77)
    t_rand_cpu = time.perf_counter() - t0
    npm._nova.nova_gb300_expand_seed(0, 0)
    return {"workload": "expand_n512 (n=512,m=8,z=16,ns=16,r=1024,rz=32,seed=%d)" % args.seed,
            "distinct": {"beliefs_per_s": r / t_gpu, "seconds": t_gpu,
                         "cpu_baseline": {"beliefs_per_s": sample / t_cpu, "cores": 1, "kind": "port",
                                          "sample": "%d beliefs of the distinct expansion" % sample},
                         "rows_bit_identical_to_oracle": "%d of %d sampled" % (ok, sample)},
            "random": {"beliefs_per_s": 2048 / t_rand, "seconds": t_rand,
                       "cpu_baseline": {"beliefs_per_s": 512 / t_rand_cpu, "cores": 1, "kind": "port",
                                        "sample": "512 beliefs of a seeded random expansion"}}}


def run_value(args):
    """V(b) and the action for the r=8192 beliefs of the n=4096 workload (dense)
    over an 8192 x 4096 alpha set: pomdp_alpha_vectors_value_batched_gpu with
    device-resident inputs, the host-array entry point end to end, and nova's
    one-belief evaluation (oracle port) on a sample of beliefs on one thread;
    the sampled results are checked bit for bit."""
    import torch
    from nova_gb300 import synth
    from nova_gb300 import nova_pomdp_alpha_vectors as npav
    from nova_gb300.pomdp_alpha_vectors import POMDPAlphaVectors
    from oracle import oracle as orc
    cfg = dict(synth.POMDP_CONFIGS["pbvi_n4096"])
    model = synth.random_pomdp(**cfg, seed=args.seed)
    n, r = cfg["n"], cfg["r"]
    rng = np.random.default_rng(args.seed + 5)
    G = rng.uniform(-20.0, 20.0, size=(r, n)).astype(np.float32)
    pi = rng.integers(0, cfg["m"], size=r).astype(np.uint32)
    B = np.zeros((r, n), np.float32)
    for i in range(r):
        B[i, model["Z"][i]] = model["B"][i]
    dG, dPi, dB = (torch.as_tensor(x, device="cuda") for x in (G, pi.astype(np.int32), B))
    dV = torch.empty(r, dtype=torch.float32, device="cuda")
    dA = torch.empty(r, dtype=torch.int32, device="cuda")
    f = npav._nova.pomdp_alpha_vectors_value_batched_gpu

    def once():
        rc = f(dG.data_ptr(), dPi.data_ptr(), r, n, dB.data_ptr(), r, dV.data_ptr(), dA.data_ptr())
        if rc != 0:
            raise RuntimeError("pomdp_alpha_vectors_value_batched_gpu failed: %d" % rc)

    for _ in range(args.warmup):
        once()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        once()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    pol = POMDPAlphaVectors()
    assert npav._nova.pomdp_alpha_vectors_initialize(pol, n, cfg["m"], r) == 0
    import ctypes as ct
    ct.memmove(pol.Gamma, G.ctypes.data, G.nbytes)
    ct.memmove(pol.pi, pi.ctypes.data, pi.nbytes)
    t0 = time.perf_counter()
    V, a = pol.value_and_action_batched(B)
    t_e2e = time.perf_counter() - t0
    sample = 32
    t0 = time.perf_counter()
    ref = [orc.alpha_value(G, pi, B[i]) for i in range(sample)]
    t_cpu = time.perf_counter() - t0
    ok = sum(int(np.float32(V[i]).view(np.uint32) == np.float32(ref[i][0]).view(np.uint32) and a[i] == ref[i][1])
             for i in range(sample))
    _, tc_peak, _ = measured_peaks()
    flops = 2.0 * r * r * n
    return {"workload": "value_n4096 (8192 dense beliefs x 8192 alphas x n=4096, seed=%d)" % args.seed,
            "beliefs_per_s": r / (ms * 1e-3), "ms": ms, "fp32_tflops": flops / (ms * 1e-3) / 1e12,
            "e2e": {"beliefs_per_s": r / t_e2e, "seconds": t_e2e,
                    "api": "pomdp_alpha_vectors_value_and_action_batched (host arrays, wall clock)"},
            "cpu_baseline": {"beliefs_per_s": sample / t_cpu, "cores": 1, "kind": "port",
                             "sample": "%d beliefs of nova's value_and_action" % sample},
            "bit_identical": "%d of %d sampled" % (ok, sample)}


def run_mdp(args, dist_rank):
    """Bellman sweep n=2^20, m=8, ns=16 (memory-bound): GB/s of algorithmic bytes.
    Sweeps are timed through mdp_vi_execute_gpu (sweeps queued back to back):
    the time of a 201-sweep solve minus that of a 1-sweep solve, over 200."""
    import torch
    from nova_gb300 import synth
    from nova_gb300.mdp import MDP
    from nova_gb300.mdp_vi import MDPValueIterationGPU
    from nova_gb300 import nova_mdp_vi as nmvi
    from nova_gb300 import mdp_value_function as mvf
    cfg = synth.MDP_CONFIGS["vi_n1m"]
    md = synth.random_mdp(n=cfg["n"], m=cfg["m"], ns=cfg["ns"], gamma=cfg["gamma"], horizon=cfg["horizon"],
                          seed=args.seed)
    m = MDP.from_arrays(md)
    m.initialize_gpu()
    f = nmvi._nova

    def solve(h):
        m.horizon = h
        vi = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32))
        pol = mvf.MDPValueFunction()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = f.mdp_vi_execute_gpu(vi.mdpPtr, vi, pol)
        e1.record()
        torch.cuda.synchronize()
        if rc != 0:
            raise RuntimeError("mdp_vi_execute_gpu failed: %d" % rc)
        return e0.elapsed_time(e1)

    from nova_gb300 import mdp_vi as mvi
    mvi.set_tiling(nmvi.TILING_NEVER)
    solve(20)
    gather_ms = (solve(201) - solve(1)) / 200.0
    mvi.set_tiling(nmvi.TILING_AUTO)
    solve(20)
    kernel = {1: "tiled (shared-memory V tiles)", 2: "per-row gather"}.get(mvi.tiling_status(), "unknown")
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        t1 = solve(1)
        t201 = solve(201)
    ms = (t201 - t1) / 200.0
    n, mm, ns = md["n"], md["m"], md["ns"]
    alg_bytes = 2 * n * mm * ns * 4 + n * mm * 4 + 3 * n * 4
    hbm, _, _ = measured_peaks()
    gbs = alg_bytes / (ms * 1e-3) / 1e9
    m.horizon = cfg["horizon"]
    pol, nsweeps, resid = MDPValueIterationGPU(m, Vinitial=np.zeros(md["n"], np.float32)).solve_until_converged(
        tol=1e-6, maxSweeps=cfg["horizon"])
    return {"workload": "vi_n1m (n=2^20,m=8,ns=16,gamma=0.99)", "ms_per_sweep": ms, "GB_per_s": gbs,
            "sweep_kernel": kernel, "gather_ms_per_sweep": gather_ms,
            "algorithmic_bytes_per_sweep": alg_bytes, "frac_of_hbm": gbs / hbm, "clocks": clocks.summary(),
            "converged_sweeps": nsweeps, "final_residual_fp64": resid, "converged": bool(resid < 1e-6),
            "note": "FP32 values near 78 have a 7.6e-6 ulp; the FP64 residual of the FP32 iteration stalls above 1e-6"}


def replica_throughput(dist, world, units_per_rank, ms_local, device):
    """Whole-job throughput of `world` independent replicas that each process
    units_per_rank units: the job takes as long as its slowest rank (an
    all-reduce MAX of the per-rank milliseconds), and the units of all ranks
    count. Returns (units per second, job milliseconds)."""
    ms = float(ms_local)
    if dist is not None:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return world * units_per_rank / (ms * 1e-3), ms


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.config == "value_n4096":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"value": run_value(args)}))
        return
    if args.config == "expand_n512":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"expand": run_expand(args)}))
        return
    if args.config == "batch256":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"batch": run_batch(args)}))
        return
    if args.config == "margins_n4096":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"margins": run_margins(args)}))
        return
    if args.config == "grad_n1024":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"gradient": run_gradient(args)}))
        return
    if args.config == "vi_n1m":
        import torch
        torch.cuda.set_device(local_rank)
        if rank == 0:
            print(json.dumps({"mdp_vi": run_mdp(args, rank)}))
        return

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from nova_gb300 import nova_pomdp_pbvi as npp
    from nova_gb300.pomdp import POMDP
    from nova_gb300.pomdp_pbvi import POMDPPBVIGPU, POMDPPBVICPU
    lib = npp._nova

    model, cfg = workload(args)
    p = POMDP.from_arrays(model)
    p.initialize_gpu()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    alg = POMDPPBVIGPU(p, GammaInitial=model["GammaInitial"])
    alg.set_scoring(npp.SCORING_FP16)  # the library's default tensor-core mode

    for _ in range(args.warmup):
        alg.update()
    torch.cuda.synchronize()
    # Device memory the solver holds (scoring operand, projection table,
    # candidate lists, alpha sets), beside the model's own arrays.
    solver_bytes = free_before - torch.cuda.mem_get_info()[0]

    # ---- timed region: K backups, device-resident inputs --------------------
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    launches0 = lib.nova_gb300_kernel_launches()
    with ClockSampler(local_rank) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            alg.update()
            stats.append(alg.stats())
        e1.record()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    launches = lib.nova_gb300_kernel_launches() - launches0
    r = cfg["r"]
    value, ms = replica_throughput(dist, world, r * args.steps, e0.elapsed_time(e1), "cuda")

    # ---- roofline of the scoring kernel --------------------------------------
    hbm, tc_peak, peak_kind = measured_peaks()
    n_pad = ((cfg["n"] + 63) // 64) * 64
    gemm = [(s["uniqueAlphas"], s["msGemm"]) for s in stats if s["msGemm"] > 0]
    if gemm:
        flops = [2.0 * r * u * n_pad * cfg["m"] * cfg["z"] for u, _ in gemm]
        achieved = sum(flops) / (sum(t for _, t in gemm) * 1e-3) / 1e12
        groups = [s["tcGroups"] for s in stats if s["msGemm"] > 0][-1]
        units = cfg["m"] * cfg["z"] * ((r + 127) // 128) * max(1, groups)
        traffic, traffic_note = gemm_traffic(units, split=False)
        roofline = {"bound": "tensor", "achieved": achieved, "peak": tc_peak, "unit": "TFLOP/s",
                    "frac": achieved / tc_peak, "traffic": traffic, "traffic_note": traffic_note,
                    "kernel": "tcgen05 FP16 scoring GEMM (kind::f16, FP32 accumulate in TMEM) with fused candidate-list epilogue",
                    "flops_per_launch": flops[-1], "peak_source": peak_kind}
    else:
        roofline = {"bound": "tensor", "achieved": None, "peak": tc_peak, "unit": "TFLOP/s", "frac": None,
                    "traffic": None, "kernel": "tensor-core scoring did not run (exact scoring only)",
                    "peak_source": peak_kind}

    # ---- e2e through the host-buffer entry point ----------------------------
    # Measured right after the device-resident steps, under the same clocks;
    # the BF16 and plain legs below run afterwards on a new device solver.
    pol = alg.get_policy()
    Gnow = pol.gamma_array()
    del pol
    del alg  # frees the device solver (its operands and projection table)
    torch.cuda.synchronize()
    e2e = None
    if args.e2e_steps > 0:
        host = POMDPPBVICPU(p, GammaInitial=Gnow)
        host.update()  # uploads the model and builds the tables; not timed
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        marks = []
        for _ in range(args.e2e_steps):
            host.update()
            marks.append(time.perf_counter())
        wall = time.perf_counter() - t0
        step_ms = [round((b - a) * 1e3, 1) for a, b in zip([t0] + marks[:-1], marks)]
        rn4 = cfg["r"] * cfg["n"] * 4
        # Each call uploads the input set and pi and reads back the output set
        # and pi; the host output set is uploaded too only when some belief
        # keeps its row (no action above the -1e10 sentinel), never here.
        e2e = {"value": r * args.e2e_steps / wall, "unit": UNIT, "h2d_bytes_per_step": rn4 + 4 * cfg["r"],
               "d2h_bytes_per_step": rn4 + 4 * cfg["r"],
               "step_ms": step_ms, "api": "pomdp_pbvi_update_cpu (host Gamma/GammaPrime/pi; wall clock)"}
        del host

    # ---- a device solver for the parity check and the BF16 and plain legs ---
    parity = {}
    second = args.bf16_steps > 0 or args.plain_steps > 0 or args.parity_beliefs > 0 or args.table_free_steps > 0
    if second:
        free_before2 = torch.cuda.mem_get_info()[0]
        alg = POMDPPBVIGPU(p, GammaInitial=Gnow)
        alg.set_scoring(npp.SCORING_FP16)
        alg.update()  # builds the operands and tables; not timed
        torch.cuda.synchronize()
        if rank == 0 and args.parity_beliefs > 0:
            parity["fp16"] = sampled_parity(alg, model, args.parity_beliefs, seed=1,
                                            backup0=args.warmup + args.steps)

    # ---- BF16 tensor-core scoring on the same state ----------------------------
    bf16 = None
    if args.bf16_steps > 0:
        alg.set_scoring(npp.SCORING_BF16)
        alg.update()  # rebuilds the scoring operand in BF16; not timed
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fst = []
        f0.record()
        for _ in range(args.bf16_steps):
            alg.update()
            fst.append(alg.stats())
        f1.record()
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1)
        fl = fst[-1]
        fgemm = [(s["uniqueAlphas"], s["msGemm"]) for s in fst if s["msGemm"] > 0]
        fach = (sum(2.0 * r * u * n_pad * cfg["m"] * cfg["z"] for u, _ in fgemm) /
                (sum(t for _, t in fgemm) * 1e-3) / 1e12) if fgemm else None
        fgroups = [st["tcGroups"] for st in fst if st["msGemm"] > 0]
        ftraffic, ftraffic_note = gemm_traffic(cfg["m"] * cfg["z"] * ((r + 127) // 128) * max(1, fgroups[-1]),
                                               split=True) if fgroups else (None, None)
        bf16 = {"value": r * args.bf16_steps / (fms * 1e-3), "unit": UNIT, "steps": args.bf16_steps,
                "gemm_traffic": ftraffic, "gemm_traffic_note": ftraffic_note,
                "ms_per_step": fms / args.bf16_steps, "gemm_tflops_fp16_equivalent": fach,
                "gemm_tflops": 2.0 * fach if fach else None,
                "rows_rescored": fl["rowsMultiCand"], "rows_exact_scan": fl["rowsOverflow"],
                "candidates_rescored": fl["candidates"],
                "note": "same tcgen05 kernel with BF16 operands: beliefs in one BF16 term, alphas as a hi + lo pair "
                        "of BF16 terms (twice the FP16 form's MMA work); proven-margin exact re-score",
                "step_breakdown_ms": {k: fl[k] for k in ("msDedup", "msProject", "msScore", "msGemm", "msRescore",
                                                         "msActions", "msAssemble", "msTotal")}}
        if rank == 0 and args.parity_beliefs > 0:
            parity["bf16"] = sampled_parity(alg, model, args.parity_beliefs, seed=2,
                                            backup0=args.warmup + args.steps)
        alg.set_scoring(npp.SCORING_FP16)

    # ---- plain FP32 form on the same state -----------------------------------
    plain = None
    if args.plain_steps > 0:
        alg.set_scoring(npp.SCORING_EXACT)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record()
        for _ in range(args.plain_steps):
            alg.update()
        p1.record()
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p1)
        plain = {"value": r * args.plain_steps / (pms * 1e-3), "unit": UNIT, "steps": args.plain_steps,
                 "ms_per_step": pms / args.plain_steps,
                 "form": "FP32 SIMT scoring of every unique alpha in nova's operation order"}
        alg.set_scoring(npp.SCORING_FP16)

    # ---- FP16 without the projection table, on the same state ----------------
    table_free = None
    if args.table_free_steps > 0:
        alg.set_scoring(npp.SCORING_FP16)
        alg.set_table(npp.TABLE_NEVER)  # frees the table
        alg.update()  # not timed
        torch.cuda.synchronize()
        held = free_before2 - torch.cuda.mem_get_info()[0]
        t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tst = []
        t0e.record()
        for _ in range(args.table_free_steps):
            alg.update()
            tst.append(alg.stats())
        t1e.record()
        torch.cuda.synchronize()
        tms = t0e.elapsed_time(t1e)
        tl = tst[-1]
        table_free = {"value": r * args.table_free_steps / (tms * 1e-3), "unit": UNIT,
                      "steps": args.table_free_steps, "ms_per_step": tms / args.table_free_steps,
                      "solver_device_gb": held / 1e9,
                      "rows_rescored": tl["rowsMultiCand"], "candidates_rescored": tl["candidates"],
                      "rows_exact_scan": tl["rowsOverflow"],
                      "form": "FP16 tensor-core scoring; candidates re-scored, open rows' (belief, action) pairs "
                              "scored and new alphas assembled straight from the alphas "
                              "(pomdp_pbvi_set_table_gpu NOVA_PBVI_TABLE_NEVER; same bits)",
                      "step_breakdown_ms": {k: tl[k] for k in ("msDedup", "msProject", "msScore", "msGemm",
                                                               "msRescore", "msActions", "msAssemble", "msTotal")}}
        alg.set_table(npp.TABLE_AUTO)
    if second:
        del alg  # frees the second device solver before the remaining legs
        torch.cuda.synchronize()

    # ---- CPU baseline (oracle port of nova's loop) on a bounded sample ------
    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        cores = host_cores()
        v, pairs, wall = cpu_sample(model, Gnow, args.cpu_seconds, cores)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d (belief, action) pairs of nova's loop-form backup against the current alpha set "
                         "(r=%d) in %.1f s on %d threads" % (pairs, cfg["r"], wall, cores)}

    mdp = None if args.no_mdp else run_mdp(args, rank)
    precision = run_precision(args) if (rank == 0 and args.precision_steps > 0) else None
    if rank == 0 and args.precision_horizon > 0:
        precision = precision or {}
        precision["pbvi_n4096"] = run_precision_headline(args, model, p)
        precision["max_dV_b0"] = max(v["dV_b0"] for k, v in precision.items() if isinstance(v, dict))

    last = stats[-1]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16", "data": "synthetic",
        "config": {"workload": workload_name(cfg, args), "start_horizon": args.warmup,
                   "scoring": "FP16 tensor cores + proven-margin exact re-score (results bit-identical to FP32)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (FP16 scoring operands %.1f GB, alpha set %.0f MB)"
                         % (2.0 * cfg["r"] * n_pad * cfg["m"] * cfg["z"] / 1e9, cfg["r"] * cfg["n"] * 4 / 1e6)},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "plain_fp32": plain,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "step_breakdown_ms": {k: last[k] for k in ("msDedup", "msProject", "msScore", "msGemm", "msRescore",
                                                   "msActions", "msAssemble", "msTotal")},
        "solver_device_gb": solver_bytes / 1e9,
        "bf16_tc": bf16,
        "table_free": table_free,
        "unique_alphas": [s["uniqueAlphas"] for s in stats],
        "rows_rescored": last["rowsMultiCand"], "pairs_full_exact": last["rowsOverflow"],
        "mdp_vi": mdp,
        "precision_vs_fp64": precision,
        "parity_sampled": parity or None,
        "tc_vs_plain_fp32": {"fp16": value / plain["value"] if plain else None,
                             "bf16": bf16["value"] / plain["value"] if (plain and bf16) else None},
    }
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
