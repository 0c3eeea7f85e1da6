"""Gradient of a PBVI solution's value V(b0) with respect to the model.

H backups run on the GPU (pomdp_pbvi_execute_recorded_gpu) and record
their selections (the action per belief and the alpha chosen per
observation) together with Gamma checkpoints every k steps. With those
selections fixed, V(b0) = max_i b0 . Gamma_H[i] is a smooth function of R,
T and O, and pomdp_pbvi_adjoint_gpu returns its gradient (reverse mode,
FP64 accumulation, alphas between checkpoints recomputed bit-identically).

    spec = PBVIGradSpec(model, b0, horizon=50, checkpoint_every=10)
    V = pbvi_value(R, T, O, spec)          # R [n,m], T [n,m,ns], O [m,n,z] tensors
    V.backward()                            # R.grad, T.grad, O.grad

GammaInitial is an input of the solver, held fixed (it is not recomputed
from R). The selections are those of nova's FP32 backup (the library's
results are bit-identical to pomdp_pbvi_cpu.cpp:37-162), so the gradient is
that of the piecewise-smooth map on the piece the solve landed on.
"""
import ctypes as ct
from dataclasses import dataclass

import numpy as np
import torch

from . import nova_pomdp_pbvi as npp
from .pomdp import POMDP
from .pomdp_pbvi import POMDPPBVIGPU


@dataclass
class PBVIGradSpec:
    """Everything but the differentiated arrays: a model dict of synth.py's
    layout (S, Z, B, dimensions, gamma, GammaInitial), the belief b0, the
    horizon and the checkpoint interval."""
    model: dict
    b0: np.ndarray
    horizon: int
    checkpoint_every: int = 10


def _check(rc, name):
    if rc != 0:
        raise RuntimeError("%s failed with code %d" % (name, rc))


class PBVIValue(torch.autograd.Function):
    """V(b0) after `horizon` PBVI backups as a function of (R, T, O)."""

    @staticmethod
    def forward(ctx, R, T, O, spec):
        md = dict(spec.model)
        md["R"] = R.detach().to("cpu", torch.float32).numpy()
        md["T"] = T.detach().to("cpu", torch.float32).numpy()
        md["O"] = O.detach().to("cpu", torch.float32).numpy()
        n, m, z, r = md["n"], md["m"], md["z"], md["r"]
        H, k = int(spec.horizon), int(spec.checkpoint_every)
        pomdp = POMDP.from_arrays(md)
        pomdp.initialize_gpu()
        alg = POMDPPBVIGPU(pomdp, GammaInitial=md["GammaInitial"])
        dev = torch.device("cuda", torch.cuda.current_device())
        nck = (H + k - 1) // k
        ck = torch.empty((nck, r, n), dtype=torch.float32, device=dev)
        acts = torch.empty((H, r), dtype=torch.int32, device=dev)
        sels = torch.empty((H, r, z), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        _check(npp._nova.pomdp_pbvi_execute_recorded_gpu(alg.pomdpPtr, alg, H, k, ck.data_ptr(), acts.data_ptr(),
                                                         sels.data_ptr()), "pomdp_pbvi_execute_recorded_gpu")
        V, _ = alg.value(spec.b0)
        del alg
        ctx.pomdp = pomdp
        ctx.spec = spec
        ctx.devices = (R.device, T.device, O.device)
        ctx.dtypes = (R.dtype, T.dtype, O.dtype)
        ctx.save_for_backward(ck, acts, sels)
        return torch.tensor(V, dtype=torch.float64, device=R.device)

    @staticmethod
    def backward(ctx, gV):
        ck, acts, sels = ctx.saved_tensors
        spec, pomdp = ctx.spec, ctx.pomdp
        md = spec.model
        n, m, z, ns = md["n"], md["m"], md["z"], md["ns"]
        dev = ck.device
        b = torch.as_tensor(np.asarray(spec.b0, np.float32), device=dev)
        dR = torch.empty((n, m), dtype=torch.float64, device=dev)
        dT = torch.empty((n, m, ns), dtype=torch.float64, device=dev)
        dO = torch.empty((m, n, z), dtype=torch.float64, device=dev)
        V = ct.c_double(0.0)
        ia = ct.c_uint(0)
        torch.cuda.synchronize()
        _check(npp._nova.pomdp_pbvi_adjoint_gpu(ct.byref(pomdp), int(spec.horizon), int(spec.checkpoint_every),
                                                ck.data_ptr(), acts.data_ptr(), sels.data_ptr(), b.data_ptr(),
                                                dR.data_ptr(), dT.data_ptr(), dO.data_ptr(), None, ct.byref(V),
                                                ct.byref(ia)), "pomdp_pbvi_adjoint_gpu")
        g = gV.to(dev, torch.float64)
        out = []
        for d, device, dtype in zip((dR, dT, dO), ctx.devices, ctx.dtypes):
            out.append((g * d).to(device=device, dtype=dtype))
        return out[0], out[1], out[2], None


def pbvi_value(R, T, O, spec):
    """V(b0) (FP64 scalar tensor) after spec.horizon backups; differentiable
    in R, T and O."""
    return PBVIValue.apply(R, T, O, spec)


def pbvi_record_and_adjoint(model, b0, horizon, checkpoint_every=10):
    """The forward and reverse passes without autograd, returning numpy
    arrays: (V, istar, dR, dT, dO, dGamma0, actions [H][r], selects [H][r][z])."""
    n, m, z, r, ns = model["n"], model["m"], model["z"], model["r"], model["ns"]
    H, k = int(horizon), int(checkpoint_every)
    pomdp = POMDP.from_arrays(model)
    pomdp.initialize_gpu()
    alg = POMDPPBVIGPU(pomdp, GammaInitial=model["GammaInitial"])
    dev = torch.device("cuda", torch.cuda.current_device())
    ck = torch.empty(((H + k - 1) // k, r, n), dtype=torch.float32, device=dev)
    acts = torch.empty((H, r), dtype=torch.int32, device=dev)
    sels = torch.empty((H, r, z), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    _check(npp._nova.pomdp_pbvi_execute_recorded_gpu(alg.pomdpPtr, alg, H, k, ck.data_ptr(), acts.data_ptr(),
                                                     sels.data_ptr()), "pomdp_pbvi_execute_recorded_gpu")
    del alg
    b = torch.as_tensor(np.asarray(b0, np.float32), device=dev)
    dR = torch.empty((n, m), dtype=torch.float64, device=dev)
    dT = torch.empty((n, m, ns), dtype=torch.float64, device=dev)
    dO = torch.empty((m, n, z), dtype=torch.float64, device=dev)
    dG = torch.empty((r, n), dtype=torch.float64, device=dev)
    V = ct.c_double(0.0)
    ia = ct.c_uint(0)
    _check(npp._nova.pomdp_pbvi_adjoint_gpu(ct.byref(pomdp), H, k, ck.data_ptr(), acts.data_ptr(), sels.data_ptr(),
                                            b.data_ptr(), dR.data_ptr(), dT.data_ptr(), dO.data_ptr(), dG.data_ptr(),
                                            ct.byref(V), ct.byref(ia)), "pomdp_pbvi_adjoint_gpu")
    torch.cuda.synchronize()
    out = (V.value, ia.value, dR.cpu().numpy(), dT.cpu().numpy(), dO.cpu().numpy(), dG.cpu().numpy(),
           acts.cpu().numpy().astype(np.uint32), sels.cpu().numpy().astype(np.uint32))
    pomdp.uninitialize_gpu()
    return out


def pbvi_value_vs_fp64(model, b0, horizon, scoring=None, pomdp=None):
    """V(b0) after `horizon` backups from GammaInitial, and the same value
    recomputed in FP64 with the run's selections held fixed
    (pomdp_pbvi_value_replay_f64_gpu). Returns (V, V_fp64, istar, acts,
    sels): V is the FP64 reduction of the FP32 alphas at their maximising
    row istar, V_fp64 that row of the FP64 replay, so |V - V_fp64| is the
    arithmetic error of the FP32 backups; acts [H][r] and sels [H][r][z] are
    the recorded selections (numpy)."""
    n, z, r = model["n"], model["z"], model["r"]
    H = int(horizon)
    own = pomdp is None
    if own:
        pomdp = POMDP.from_arrays(model)
        pomdp.initialize_gpu()
    alg = POMDPPBVIGPU(pomdp, GammaInitial=model["GammaInitial"])
    if scoring is not None:
        alg.set_scoring(scoring)
    dev = torch.device("cuda", torch.cuda.current_device())
    ck = torch.empty((1, r, n), dtype=torch.float32, device=dev)
    acts = torch.empty((H, r), dtype=torch.int32, device=dev)
    sels = torch.empty((H, r, z), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    _check(npp._nova.pomdp_pbvi_execute_recorded_gpu(alg.pomdpPtr, alg, H, H, ck.data_ptr(), acts.data_ptr(),
                                                     sels.data_ptr()), "pomdp_pbvi_execute_recorded_gpu")
    V, _ = alg.value(b0)
    # the maximising row of the FP32 alphas (FP64 reduction, lowest index on ties)
    pol = alg.get_policy()
    vals = pol.gamma_array().astype(np.float64) @ np.asarray(b0, np.float64)
    del pol
    del alg
    istar = int(np.argmax(vals))
    b = torch.as_tensor(np.asarray(b0, np.float32), device=dev)
    V64 = ct.c_double(0.0)
    used = ct.c_uint(0)
    _check(npp._nova.pomdp_pbvi_value_replay_f64_gpu(ct.byref(pomdp), H, ck.data_ptr(), acts.data_ptr(),
                                                     sels.data_ptr(), b.data_ptr(), istar, ct.byref(V64),
                                                     ct.byref(used)), "pomdp_pbvi_value_replay_f64_gpu")
    torch.cuda.synchronize()
    out = (V, V64.value, istar, acts.cpu().numpy().astype(np.uint32), sels.cpu().numpy().astype(np.uint32))
    if own:
        pomdp.uninitialize_gpu()
    return out
