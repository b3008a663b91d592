"""Training and evaluation of the learned thermal preconditioner.

Problems: cubic volumes of random non-overlapping spheres (radius 4-16 voxels
scaled to the volume, solid fraction 0.2-0.4, per-sample seed), conductivity
k_s = 200 k_f in the spheres, a uniform +x velocity in the fluid, inlet plane
Dirichlet, pseudo-time step dt = 1000 of the reference operator A = I + dt L.
Training pairs (r, e) are generated by the plain solver itself: e = A^-1 r to
an FP64 relative residual of 1e-9 for right-hand sides that mix point sources,
smooth fields and noise.  Evaluation: flexible GMRES to a 1e-8 FP64 residual
with the network as preconditioner (plain V-cycle fallback on stall) against
the same FGMRES with one V-cycle, on held-out seeds, and the device-resident
plain BiCGSTAB beside them.  The default mode uses the network as a correction
after one V-cycle (LearnedCorrection), trained with a relative loss on the
residual a V-cycle leaves; `correction_quality` measures what one application
gains over the V-cycle alone.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from .geometry import random_spheres_mask
from .learned import LearnedCorrection, LearnedPreconditioner, UNetPreconditioner
from .solver import mg_pcg
from .solver.nlevel_mg_cuda import NLevelGeometricMGSolver

ALPHA_F = 0.01
K_RATIO = 200.0
U_FLUID = 0.05
DT = 1000.0


def make_problem(n: int, seed: int, dev, radii=None):
    """Binary conductivity from random spheres (k_s/k_f = 200), uniform flow along +x in the fluid,
    inlet plane Dirichlet, A = I + dt L with dt = 1000.  radii = (rmin, rmax); by default they scale
    with n (2-4 cells at 32^3), the 256^3 held-out set uses 4-16 cells."""
    rmin, rmax = radii if radii else (max(2.0, 4.0 * n / 256 * 4), max(4.0, 16.0 * n / 256 * 2))
    solid = random_spheres_mask(n, seed, rmin=rmin, rmax=rmax, device=dev)
    k = torch.full((n, n, n), ALPHA_F, device=dev)
    k[solid] = ALPHA_F * K_RATIO
    rcp = torch.ones((n, n, n), device=dev)
    u = torch.full((n, n, n), U_FLUID, device=dev)
    u[solid] = 0.0
    z = torch.zeros((n, n, n), device=dev)
    mask = torch.ones((n, n, n), dtype=torch.bool, device=dev)
    mask[0] = False
    mg = NLevelGeometricMGSolver(dev, torch.float32, 0, +1, 1.0, omega=0.6)
    mg.build_if_needed(k, rcp, u, z, z, mask, DT)
    return mg, k, solid


def random_rhs(n: int, rng: np.random.Generator, dev, solid):
    kind = rng.integers(3)
    if kind == 0:      # a few heat sources inside the solid
        b = torch.zeros((n, n, n), device=dev)
        idx = torch.nonzero(solid)
        if idx.numel():
            sel = idx[torch.tensor(rng.integers(0, idx.shape[0], size=8), device=dev)]
            b[sel[:, 0], sel[:, 1], sel[:, 2]] = torch.tensor(rng.uniform(0.5, 2.0, size=8), device=dev,
                                                              dtype=torch.float32)
    elif kind == 1:    # smooth random field
        c = torch.tensor(rng.standard_normal((1, 1, 4, 4, 4)), device=dev, dtype=torch.float32)
        b = torch.nn.functional.interpolate(c, size=(n, n, n), mode="trilinear", align_corners=False)[0, 0]
    else:              # white noise
        b = torch.tensor(rng.standard_normal((n, n, n)), device=dev, dtype=torch.float32)
    b[0] = 0.0
    return b.contiguous()


def residual_after_vcycle(mg, b: torch.Tensor) -> torch.Tensor:
    """b - A V(b) (FP32, masked): what one plain V-cycle leaves of the right-hand side b."""
    from . import _lib
    from ._torch import ptr, stream_ptr
    lv0 = mg._levels[0]
    nx, ny, nz = lv0["shape"]
    lv0["b_buf"].copy_(b.reshape(lv0["shape"]))
    mg._vcycle(0, zero_guess=True)
    r1 = torch.empty(lv0["shape"], dtype=torch.float32, device=b.device)
    _lib.call("fc_mg_mop_f32", ptr(lv0["x"]), *mg._cptrs(lv0), float(mg._dt_cache), nx, ny, nz, mg.ax,
              lv0["out_idx"], ptr(lv0["b_buf"]), ptr(lv0["mask_f"]), ptr(r1), stream_ptr())
    return r1


def generate_pairs(n: int, n_geom: int, per_geom: int, seed0: int, dev, correction: bool = False):
    """(r, e = A^-1 r, k) triples solved by the plain solver; with `correction`, r is the residual
    one V-cycle leaves of a random right-hand side (the network's input inside LearnedCorrection)."""
    rng = np.random.default_rng(seed0)
    data = []
    for g in range(n_geom):
        mg, k, solid = make_problem(n, seed0 + g, dev)
        for _ in range(per_geom):
            b = random_rhs(n, rng, dev, solid)
            if correction:
                b = residual_after_vcycle(mg, b).contiguous()
            x, info = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-9, max_it=400)
            data.append((b, x.float().contiguous(), k))
    return data


def train(net: UNetPreconditioner, data, steps: int, batch: int = 2, lr: float = 2e-3, seed: int = 0,
          relative: bool = True):
    rng = np.random.default_rng(seed)
    losses = []
    t0 = time.perf_counter()
    for it in range(steps):
        idx = rng.integers(0, len(data), size=batch)
        r = torch.stack([data[i][0] for i in idx])
        e = torch.stack([data[i][1] for i in idx])
        k = torch.stack([data[i][2] for i in idx])
        loss, _ = net.loss_and_grad(r, k, e, relative=relative)
        lr_t = lr * 0.5 * (1 + math.cos(math.pi * it / max(1, steps)))
        net.adam_step(lr=lr_t)
        losses.append(loss)
    torch.cuda.synchronize()
    return losses, time.perf_counter() - t0


def evaluate(net: UNetPreconditioner, n: int, seeds, dev, tol=1e-8, repeats=3, correction: bool = False):
    rows = []
    rng = np.random.default_rng(12345)
    for s in seeds:
        mg, k, solid = make_problem(n, s, dev)
        b = random_rhs(n, rng, dev, solid)
        pc = LearnedCorrection(net, mg, k) if correction else LearnedPreconditioner(net, mg, k)

        def timed(fn):
            best, info = None, None
            for _ in range(repeats):
                torch.cuda.synchronize()
                t = time.perf_counter()
                _, info = fn()
                torch.cuda.synchronize()
                dt = (time.perf_counter() - t) * 1e3
                best = dt if best is None else min(best, dt)
            return best, info
        plain_ms, plain = timed(lambda: mg_pcg.fgmres_mg_f64(mg, b, tol=tol, max_it=300, restart=30))
        learn_ms, learn = timed(lambda: mg_pcg.fgmres_mg_f64(mg, b, tol=tol, max_it=300, restart=30, precond=pc,
                                                              stall_fallback=mg_pcg._vcycle_pc(mg)))
        bicg_ms, bicg = timed(lambda: mg_pcg.bicgstab_mg_f64(mg, b, tol=tol, max_it=300))
        rows.append({"seed": int(s), "plain_ms": round(plain_ms, 3), "plain_it": plain["it"],
                     "plain_res": plain["res_rel"], "learned_ms": round(learn_ms, 3), "learned_it": learn["it"],
                     "learned_res": learn["res_rel"], "learned_fell_back": learn["fell_back"],
                     "learned_fell_back_at": learn.get("fell_back_at"),
                     "plain_bicgstab_ms": round(bicg_ms, 3), "plain_bicgstab_it": bicg["it"],
                     "plain_bicgstab_res": bicg["res_rel"]})
    return rows


def correction_quality(net: UNetPreconditioner, n: int, seeds, dev) -> list:
    """Relative error after one plain V-cycle and after the V-cycle plus the network correction,
    against the exact solution (FP64 solve to 1e-10), on held-out problems."""
    rows = []
    rng = np.random.default_rng(7)
    for s in seeds:
        mg, k, solid = make_problem(n, s, dev)
        b = random_rhs(n, rng, dev, solid)
        e, _ = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=500)
        e = e.float()
        pc = LearnedCorrection(net, mg, k)
        r1 = pc.residual_after_vcycle(b.contiguous())
        v = mg._levels[0]["x"].clone()
        y = net.forward(r1.reshape((1,) + tuple(r1.shape[-3:])), pc.k).reshape(v.shape)
        nrm = float(torch.linalg.norm(e))
        rows.append({"seed": int(s), "vcycle_rel_err": float(torch.linalg.norm(e - v)) / nrm,
                     "vcycle_plus_net_rel_err": float(torch.linalg.norm(e - v - y)) / nrm})
    return rows


def eval_large(net: UNetPreconditioner, dev, n=256, seeds=(2001, 2002), tol=1e-8):
    """Held-out 256^3 problems (spheres of radius 4-16 cells): the one-shot quality of the
    V-cycle + network correction and the solve times of plain BiCGSTAB, plain FGMRES and FGMRES
    with the learned correction (plain V-cycle fallback on stall), all to an FP64 residual `tol`."""
    rows = []
    rng = np.random.default_rng(4242)
    for s in seeds:
        mg, k, solid = make_problem(n, s, dev, radii=(4.0, 16.0))
        b = random_rhs(n, rng, dev, solid)
        e, _ = mg_pcg.bicgstab_mg_f64(mg, b, tol=1e-10, max_it=500)
        e = e.float()
        pc = LearnedCorrection(net, mg, k)
        r1 = pc.residual_after_vcycle(b.contiguous())
        v = mg._levels[0]["x"].clone()
        y = net.forward(r1.reshape((1,) + tuple(r1.shape[-3:])), pc.k).reshape(v.shape)
        nrm = float(torch.linalg.norm(e))
        row = {"seed": int(s), "vcycle_rel_err": float(torch.linalg.norm(e - v)) / nrm,
               "vcycle_plus_net_rel_err": float(torch.linalg.norm(e - v - y)) / nrm}
        del e, v, y
        for name, fn in (("plain_bicgstab", lambda: mg_pcg.bicgstab_mg_f64(mg, b, tol=tol, max_it=400)),
                         ("plain_fgmres", lambda: mg_pcg.fgmres_mg_f64(mg, b, tol=tol, max_it=400, restart=30)),
                         ("learned_fgmres", lambda: mg_pcg.fgmres_mg_f64(mg, b, tol=tol, max_it=400, restart=30,
                                                                         precond=pc,
                                                                         stall_fallback=mg_pcg._vcycle_pc(mg)))):
            torch.cuda.synchronize()
            t = time.perf_counter()
            _, info = fn()
            torch.cuda.synchronize()
            row[name] = {"ms": round((time.perf_counter() - t) * 1e3, 1), "it": info["it"], "res": info["res_rel"],
                         "fell_back": info.get("fell_back"), "fell_back_at": info.get("fell_back_at")}
        rows.append(row)
        del mg, pc
        torch.cuda.empty_cache()
    return rows


def run(dev, n_train=32, n_eval=64, n_geom=24, per_geom=4, steps=1500, lr=5e-4, eval_seeds=(1001, 1002, 1003),
        correction: bool = True):
    """Train (output layer started at zero, Adam at lr with a cosine schedule) on MG-generated pairs,
    then measure the one-shot correction quality and the FGMRES A/B on held-out problems."""
    t = time.perf_counter()
    data = generate_pairs(n_train, n_geom, per_geom, 100, dev, correction=correction)
    gen_s = time.perf_counter() - t
    net = UNetPreconditioner(device=dev, seed=0, zero_last=True)
    losses, train_s = train(net, data, steps, lr=lr)
    rows = evaluate(net, n_eval, eval_seeds, dev, correction=correction)
    quality = correction_quality(net, n_eval, eval_seeds[:2], dev) if correction else []
    out = {"mode": "V-cycle + network correction" if correction else "network alone",
           "train_volume": n_train, "pairs": len(data), "pair_generation_s": round(gen_s, 2), "train_steps": steps,
           "learning_rate": lr,
           "train_s": round(train_s, 2), "loss_first": float(np.mean(losses[:10])),
           "loss_last": float(np.mean(losses[-10:])), "eval_volume": n_eval, "eval": rows,
           "speedup_plain_over_learned": round(float(np.median([r["plain_ms"] / r["learned_ms"] for r in rows])), 3),
           "iteration_ratio_plain_over_learned": round(float(np.median([r["plain_it"] / max(1, r["learned_it"])
                                                                        for r in rows])), 3),
           "speedup_plain_bicgstab_over_learned": round(float(np.median([r["plain_bicgstab_ms"] / r["learned_ms"]
                                                                         for r in rows])), 3),
           "correction_quality": quality,
           "held_out_256": eval_large(net, dev),
           "device_error": net.check_device_error()}
    return out
