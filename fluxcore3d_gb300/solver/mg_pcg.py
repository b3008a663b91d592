"""Drop-in replacement for the reference's solver/mg_pcg.py, plus FP64-certified solvers.

Reference surface (solver/mg_pcg.py):
  pcg_mg(mg_solver, b, x0=None, tol=1e-3, max_it=15)        :33-97
  bicgstab_mg(mg_solver, b, x0=None, tol=1e-3, max_it=15)   :103-175
  _precond(mg_solver, r)                                      :178-187  (one V-cycle)
  chebyshev_smooth(mg_solver, level, n_steps=2, lam_min_ratio=0.1) :195-244
  patch_mg_pcg(mg_solver, pe_threshold=1.5)                   :250-275
They keep the reference's FP32 vectors and iteration logic; dot products
accumulate in FP64 in the native library.

Certified solvers (new): `bicgstab_mg_f64` and `fgmres_mg_f64` iterate on FP64
vectors with the operator applied in FP64, precondition with the FP32 V-cycle
(or any callable r32 -> z32, e.g. the learned preconditioner), and stop on the
true FP64 relative residual ||mask (b - A x)|| / ||mask b||.  FGMRES is
flexible, so a preconditioner that changes between applications (the learned
one, or one that falls back to the V-cycle) is allowed.
"""
from __future__ import annotations

import math
import types
from typing import Callable, Optional, Tuple

import torch

from .. import _lib
from .._torch import capture_graph, ptr, stream_ptr

Tensor = torch.Tensor


class _Vec:
    """FP64-accumulated vector kernels bound to one solver's fine level."""

    def __init__(self, mg):
        self.mg = mg
        lv0 = mg._levels[0]
        self.n = lv0["mask_f"].numel()
        nbytes = _lib.call("fc_vec_workspace_bytes", self.n)
        self.ws = torch.empty(int(nbytes), dtype=torch.uint8, device=mg.device)
        self.sc = torch.zeros(64, dtype=torch.float64, device=mg.device)

    def dot_dev(self, a: Tensor, b: Tensor, slot: int, weight: Optional[Tensor] = None) -> Tensor:
        if a.dtype == torch.float64 and b.dtype == torch.float64:
            kind = 0
        elif a.dtype == torch.float32 and b.dtype == torch.float32:
            kind = 1
        else:
            if a.dtype == torch.float32:
                a, b = b, a
            kind = 2
        _lib.call("fc_vec_dot", kind, ptr(a), ptr(b), self.n, ptr(weight), ptr(self.ws), self.ws.numel(),
                  ptr(self.sc[slot:slot + 1]), stream_ptr())
        return self.sc[slot:slot + 1]

    def dot(self, a: Tensor, b: Tensor, slot: int = 0) -> float:
        return float(self.dot_dev(a, b, slot).item())

    def axpby(self, y: Tensor, x: Tensor, alpha: float, beta: float = 1.0, num: Optional[Tensor] = None,
              den: Optional[Tensor] = None, mask: Optional[Tensor] = None) -> None:
        _lib.call("fc_vec_axpby", int(y.dtype == torch.float64), ptr(y), ptr(x), self.n, float(alpha), ptr(num),
                  ptr(den), float(beta), ptr(mask), stream_ptr())

    def convert(self, dst: Tensor, src: Tensor, mask: Optional[Tensor] = None, scale: float = 1.0) -> None:
        kind = {(torch.float32, torch.float64): 0, (torch.float64, torch.float32): 1,
                (torch.float32, torch.float32): 2, (torch.float64, torch.float64): 3}[(src.dtype, dst.dtype)]
        _lib.call("fc_vec_convert", kind, ptr(dst), ptr(src), self.n, ptr(mask), float(scale), stream_ptr())

    def mop64(self, x: Tensor, y: Tensor, b: Optional[Tensor] = None, mask: Optional[Tensor] = None) -> None:
        mg = self.mg
        lv = mg._levels[0]
        nx, ny, nz = lv["shape"]
        _lib.call("fc_mg_mop_f64", ptr(x), *mg._cptrs(lv), float(mg._dt_cache), nx, ny, nz, mg.ax, lv["out_idx"],
                  ptr(b), ptr(mask), ptr(y), stream_ptr())


def _vec(mg) -> _Vec:
    v = getattr(mg, "_fc_vec", None)
    if v is None or v.n != mg._levels[0]["mask_f"].numel():
        v = _Vec(mg)
        mg._fc_vec = v
    return v


def _precond(mg_solver, r: Tensor) -> Tensor:
    """One V-cycle from a zero guess applied to r (reference mg_pcg.py:178-187)."""
    lv0 = mg_solver._levels[0]
    V = _vec(mg_solver)
    V.convert(lv0["b_buf"], r.contiguous(), lv0["mask_f"])
    mg_solver._vcycle(0, zero_guess=True)
    z = torch.empty_like(lv0["x"])
    V.convert(z, lv0["x"], lv0["mask_f"])
    return z


def pcg_mg(mg_solver, b: Tensor, x0: Optional[Tensor] = None, tol: float = 1e-3,
           max_it: int = 15) -> Tuple[Tensor, dict]:
    """Preconditioned CG with one V-cycle as M^-1 (reference mg_pcg.py:33-97)."""
    lv0 = mg_solver._levels[0]
    mask = lv0["mask_f"]
    V = _vec(mg_solver)
    b = b.contiguous().to(torch.float32)
    x = torch.zeros_like(b)
    if x0 is not None:
        V.convert(x, x0.contiguous().to(torch.float32), mask)
    mg_solver._Mop(x, 0)
    r = b.clone()
    V.axpby(r, lv0["Lo"], -1.0, 1.0, mask=mask)           # r = (b - A x) * mask
    z = _precond(mg_solver, r)
    p = z.clone()
    rz = V.dot(r, z, 0)
    bnorm = math.sqrt(V.dot(b, b, 1)) + 1e-30
    converged = False
    it = 0
    for it in range(max_it):
        res_rel = math.sqrt(V.dot(r, r, 2)) / bnorm
        if res_rel < tol:
            converged = True
            break
        mg_solver._Mop(p, 0)
        Ap = lv0["Lo"].clone()
        pAp = V.dot(p, Ap, 3)
        if abs(pAp) < 1e-30:
            break
        alpha = rz / pAp
        V.axpby(x, p, alpha)
        V.axpby(r, Ap, -alpha, 1.0, mask=mask)
        z = _precond(mg_solver, r)
        rz_new = V.dot(r, z, 4)
        beta = rz_new / (rz + 1e-30)
        V.axpby(p, z, 1.0, beta)
        rz = rz_new
    V.convert(x, x, mask)
    return x, {"converged": converged, "it": it + 1, "res_rel": math.sqrt(V.dot(r, r, 5)) / bnorm}


def bicgstab_mg(mg_solver, b: Tensor, x0: Optional[Tensor] = None, tol: float = 1e-3,
                max_it: int = 15) -> Tuple[Tensor, dict]:
    """Preconditioned BiCGSTAB, one V-cycle per application (reference mg_pcg.py:103-175)."""
    lv0 = mg_solver._levels[0]
    mask = lv0["mask_f"]
    V = _vec(mg_solver)
    b = b.contiguous().to(torch.float32)
    x = torch.zeros_like(b)
    if x0 is not None:
        V.convert(x, x0.contiguous().to(torch.float32), mask)
    mg_solver._Mop(x, 0)
    r = b.clone()
    V.axpby(r, lv0["Lo"], -1.0, 1.0, mask=mask)
    r_hat = r.clone()
    bnorm = math.sqrt(V.dot(b, b, 0)) + 1e-30
    rho = alpha = omega = 1.0
    v = torch.zeros_like(b)
    p = torch.zeros_like(b)
    converged = False
    it = 0
    for it in range(max_it):
        res_rel = math.sqrt(V.dot(r, r, 1)) / bnorm
        if res_rel < tol:
            converged = True
            break
        rho_new = V.dot(r_hat, r, 2)
        if abs(rho_new) < 1e-30:
            break
        beta = (rho_new / (rho + 1e-30)) * (alpha / (omega + 1e-30))
        V.axpby(p, r, 1.0, beta)                  # p = beta p + r
        V.axpby(p, v, -beta * omega)              # p -= beta omega v
        p_hat = _precond(mg_solver, p)
        mg_solver._Mop(p_hat, 0)
        v = lv0["Lo"].clone()
        alpha = rho_new / (V.dot(r_hat, v, 3) + 1e-30)
        s = r.clone()
        V.axpby(s, v, -alpha, 1.0, mask=mask)
        if math.sqrt(V.dot(s, s, 4)) / bnorm < tol:
            V.axpby(x, p_hat, alpha)
            converged = True
            break
        s_hat = _precond(mg_solver, s)
        mg_solver._Mop(s_hat, 0)
        t = lv0["Lo"].clone()
        omega = V.dot(t, s, 5) / (V.dot(t, t, 6) + 1e-30)
        V.axpby(x, p_hat, alpha)
        V.axpby(x, s_hat, omega, 1.0, mask=mask)
        r = s.clone()
        V.axpby(r, t, -omega, 1.0, mask=mask)
        rho = rho_new
    V.convert(x, x, mask)
    return x, {"converged": converged, "it": it + 1, "res_rel": math.sqrt(V.dot(r, r, 7)) / bnorm}


def chebyshev_smooth(mg_solver, level: int, n_steps: int = 2, lam_min_ratio: float = 0.1) -> None:
    """Chebyshev smoothing on one level in place (reference mg_pcg.py:195-244)."""
    lv = mg_solver._levels[level]
    x, b, inv, mask = lv["x"], lv["b_buf"], lv["inv_diagM"], lv["mask_f"]
    n = x.numel()
    st = stream_ptr()
    lam_max = float(torch.amax(lv["diagL"]).item()) * float(mg_solver._dt_cache) + 1.0
    lam_min = lam_min_ratio * lam_max
    d = (lam_max + lam_min) / 2.0
    c = (lam_max - lam_min) / 2.0

    def resid(src, out):
        mg_solver._Mop(src, level)
        _lib.call("fc_vec_convert", 2, ptr(out), ptr(b), n, None, 1.0, st)
        _lib.call("fc_vec_axpby", 0, ptr(out), ptr(lv["Lo"]), n, -1.0, None, None, 1.0, ptr(mask), st)
        _lib.call("fc_vec_convert", 2, ptr(out), ptr(out), n, ptr(inv), 1.0, st)   # out = invD r

    p = torch.empty_like(x)
    resid(x, p)
    x_new = x.clone()
    _lib.call("fc_vec_axpby", 0, ptr(x_new), ptr(p), n, 1.0, None, None, 1.0, None, st)
    if n_steps == 1:
        x.copy_(x_new)
        return
    rho_prev = 1.0
    q = torch.empty_like(x)
    for _ in range(1, n_steps):
        rho_new = 1.0 / (2.0 * d / c - rho_prev)
        resid(x_new, q)
        # p = rho_new (2d/c invD r + rho_prev p)
        _lib.call("fc_vec_axpby", 0, ptr(p), ptr(q), n, rho_new * 2.0 * d / c, None, None, rho_new * rho_prev,
                  None, st)
        _lib.call("fc_vec_axpby", 0, ptr(x_new), ptr(p), n, 1.0, None, None, 1.0, None, st)
        rho_prev = rho_new
    _lib.call("fc_vec_convert", 2, ptr(x), ptr(x_new), n, ptr(mask), 1.0, st)


def patch_mg_pcg(mg_solver, pe_threshold: float = 1.5, method: Optional[str] = None):
    """Replace mg_solver.solve with PCG / BiCGSTAB chosen by the reference's Peclet heuristic
    (reference mg_pcg.py:250-275: pe = 0.1 max(diagL)).

    method="bicgstab_f64" (no counterpart in the reference) instead solves with the device-resident
    FP64 BiCGSTAB around the FP32 V-cycle (bicgstab_mg_f64), certified on the FP64 true residual:
    the FP32 stationary V-cycle iteration stalls where its FP32 residual A x loses the digits of
    b (A = I + dt L with a large dt); FP64 residuals remove that floor.  The result is returned in
    the right-hand side's precision."""

    def _solve_pcg(self, b, x0=None, max_cycles=15, tol=1e-3):
        pe = float(torch.amax(self._levels[0]["diagL"]).item()) * 0.1
        if pe > pe_threshold:
            return bicgstab_mg(self, b, x0, tol=tol, max_it=max_cycles)
        return pcg_mg(self, b, x0, tol=tol, max_it=max_cycles)

    def _solve_f64(self, b, x0=None, max_cycles=15, tol=1e-3):
        x, info = bicgstab_mg_f64(self, b, x0, tol=tol, max_it=max_cycles)
        out = {"converged": info["converged"], "diverged": not math.isfinite(info["res_rel"]), "it": info["it"],
               "res_rel": info["res_rel"], "res0_rel": info.get("res0_rel", float("nan"))}
        return x.to(b.dtype), out

    if method not in (None, "bicgstab_f64"):
        raise ValueError("method must be None (the reference's PCG/BiCGSTAB choice) or 'bicgstab_f64'")
    mg_solver.solve = types.MethodType(_solve_f64 if method == "bicgstab_f64" else _solve_pcg, mg_solver)
    what = "FP64 BiCGSTAB (FP32 V-cycle)" if method else f"PCG/BiCGSTAB (pe_threshold={pe_threshold})"
    print(f"[MG-PCG] Patched mg_solver.solve -> {what}")


# ---------------------------------------------------------------------------
# FP64-certified solvers
# ---------------------------------------------------------------------------
def _vcycle_pc(mg_solver) -> Callable[[Tensor, Tensor], None]:
    """One V-cycle from zero as the map r64 -> z64.  The fine level is looked up at every call:
    a rebuilt hierarchy (new coefficients) replaces the level buffers."""
    V = _vec(mg_solver)

    def apply(r64: Tensor, z64: Tensor) -> None:
        lv0 = mg_solver._levels[0]
        V.convert(lv0["b_buf"], r64, lv0["mask_f"])          # FP64 residual -> FP32 right-hand side
        mg_solver._vcycle(0, zero_guess=True)
        V.convert(z64, lv0["x"], lv0["mask_f"])
    return apply


def _hier_key(mg):
    """Identity of the solver's current hierarchy for the captured graphs: a rebuild (new velocity,
    new coefficients) gets a new generation even when the allocator hands back the same addresses."""
    return (id(mg._levels), getattr(mg, "_generation", 0))


def _coarse_key(mg):
    """What a captured V-cycle bakes in about the coarsest-level solve (the FP64 inverse's buffer)."""
    inv = getattr(mg, "_coarse_inv", None)
    return (getattr(mg, "coarse_solve", "jacobi"), inv.data_ptr() if inv is not None else 0)


class _GraphVcyclePC:
    """The V-cycle preconditioner r64 -> z64 replayed from one CUDA graph per (r64, z64) buffer
    pair (two conversions and the ~40 launches of a 5-level V-cycle become one launch).  The
    graphs are recaptured whenever the hierarchy or dt changes, since both are baked into them."""

    def __init__(self, mg):
        self.mg = mg
        self.eager = _vcycle_pc(mg)
        self.graphs = {}
        self.key = None

    def _version(self):
        mg = self.mg
        return (_hier_key(mg), mg._dt_cache, tuple(lv["x"].data_ptr() for lv in mg._levels), mg.n_pre, mg.n_post,
                mg.n_coarse, _coarse_key(mg))

    def __call__(self, r64: Tensor, z64: Tensor) -> None:
        ver = self._version()
        if ver != self.key:
            self.graphs.clear()
            self.key = ver
        k = (r64.data_ptr(), z64.data_ptr())
        g = self.graphs.get(k)
        if g is None:
            g = capture_graph(lambda: self.eager(r64, z64))
            self.graphs[k] = g
        g.replay()


def _graph_pc(mg) -> _GraphVcyclePC:
    pc = getattr(mg, "_fc_graph_pc", None)
    if pc is None:
        pc = _GraphVcyclePC(mg)
        mg._fc_graph_pc = pc
    return pc


def _bicg_work(mg, shape, dtype, dev) -> dict:
    """Work vectors and device scalars of the device-resident BiCGSTAB, kept on the solver
    object so the captured iteration graphs (which bake their addresses) are reused from one
    solve to the next."""
    key = "_fc_bicg64" if dtype == torch.float64 else "_fc_bicg32"
    W = getattr(mg, key, None)
    if W is None or W["r"].shape != tuple(shape):
        n = int(torch.tensor(shape).prod())
        W = {name: torch.zeros(shape, dtype=dtype, device=dev)
             for name in ("x", "b", "r", "r_hat", "p", "v", "ph", "sh", "t")}
        W["sc"] = torch.zeros(9, dtype=torch.float64, device=dev)
        W["init"] = torch.tensor([0, 1, 1, 1, 0, 0, 0, 0, 0], dtype=torch.float64, device=dev)
        W["ws"] = torch.empty(int(_lib.call("fc_vec_dot2_workspace_bytes", n)), dtype=torch.uint8, device=dev)
        W["host"] = torch.zeros(2, dtype=torch.float64).pin_memory()
        W["ev"] = [torch.cuda.Event() for _ in range(2)]
        W["graphs"] = {}
        setattr(mg, key, W)
    return W


def _bicg_solve(mg, V: _Vec, b: Tensor, x: Tensor, bnorm: float, tol: float, max_it: int, mask: Tensor) -> dict:
    """Right-preconditioned BiCGSTAB on FP64 or FP32 vectors (the dtype of b and x) with the
    recurrence scalars on the device.  One iteration -- two V-cycles, two operator applies,
    three reductions and the fused updates -- is replayed from a CUDA graph; two graphs
    alternate the pinned slot that receives the iteration's residual norm, and the host tests
    iteration k-1's norm while iteration k runs, then confirms with the true residual in the
    vectors' precision (restarting from it if the recursive residual drifted).  x is updated
    in place."""
    f64 = b.dtype == torch.float64
    n = V.n
    W = _bicg_work(mg, tuple(b.shape), b.dtype, b.device)
    xw, bw, r, r_hat, p, v, ph, sh, t, sc = (W[k] for k in ("x", "b", "r", "r_hat", "p", "v", "ph", "sh", "t",
                                                            "sc"))
    ws = W["ws"]
    pc = _graph_pc(mg).eager
    lv0 = mg._levels[0]
    if not f64:
        # FP32 vectors: the V-cycle reads its right-hand side from the Krylov vector and leaves its
        # result in the destination vector (no masked copies in or out).  Every vector of this
        # recurrence is zero on the Dirichlet rows (the operator apply masks them, and the
        # smoother's inverse diagonal is zero there), so the copies would change nothing.
        def pc(src, dst):
            saved = (lv0["b_buf"], lv0["x"])
            lv0["b_buf"], lv0["x"] = src, dst
            try:
                mg._vcycle(0, zero_guess=True)
            finally:
                lv0["b_buf"], lv0["x"] = saved
    nx, ny, nz = lv0["shape"]
    mop_name = "fc_mg_mop_f64" if f64 else "fc_mg_mop_f32"
    dt = float(mg._dt_cache)
    cps = mg._cptrs(lv0)
    k = int(f64)

    def mop(xv, yv, bv=None):
        _lib.call(mop_name, ptr(xv), *cps, dt, nx, ny, nz, mg.ax, lv0["out_idx"], ptr(bv), ptr(mask), ptr(yv),
                  stream_ptr())

    def dot_into(a_, b_, slot):
        _lib.call("fc_vec_dot", 0 if f64 else 1, ptr(a_), ptr(b_), n, None, ptr(ws), ws.numel(),
                  ptr(sc[slot:slot + 1]), stream_ptr())

    def iteration(slot):
        st = stream_ptr()
        dot_into(r_hat, r, 0)                                                      # rho_new
        _lib.call("fc_bicgstab_p", k, ptr(p), ptr(r), ptr(v), n, ptr(sc), st)     # p = r + beta (p - omega v)
        pc(p, ph)
        mop(ph, v)
        dot_into(r_hat, v, 4)
        _lib.call("fc_bicgstab_xr", k, ptr(xw), ptr(r), ptr(ph), ptr(v), n, ptr(sc), 0, ptr(ws), ws.numel(), st)
        pc(r, sh)
        mop(sh, t)
        _lib.call("fc_vec_dot2", k, ptr(t), ptr(r), ptr(t), n, ptr(ws), ws.numel(), ptr(sc[5:7]), st)
        _lib.call("fc_bicgstab_xr", k, ptr(xw), ptr(r), ptr(sh), ptr(t), n, ptr(sc), 1, ptr(ws), ws.numel(), st)
        W["host"][slot:slot + 1].copy_(sc[7:8], non_blocking=True)

    gkey = (_hier_key(mg), dt, tuple(lv["x"].data_ptr() for lv in mg._levels), mask.data_ptr(), mg.n_pre,
            mg.n_post, mg.n_coarse, _coarse_key(mg))
    graphs = W["graphs"].get(gkey)
    if graphs is None:
        W["graphs"].clear()
        graphs = []
        for slot in range(2):
            graphs.append(capture_graph(lambda: iteration(slot)))
        W["graphs"][gkey] = graphs

    def true_res() -> float:
        mop(xw, t, bw)
        dot_into(t, t, 7)
        return math.sqrt(max(float(sc[7].item()), 0.0)) / bnorm

    def restart():
        mop(xw, r, bw)                                # r = b - A x
        r_hat.copy_(r)
        p.zero_()
        v.zero_()
        sc.copy_(W["init"])                           # rho_old = alpha = omega = 1

    bw.copy_(b)
    xw.copy_(x)
    restart()
    thr = (tol * bnorm) ** 2
    hist = []
    converged = False
    it = 0
    while it < max_it:
        it += 1
        slot = it % 2
        graphs[slot].replay()
        W["ev"][slot].record()
        if it == 1:
            continue
        prev = 1 - slot
        W["ev"][prev].synchronize()
        rr = float(W["host"][prev])
        if not math.isfinite(rr):
            break
        hist.append(math.sqrt(max(rr, 0.0)) / bnorm)
        if rr < thr:
            if true_res() < tol:                       # iteration `it` has run too
                converged = True
                break
            restart()
    res = true_res()
    x.copy_(xw)
    return {"converged": converged and res < tol, "it": it, "res_rel": res, "history": hist}


def bicgstab_mg_mixed(mg_solver, b: Tensor, x0: Optional[Tensor] = None, tol: float = 1e-8, max_it: int = 300,
                      inner_tol: float = 1e-4, inner_max: int = 80) -> Tuple[Tensor, dict]:
    """Mixed-precision solve to an FP64 relative residual `tol`: FP64 iterative refinement
    (r = b - A x in FP64, x += e) around an FP32 BiCGSTAB on A e = r / |r| preconditioned by the
    FP32 V-cycle, each inner solve to `inner_tol`.  Only the refinement residuals touch FP64
    arithmetic, which on GB300 runs far below the FP32 rate."""
    lv0 = mg_solver._levels[0]
    mask = lv0["mask_f"]
    V = _vec(mg_solver)
    dev = b.device
    f64 = dict(dtype=torch.float64, device=dev)
    b64 = torch.empty(lv0["shape"], **f64)
    V.convert(b64, b.contiguous(), mask)
    x = torch.zeros(lv0["shape"], **f64)
    if x0 is not None:
        V.convert(x, x0.contiguous(), mask)
    bnorm = math.sqrt(V.dot(b64, b64, 0)) + 1e-300
    r64 = torch.empty_like(x)
    t64 = torch.empty_like(x)
    r32 = torch.empty(lv0["shape"], dtype=torch.float32, device=dev)
    e32 = torch.zeros_like(r32)
    total = 0
    outer = 0
    hist = []
    res = float("inf")
    while True:
        V.mop64(x, r64, b=b64, mask=mask)              # r = b - A x  (FP64)
        rn = math.sqrt(V.dot(r64, r64, 11))
        res = rn / bnorm
        hist.append(res)
        if res < tol or total >= max_it or not math.isfinite(res) or outer >= 12:
            break
        V.convert(r32, r64, mask, scale=1.0 / rn)      # unit right-hand side in FP32
        e32.zero_()
        info = _bicg_solve(mg_solver, V, r32, e32, 1.0, inner_tol, min(inner_max, max_it - total), mask)
        total += info["it"]
        V.convert(t64, e32, mask, scale=rn)
        V.axpby(x, t64, 1.0)                            # x += e
        outer += 1
    return x, {"converged": res < tol, "it": total, "outer": outer, "res_rel": res, "history": hist}


def _true_res(V: _Vec, x64, b64, mask, tmp64) -> float:
    V.mop64(x64, tmp64, b=b64, mask=mask)
    return math.sqrt(V.dot(tmp64, tmp64, 10))


def bicgstab_mg_f64(mg_solver, b: Tensor, x0: Optional[Tensor] = None, tol: float = 1e-8, max_it: int = 200,
                    precond: Optional[Callable] = None) -> Tuple[Tensor, dict]:
    """Right-preconditioned BiCGSTAB on FP64 vectors; stops on the true FP64 relative residual."""
    lv0 = mg_solver._levels[0]
    mask = lv0["mask_f"]
    V = _vec(mg_solver)
    M = precond or _vcycle_pc(mg_solver)
    f64 = dict(dtype=torch.float64, device=b.device)
    b64 = torch.empty(lv0["shape"], **f64)
    V.convert(b64, b.contiguous(), mask)
    x = torch.zeros(lv0["shape"], **f64)
    if x0 is not None:
        V.convert(x, x0.contiguous(), mask)
    bnorm = math.sqrt(V.dot(b64, b64, 0)) + 1e-300
    if precond is None and b.is_cuda:
        info = _bicg_solve(mg_solver, V, b64, x, bnorm, tol, max_it, mask)
        return x, info
    r = torch.empty_like(x)
    V.mop64(x, r, b=b64, mask=mask)
    r_hat = r.clone()
    p = torch.zeros_like(x)
    v = torch.zeros_like(x)
    ph = torch.empty_like(x)
    sh = torch.empty_like(x)
    t = torch.empty_like(x)
    rho = alpha = omega = 1.0
    hist = []
    converged = False
    it = 0
    for it in range(1, max_it + 1):
        rho_new = V.dot(r_hat, r, 1)
        if abs(rho_new) < 1e-300:
            break
        beta = (rho_new / rho) * (alpha / omega) if it > 1 else 0.0
        V.axpby(p, v, -omega)                       # p -= omega v
        V.axpby(p, r, 1.0, beta)                    # p = r + beta p
        M(p, ph)
        V.mop64(ph, v, mask=mask)
        alpha = rho_new / V.dot(r_hat, v, 2)
        V.axpby(r, v, -alpha)                       # r becomes s
        V.axpby(x, ph, alpha)
        s_norm = math.sqrt(V.dot(r, r, 3)) / bnorm
        if s_norm < tol:
            res = _true_res(V, x, b64, mask, t) / bnorm
            hist.append(res)
            if res < tol:
                converged = True
                break
        M(r, sh)
        V.mop64(sh, t, mask=mask)
        tt = V.dot(t, t, 4)
        omega = V.dot(t, r, 5) / tt if tt > 0 else 0.0
        V.axpby(x, sh, omega)
        V.axpby(r, t, -omega)
        rho = rho_new
        res = math.sqrt(V.dot(r, r, 6)) / bnorm
        hist.append(res)
        if res < tol:
            res = _true_res(V, x, b64, mask, t) / bnorm
            if res < tol:
                converged = True
                break
            V.mop64(x, r, b=b64, mask=mask)          # restart from the true residual
            r_hat.copy_(r)
            p.zero_()
            v.zero_()
            rho = alpha = omega = 1.0
        if omega == 0.0 or not math.isfinite(res):
            break
    res = _true_res(V, x, b64, mask, t) / bnorm
    return x, {"converged": converged and res < tol, "it": it, "res_rel": res, "history": hist}


def fgmres_mg_f64(mg_solver, b: Tensor, x0: Optional[Tensor] = None, tol: float = 1e-8, max_it: int = 200,
                  restart: int = 30, precond: Optional[Callable] = None,
                  stall_fallback: Optional[Callable] = None, stall_window: int = 1) -> Tuple[Tensor, dict]:
    """Flexible GMRES(restart) on FP64 vectors with a right preconditioner r -> z.

    `precond(r64, z64)` may change between applications.  When `stall_fallback`
    is given, a residual that drops by less than 10 % over `stall_window`
    consecutive inner iterations switches the remaining iterations to that
    preconditioner (the plain V-cycle); `fell_back_at` in the result is the
    iteration where that happened."""
    lv0 = mg_solver._levels[0]
    mask = lv0["mask_f"]
    V = _vec(mg_solver)
    M = precond or _vcycle_pc(mg_solver)
    f64 = dict(dtype=torch.float64, device=b.device)
    shape = lv0["shape"]
    b64 = torch.empty(shape, **f64)
    V.convert(b64, b.contiguous(), mask)
    x = torch.zeros(shape, **f64)
    if x0 is not None:
        V.convert(x, x0.contiguous(), mask)
    bnorm = math.sqrt(V.dot(b64, b64, 0)) + 1e-300
    m = int(restart)
    Vb = torch.zeros((m + 1,) + tuple(shape), **f64)
    Zb = torch.zeros((m,) + tuple(shape), **f64)
    w = torch.empty(shape, **f64)
    total = 0
    hist = []
    fell_back = False
    fell_back_at = None
    converged = False
    w_stall = max(1, int(stall_window))
    while total < max_it:
        V.mop64(x, Vb[0], b=b64, mask=mask)
        beta = math.sqrt(V.dot(Vb[0], Vb[0], 1))
        res = beta / bnorm
        hist.append(res)
        if res < tol:
            converged = True
            break
        V.axpby(Vb[0], Vb[0], 0.0, 1.0 / beta)
        H = [[0.0] * m for _ in range(m + 1)]
        cs, sn = [0.0] * m, [0.0] * m
        g = [0.0] * (m + 1)
        g[0] = beta
        j_done = 0
        for j in range(m):
            if total >= max_it:
                break
            M(Vb[j], Zb[j])
            V.mop64(Zb[j], w, mask=mask)
            for i in range(j + 1):                       # modified Gram-Schmidt
                hij = V.dot(w, Vb[i], 2)
                H[i][j] = hij
                V.axpby(w, Vb[i], -hij)
            hn = math.sqrt(V.dot(w, w, 3))
            H[j + 1][j] = hn
            if hn > 0:
                V.axpby(Vb[j + 1], w, 1.0 / hn, 0.0)
            for i in range(j):                           # apply previous rotations
                a, c = H[i][j], H[i + 1][j]
                H[i][j] = cs[i] * a + sn[i] * c
                H[i + 1][j] = -sn[i] * a + cs[i] * c
            a, c = H[j][j], H[j + 1][j]
            d = math.hypot(a, c)
            cs[j], sn[j] = (a / d, c / d) if d > 0 else (1.0, 0.0)
            H[j][j] = cs[j] * a + sn[j] * c
            H[j + 1][j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            total += 1
            j_done = j + 1
            est = abs(g[j + 1]) / bnorm
            hist.append(est)
            if est < tol or hn == 0:
                break
            if (stall_fallback is not None and not fell_back and j >= max(2, w_stall)
                    and est > 0.9 * hist[-1 - w_stall]):
                M = stall_fallback
                fell_back = True
                fell_back_at = total
        # x += Z y with H y = g
        y = [0.0] * j_done
        for i in range(j_done - 1, -1, -1):
            s = g[i] - sum(H[i][k] * y[k] for k in range(i + 1, j_done))
            y[i] = s / H[i][i] if H[i][i] != 0 else 0.0
        for i in range(j_done):
            V.axpby(x, Zb[i], y[i])
        if hist and hist[-1] < tol:
            tmp = w
            res = _true_res(V, x, b64, mask, tmp) / bnorm
            if res < tol:
                converged = True
                hist.append(res)
                break
    res = _true_res(V, x, b64, mask, w) / bnorm
    return x, {"converged": converged and res < tol, "it": total, "res_rel": res, "history": hist,
               "fell_back": fell_back, "fell_back_at": fell_back_at}
