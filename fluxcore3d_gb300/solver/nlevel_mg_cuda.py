"""Drop-in replacement for the reference's solver/nlevel_mg_cuda.py.

NLevelGeometricMGSolver keeps the reference constructor, public methods and the
private members other modules use (`_levels[l]` keys x, r, b_buf, Lo, mask_f,
inv_diagM, diagL, aE..aD, shape, out_idx; `_vcycle`, `_Mop`, `_ready`,
`_dt_cache`), solver/nlevel_mg_cuda.py:38-537.  The system is
A theta = b with A = I + dt L, L the harmonic-mean diffusion + first-order
upwind convection operator; coarse levels are re-discretised from 2x
mean-restricted fields; the smoother is damped Jacobi; the coarsest level gets
n_coarse sweeps; the coarse correction is added with weight 0.75.

Every operation runs in libfluxcore3d_gb300.so; the V-cycle uses fused
kernels (one pass per Jacobi sweep, residual fused with restriction,
prolongation fused with the correction and mask, zero-guess first sweep).
The residual norm of `solve` is accumulated in FP64.  The per-level neighbour
buffers of the reference's torch fallback are not allocated.

Extra constructor options: max_levels (None = coarsen until the smallest
half-extent is <= min_coarse_cells, as the reference does) and coarse_solve:
"jacobi" (default, the reference's n_coarse damped-Jacobi sweeps in FP32) or
"fp64" (the coarsest level solved exactly in FP64: its operator is assembled
and inverted on the device whenever the hierarchy or dt changes, and every
V-cycle applies the inverse as an FP64 matrix-vector product; levels of at
most 4096 cells).
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch

from .. import _lib
from .._torch import ptr, require, stream_ptr

Tensor = torch.Tensor

try:
    from .mg_cuda_ext import MG_CUDA, MG_CUDA_AVAILABLE  # noqa: F401
except ImportError:  # pragma: no cover
    MG_CUDA, MG_CUDA_AVAILABLE = None, False


class NLevelGeometricMGSolver:
    def __init__(self, device, dtype, flow_axis: int, flow_sign: int, thermal_dt_scale: float,
                 omega: float = 0.8, n_pre: int = 2, n_post: int = 2, n_coarse: int = 20,
                 min_coarse_cells: int = 4, max_levels: Optional[int] = None, coarse_solve: str = "jacobi"):
        self.device = torch.device(device)
        self.dtype = dtype
        self.ax = int(flow_axis)
        self.sign = int(flow_sign)
        self.s = float(thermal_dt_scale)
        self.omega = float(omega)
        self.n_pre = int(n_pre)
        self.n_post = int(n_post)
        self.n_coarse = int(n_coarse)
        self.min_coarse_cells = int(min_coarse_cells)
        self.max_levels = max_levels
        if coarse_solve not in ("jacobi", "fp64"):
            raise ValueError("coarse_solve must be 'jacobi' or 'fp64'")
        self.coarse_solve = coarse_solve
        self._coarse_inv = None
        self._ready = False
        self._dt_cache: Optional[float] = None
        self._shape_cache: Optional[tuple] = None
        self._levels: list = []
        self._nlevels = 0
        self._use_cuda_ext = True
        if self.device.type != "cuda":
            raise RuntimeError("NLevelGeometricMGSolver: fluxcore3d_gb300 runs on CUDA devices only")
        if dtype != torch.float32:
            raise RuntimeError("NLevelGeometricMGSolver: the multigrid levels are FP32 "
                               "(FP64 certification runs in mg_pcg)")
        _lib.lib()
        self._ws = None
        self._scalar = torch.zeros(4, dtype=torch.float64, device=self.device)

    # ------------------------------------------------------------ public API
    def build_if_needed(self, k, rho_cp, u, v, w, mask, dt) -> None:
        shape = tuple(k.shape)
        dt = float(dt)
        if not self._ready or self._shape_cache != shape:
            self._build_hierarchy(k, rho_cp, u, v, w, mask)
            self._dt_cache = None
        if self._dt_cache != dt:
            self._update_inv_diag(dt)
            self._dt_cache = dt

    def solve(self, b: Tensor, x0: Optional[Tensor] = None, max_cycles: int = 50,
              tol: float = 1e-6) -> Tuple[Tensor, dict]:
        assert self._ready, "Call build_if_needed() before solve()."
        lv0 = self._levels[0]
        mask_f = lv0["mask_f"]
        n = mask_f.numel()
        st = stream_ptr()
        if x0 is not None:
            _lib.call("fc_vec_convert", 2, ptr(lv0["x"]), ptr(x0.contiguous().to(torch.float32)), n, ptr(mask_f),
                      1.0, st)
        else:
            lv0["x"].zero_()
        _lib.call("fc_vec_convert", 2, ptr(lv0["b_buf"]), ptr(b.contiguous().to(torch.float32)), n, ptr(mask_f),
                  1.0, st)
        b_norm = self._norm(b.contiguous().to(torch.float32)) + 1e-30
        res_rel = float("inf")
        res0_rel = float("inf")
        converged = False
        cyc = 0
        for cyc in range(max_cycles):
            self._vcycle(0)
            res_rel = self._residual_norm(0, masked=False) / b_norm
            if cyc == 0:
                res0_rel = res_rel
            if not (res_rel < float("inf")):
                converged = False
                break
            if cyc > 2 and res_rel > 10.0 * res0_rel:
                converged = False
                break
            if res_rel < tol:
                converged = True
                break
        result = torch.empty_like(lv0["x"])
        _lib.call("fc_vec_convert", 2, ptr(result), ptr(lv0["x"]), n, ptr(mask_f), 1.0, stream_ptr())
        diverged = (not converged) and (not (res_rel < float("inf")) or (cyc > 2 and res_rel > 10.0 * res0_rel))
        return result, {"converged": converged, "diverged": diverged, "it": cyc + 1,
                        "res_rel": res_rel, "res0_rel": res0_rel}

    def L_apply_fine(self, T: Tensor) -> Tensor:
        """L_steady(T) at the fine level, as (M(T) - T) / dt (new tensor)."""
        assert self._ready
        lv = self._levels[0]
        T = T.contiguous()
        require(T, "T", torch.float32, lv["mask_f"].numel())
        out = torch.empty_like(T)
        nx, ny, nz = lv["shape"]
        _lib.call("fc_mg_apply_L", ptr(T), *self._cptrs(lv), ptr(out), float(self._dt_cache), nx, ny, nz, self.ax,
                  lv["out_idx"], stream_ptr())
        return out

    # ------------------------------------------------------- hierarchy build
    @staticmethod
    def _cptrs(lv):
        return [ptr(lv[k]) for k in ("aE", "aW", "aN", "aS", "aU", "aD", "diagL")]

    def _out_idx(self, shape):
        n = shape[self.ax]
        return n - 1 if self.sign == +1 else 0

    def _build_hierarchy(self, k, rho_cp, u, v, w, mask) -> None:
        # captured solver graphs bake the level buffers' addresses: every build is a new generation
        self._generation = getattr(self, "_generation", 0) + 1
        self._levels = []
        dev = self.device
        st = stream_ptr()
        fields = [t.to(device=dev, dtype=torch.float32).contiguous() for t in (k, rho_cp, u, v, w)]
        msk = mask.to(device=dev, dtype=torch.float32).contiguous()
        while True:
            nx, ny, nz = fields[0].shape
            shape = (nx, ny, nz)
            out_idx = self._out_idx(shape)
            dx = float(2 ** len(self._levels))
            lv = {"shape": shape, "out_idx": out_idx}
            for key in ("aE", "aW", "aN", "aS", "aU", "aD", "diagL", "inv_diagM", "x", "r", "b_buf", "Lo"):
                lv[key] = torch.empty(shape, device=dev, dtype=torch.float32)
            _lib.call("fc_mg_build_coeffs", *[ptr(t) for t in fields], nx, ny, nz, self.ax, out_idx, dx, self.s,
                      *self._cptrs(lv), st)
            lv["mask_f"] = msk
            self._levels.append(lv)
            if min(nx // 2, ny // 2, nz // 2) <= self.min_coarse_cells:
                break
            if self.max_levels is not None and len(self._levels) >= int(self.max_levels):
                break
            cshape = (nx // 2, ny // 2, nz // 2)
            nf = []
            for t in fields:
                c = torch.empty(cshape, device=dev, dtype=torch.float32)
                _lib.call("fc_mg_restrict_mean", ptr(t), nx, ny, nz, ptr(c), 0, st)
                nf.append(c)
            cm = torch.empty(cshape, device=dev, dtype=torch.float32)
            _lib.call("fc_mg_restrict_mean", ptr(msk), nx, ny, nz, ptr(cm), 1, st)
            fields, msk = nf, cm
        self._nlevels = len(self._levels)
        self._shape_cache = tuple(k.shape)
        n0 = self._levels[0]["mask_f"].numel()
        nbytes = max(_lib.call("fc_mg_reduce_workspace_bytes", n0), _lib.call("fc_vec_workspace_bytes", n0))
        self._ws = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
        print("[MG] %d-level hierarchy: %s" % (self._nlevels, " -> ".join(str(l["shape"]) for l in self._levels)))

    def _update_inv_diag(self, dt: float) -> None:
        st = stream_ptr()
        for lv in self._levels:
            _lib.call("fc_mg_inv_diag", ptr(lv["diagL"]), ptr(lv["mask_f"]), ptr(lv["inv_diagM"]), float(dt),
                      self.omega, lv["mask_f"].numel(), st)
        if self.coarse_solve == "fp64" and self._nlevels > 1:
            self._build_coarse_inverse(float(dt))
        self._ready = True

    def _build_coarse_inverse(self, dt: float) -> None:
        """FP64 inverse of the coarsest level's A = I + dt L (Dirichlet rows identity)."""
        lv = self._levels[-1]
        nx, ny, nz = lv["shape"]
        need = int(_lib.call("fc_mg_coarse_dense_bytes", nx, ny, nz))
        if need < 0:
            raise ValueError(f"coarse_solve='fp64': the coarsest level {lv['shape']} has more than 4096 cells; "
                             "raise max_levels or use coarse_solve='jacobi'")
        if self._coarse_inv is None or self._coarse_inv.numel() * 8 < need:
            self._coarse_inv = torch.empty((need + 7) // 8, dtype=torch.float64, device=self.device)
        _lib.call("fc_mg_coarse_dense_build", *self._cptrs(lv), ptr(lv["mask_f"]), float(dt), nx, ny, nz, self.ax,
                  lv["out_idx"], ptr(self._coarse_inv), self._coarse_inv.numel() * 8, stream_ptr())

    # ---------------------------------------------------------------- V-cycle
    def _smooth_n(self, level: int, n_sweeps: int, from_zero: bool = False) -> None:
        """n_sweeps damped-Jacobi sweeps on level `level`, ping-ponging between lv['x'] and lv['Lo'];
        the result always ends in lv['x']."""
        if n_sweeps <= 0:
            if from_zero:
                self._levels[level]["x"].zero_()
            return
        lv = self._levels[level]
        nx, ny, nz = lv["shape"]
        dt = float(self._dt_cache)
        st = stream_ptr()
        cp = self._cptrs(lv)
        if nx * ny * nz <= 6144:
            # a small level (the coarsest) runs all its sweeps in one single-CTA launch
            _lib.call("fc_mg_smooth_small", ptr(lv["x"]), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny,
                      nz, self.ax, lv["out_idx"], int(n_sweeps), int(from_zero), st)
            return
        cur, alt = lv["x"], lv["Lo"]
        start = 0
        if from_zero and n_sweeps >= 2:
            # sweeps 1 and 2 from the zero guess in one pass, straight into x (x is not read)
            _lib.call("fc_mg_smooth_first2", ptr(cur), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny, nz,
                      self.ax, lv["out_idx"], st)
            start = 2
        elif from_zero:
            _lib.call("fc_mg_smooth_from_zero", ptr(cur), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), cur.numel(), st)
            start = 1
        for _ in range(start, n_sweeps):
            _lib.call("fc_mg_smooth", ptr(cur), ptr(alt), ptr(lv["b_buf"]), ptr(lv["inv_diagM"]), *cp, dt, nx, ny,
                      nz, self.ax, lv["out_idx"], st)
            cur, alt = alt, cur
        if cur is not lv["x"]:
            lv["x"].copy_(cur)

    def _vcycle(self, level: int, zero_guess: bool = False) -> None:
        lv = self._levels[level]
        if level == self._nlevels - 1:
            if self.coarse_solve == "fp64" and level > 0:
                _lib.call("fc_mg_coarse_dense_apply", ptr(self._coarse_inv), ptr(lv["b_buf"]), ptr(lv["mask_f"]),
                          ptr(lv["x"]), lv["mask_f"].numel(), stream_ptr())
            else:
                self._smooth_n(level, self.n_coarse, from_zero=zero_guess)
            return
        self._smooth_n(level, self.n_pre, from_zero=zero_guess)
        nx, ny, nz = lv["shape"]
        lvc = self._levels[level + 1]
        cx, cy, cz = lvc["shape"]
        st = stream_ptr()
        _lib.call("fc_mg_residual_restrict", ptr(lv["x"]), ptr(lv["b_buf"]), ptr(lv["mask_f"]), *self._cptrs(lv),
                  float(self._dt_cache), nx, ny, nz, self.ax, lv["out_idx"], ptr(lvc["b_buf"]), cx, cy, cz, st)
        self._vcycle(level + 1, zero_guess=True)
        _lib.call("fc_mg_prolong_correct", ptr(lv["x"]), ptr(lvc["x"]), ptr(lv["mask_f"]), nx, ny, nz, cx, cy, cz,
                  0.75, st)
        self._smooth_n(level, self.n_post)

    # ------------------------------------------------------ operator apply
    def _Mop(self, T: Tensor, level: int) -> None:
        """M(T) = T + dt L(T) into levels[level]['Lo']."""
        self._Mop_cuda(T, level, self._levels[level]["Lo"])

    def _Mop_cuda(self, T: Tensor, level: int, Lo: Tensor) -> None:
        lv = self._levels[level]
        nx, ny, nz = lv["shape"]
        _lib.call("fc_mg_mop", ptr(T.contiguous()), *self._cptrs(lv), ptr(Lo), float(self._dt_cache), nx, ny, nz,
                  self.ax, lv["out_idx"], stream_ptr())

    def _smooth_step(self, x, b, Lo, inv_diagM, mask_f, r) -> None:
        _lib.call("fc_mg_jacobi", ptr(x), ptr(b), ptr(Lo), ptr(inv_diagM), x.numel(), stream_ptr())

    def _residual_norm(self, level: int, masked: bool) -> float:
        lv = self._levels[level]
        nx, ny, nz = lv["shape"]
        _lib.call("fc_mg_residual_norm2", ptr(lv["x"]), ptr(lv["b_buf"]), ptr(lv["mask_f"]) if masked else None,
                  *self._cptrs(lv), float(self._dt_cache), nx, ny, nz, self.ax, lv["out_idx"], ptr(lv["r"]),
                  ptr(self._ws), self._ws.numel(), ptr(self._scalar), stream_ptr())
        return float(self._scalar[0].item()) ** 0.5

    def _norm(self, t: Tensor) -> float:
        _lib.call("fc_vec_dot", 1, ptr(t), ptr(t), t.numel(), None, ptr(self._ws), self._ws.numel(),
                  ptr(self._scalar[1:2]), stream_ptr())
        return float(self._scalar[1].item()) ** 0.5

    # --------------------------------------------------- static helpers
    @staticmethod
    def _restrict_2x(x: Tensor) -> Tensor:
        x = x.to(torch.float32).contiguous()
        nx, ny, nz = x.shape
        out = torch.empty((nx // 2, ny // 2, nz // 2), device=x.device, dtype=torch.float32)
        _lib.call("fc_mg_restrict_mean", ptr(x), nx, ny, nz, ptr(out), 0, stream_ptr())
        return out

    def _restrict_into(self, src: Tensor, dst: Tensor) -> None:
        nx, ny, nz = src.shape
        _lib.call("fc_mg_restrict_mean", ptr(src.contiguous()), nx, ny, nz, ptr(dst), 0, stream_ptr())

    @staticmethod
    def _prolong_2x(xc: Tensor, nx: int, ny: int, nz: int) -> Tensor:
        out = torch.zeros((nx, ny, nz), device=xc.device, dtype=torch.float32)
        ones = torch.ones_like(out)
        cx, cy, cz = xc.shape
        _lib.call("fc_mg_prolong_correct", ptr(out), ptr(xc.contiguous()), ptr(ones), nx, ny, nz, cx, cy, cz, 1.0,
                  stream_ptr())
        return out
