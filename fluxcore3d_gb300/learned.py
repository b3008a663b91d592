"""Learned preconditioner for the thermal solve: a 3-level 3-D convolutional U-Net
(16/32/64 channels, 3x3x3 kernels, BF16 weights and activations, FP32
accumulation) that maps (residual, conductivity field) to an error estimate and
replaces the V-cycle as the preconditioner inside flexible GMRES.  Forward and
backward run entirely on the tcgen05 implicit-GEMM kernels and the glue kernels
of libfluxcore3d_gb300.so; training uses Adam on FP32 master weights.

The network has no biases, so with ReLU activations it is positively
homogeneous; the residual is additionally normalised by its RMS per sample and
the output rescaled, so z(a r) = a z(r) for a > 0.  Conductivity enters as
(log k - k_shift) * k_scale.

The reference solver has no learned component; the plain geometric multigrid
remains the fallback inside fgmres_mg_f64 (`stall_fallback`) and the arbiter of
convergence (the FP64 true residual).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._torch import ptr, stream_ptr

# (name, C_in, C_out, ReLU) in forward order; C_in of "a" is the 8-channel packed input
SPEC = (("a", 8, 16, True), ("b", 16, 16, True), ("c", 16, 32, True), ("d", 32, 32, True),
        ("e", 32, 64, True), ("f", 64, 64, True), ("g", 96, 32, True), ("h", 32, 32, True),
        ("i", 48, 16, True), ("j", 16, 16, False))
K_SHIFT = 0.0
K_SCALE = 0.25
INPUT_REAL_CHANNELS = 2


def kpad_of(cin: int) -> int:
    return ((27 * cin + 63) // 64) * 64


@dataclass
class _Layer:
    name: str
    cin: int
    cout: int
    relu: bool
    kpad: int
    w: torch.Tensor       # FP32 master [cout, kpad]
    wb: torch.Tensor      # BF16 copy
    m: torch.Tensor
    v: torch.Tensor
    g: torch.Tensor       # FP32 gradient [cout, kpad]


class UNetPreconditioner:
    def __init__(self, device="cuda", seed: int = 0, zero_last: bool = False):
        """zero_last: the output layer starts at zero, so the untrained network returns 0 (inside
        LearnedCorrection the preconditioner is then exactly the V-cycle) and training grows the
        correction from there instead of first shrinking a random output of the wrong scale."""
        self.device = torch.device(device)
        gen = torch.Generator().manual_seed(seed)
        self.layers = []
        for name, cin, cout, relu in SPEC:
            kp = kpad_of(cin)
            fan_in = 27 * (INPUT_REAL_CHANNELS if name == "a" else cin)
            std = math.sqrt(2.0 / fan_in) if relu else math.sqrt(1.0 / fan_in)
            if zero_last and name == SPEC[-1][0]:
                std = 0.0
            w = torch.zeros((cout, kp), dtype=torch.float32)
            w3 = torch.randn((cout, 27, cin), generator=gen) * std
            if name == "a":
                w3[:, :, INPUT_REAL_CHANNELS:] = 0.0
            w[:, :27 * cin] = w3.reshape(cout, 27 * cin)
            w = w.to(self.device)
            self.layers.append(_Layer(name, cin, cout, relu, kp, w, w.to(torch.bfloat16).contiguous(),
                                      torch.zeros_like(w), torch.zeros_like(w), torch.zeros_like(w)))
        self.L = {l.name: l for l in self.layers}
        self.step_count = 0
        self.dev_err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._ws = {}

    # ------------------------------------------------------------------ utils
    def master_weights(self):
        """FP32 weights reshaped [C_out, 27, C_in] (views for the gradient checks)."""
        return [l.w[:, :27 * l.cin].reshape(l.cout, 27, l.cin) for l in self.layers]

    def _buf(self, key, shape, dtype):
        t = self._ws.get(key)
        if t is None or t.shape != torch.Size(shape) or t.dtype != dtype:
            t = torch.empty(shape, dtype=dtype, device=self.device)
            self._ws[key] = t
        return t

    def _conv(self, x, layer: _Layer, shape, out_f32=False, key=None):
        B, D, H, W = shape
        yb = self._buf(("y", key or layer.name, B, D), (B, D, H, W, layer.cout), torch.bfloat16)
        yf = self._buf(("yf", key or layer.name, B, D), (B, D, H, W, layer.cout), torch.float32) if out_f32 else None
        _lib.call("fc_conv3d_fwd", ptr(x), ptr(layer.wb), None, B, D, H, W, layer.cin, layer.cout, layer.kpad,
                  int(layer.relu), ptr(yf), ptr(yb), ptr(self.dev_err), stream_ptr())
        return yb, yf

    def _scales(self, r):
        B = r.shape[0]
        rms = torch.sqrt(torch.mean(r.reshape(B, -1).double() ** 2, dim=1)).float() + 1e-30
        return rms, (1.0 / rms).contiguous()

    # ---------------------------------------------------------------- forward
    def forward(self, r: torch.Tensor, k: torch.Tensor, keep: bool = False):
        """r, k: [B, D, H, W] FP32 (D, H, W multiples of 4).  Returns the FP32 error estimate."""
        B, D, H, W = r.shape
        assert D % 4 == 0 and H % 4 == 0 and W % 4 == 0, "volume extents must be multiples of 4"
        rms, inv = self._scales(r)
        st = stream_ptr()
        x = self._buf(("x", B, D), (B, D, H, W, 8), torch.bfloat16)
        _lib.call("fc_nn_pack_input", ptr(r.contiguous()), ptr(k.contiguous()), ptr(inv), D * H * W, B * D * H * W,
                  K_SHIFT, K_SCALE, ptr(x), st)
        s0, s1, s2 = (B, D, H, W), (B, D // 2, H // 2, W // 2), (B, D // 4, H // 4, W // 4)
        L = self.L
        ya, _ = self._conv(x, L["a"], s0)
        yb, _ = self._conv(ya, L["b"], s0)
        p0 = self._buf(("p0", B, D), s1 + (16,), torch.bfloat16)
        _lib.call("fc_nn_avgpool2", ptr(yb), *s0, 16, ptr(p0), st)
        yc, _ = self._conv(p0, L["c"], s1)
        yd, _ = self._conv(yc, L["d"], s1)
        p1 = self._buf(("p1", B, D), s2 + (32,), torch.bfloat16)
        _lib.call("fc_nn_avgpool2", ptr(yd), *s1, 32, ptr(p1), st)
        ye, _ = self._conv(p1, L["e"], s2)
        yf, _ = self._conv(ye, L["f"], s2)
        u1 = self._buf(("u1", B, D), s1 + (96,), torch.bfloat16)
        _lib.call("fc_nn_upsample_concat", ptr(yf), 64, ptr(yd), 32, *s1, ptr(u1), st)
        yg, _ = self._conv(u1, L["g"], s1)
        yh, _ = self._conv(yg, L["h"], s1)
        u0 = self._buf(("u0", B, D), s0 + (48,), torch.bfloat16)
        _lib.call("fc_nn_upsample_concat", ptr(yh), 32, ptr(yb), 16, *s0, ptr(u0), st)
        yi, _ = self._conv(u0, L["i"], s0)
        _, yj = self._conv(yi, L["j"], s0, out_f32=True)
        if keep:
            self._saved = dict(x=x, ya=ya, yb=yb, p0=p0, yc=yc, yd=yd, p1=p1, ye=ye, yf=yf, u1=u1, yg=yg, yh=yh,
                               u0=u0, yi=yi, yj=yj, shape=(B, D, H, W), rms=rms, inv=inv)
        out = torch.empty((B, D, H, W), dtype=torch.float32, device=self.device)
        _lib.call("fc_nn_take_channel0", ptr(yj), 16, ptr(rms), D * H * W, B * D * H * W, None, ptr(out), st)
        return out

    # --------------------------------------------------------------- backward
    def _wgrad(self, x, g_bf16, layer: _Layer, shape):
        B, D, H, W = shape
        splits = max(1, min(64, (B * D * H * W) // 8192))
        nb = int(_lib.call("fc_conv3d_wgrad_workspace_bytes", B, D, H, W, layer.cin, layer.cout, splits))
        ws = self._buf(("wg", nb), (nb,), torch.uint8)
        _lib.call("fc_conv3d_wgrad", ptr(x), ptr(g_bf16), B, D, H, W, layer.cin, layer.cout, layer.kpad, splits,
                  ptr(ws), nb, ptr(layer.g), ptr(self.dev_err), stream_ptr())

    def _dgrad(self, g_bf16, layer: _Layer, shape):
        B, D, H, W = shape
        nb = int(_lib.call("fc_conv3d_dgrad_workspace_bytes", layer.cin, layer.cout))
        ws = self._buf(("dg", nb), (nb,), torch.uint8)
        gx = torch.empty((B, D, H, W, layer.cin), dtype=torch.float32, device=self.device)
        _lib.call("fc_conv3d_dgrad", ptr(g_bf16), ptr(layer.wb), B, D, H, W, layer.cin, layer.cout, layer.kpad,
                  ptr(ws), nb, ptr(gx), None, ptr(self.dev_err), stream_ptr())
        return gx

    def _act(self, g, y, relu, add=None):
        n = g.numel()
        gf = torch.empty_like(g)
        gb = torch.empty(g.shape, dtype=torch.bfloat16, device=self.device)
        _lib.call("fc_nn_act_bwd", ptr(g), ptr(add), ptr(y), int(relu), n, ptr(gf), ptr(gb), stream_ptr())
        return gf, gb

    def loss_and_grad(self, r, k, target, relative: bool = False):
        """MSE between the network output and target / rms(r) (the normalised error); fills layer.g.
        With `relative`, each sample's squared error is divided by the mean square of its
        normalised target, so a sample whose error is small next to its residual weighs as much
        as any other (otherwise predicting zero is already a low loss for it).
        Returns (loss, [grad per layer as [C_out, 27, C_in] FP32])."""
        self.forward(r, k, keep=True)
        S = self._saved
        B, D, H, W = S["shape"]
        st = stream_ptr()
        nvox = B * D * H * W
        tn2 = target.reshape(B, -1) * S["inv"][:, None]
        tn = tn2.reshape(-1).contiguous()
        wv = None
        if relative:
            trms = torch.sqrt(torch.mean(tn2.double() ** 2, dim=1)).float() + 1e-30
            wv = (1.0 / trms)[:, None].expand(B, D * H * W).reshape(-1).contiguous()
        gj = torch.empty((B, D, H, W, 16), dtype=torch.float32, device=self.device)
        nb = int(_lib.call("fc_nn_mse_workspace_bytes", nvox))
        ws = self._buf(("mse", nb), (nb,), torch.uint8)
        _lib.call("fc_nn_mse_grad", ptr(S["yj"]), 16, ptr(tn), ptr(wv), nvox, ptr(gj), ptr(ws), nb, st)
        nblk = (nvox + 255) // 256
        loss = float(ws[: nblk * 8].view(torch.float64).sum().item()) / nvox
        return loss, self._backward(gj)

    def residual_loss_and_grad(self, r, k, ops):
        """Residual-norm loss of the correction: for sample b with operator M_b = I + dt L_b
        (ops[b]: dict with the fine level's coefficient pointers `coef` (aE, aW, aN, aS, aU, aD,
        diagL), `dt`, `ax`, `out_idx` and the FP32 `mask`), the normalised residual left by the
        masked output y, rho = mask (r / rms(r) - M (mask y)), relative to the normalised
        right-hand side: loss = mean_b ||rho||^2 / ||r / rms(r)||^2.  Its gradient with respect to y,
        -2 mask M^T rho / ||r / rms(r)||^2, enters the output channel; fills layer.g.
        Returns (loss, [grad per layer as [C_out, 27, C_in] FP32])."""
        self.forward(r, k, keep=True)
        S = self._saved
        B, D, H, W = S["shape"]
        st = stream_ptr()
        gj = torch.zeros_like(S["yj"])
        loss = 0.0
        for b in range(B):
            op = ops[b]
            mask = op["mask"]
            y = (S["yj"][b, ..., 0] * mask).contiguous()
            rhat = (r[b] * S["inv"][b]).contiguous()
            rho = torch.empty_like(rhat)
            _lib.call("fc_mg_mop_f32", ptr(y), *op["coef"], float(op["dt"]), D, H, W, op["ax"], op["out_idx"],
                      ptr(rhat), ptr(mask), ptr(rho), st)
            den = float((rhat.double() ** 2).sum()) + 1e-30
            loss += float((rho.double() ** 2).sum()) / den / B
            g = torch.empty_like(rhat)
            _lib.call("fc_mg_mop_transpose_f32", ptr(rho), *op["coef"][:6], float(op["dt"]), D, H, W, op["ax"],
                      op["out_idx"], ptr(mask), ptr(g), st)
            gj[b, ..., 0] = g * mask * (-2.0 / den / B)
        return loss, self._backward(gj)

    def _backward(self, gj):
        """Back-propagate the gradient gj of the FP32 16-channel output through the saved forward
        pass; fills layer.g and returns the per-layer gradients."""
        S = self._saved
        B, D, H, W = S["shape"]
        s0, s1, s2 = (B, D, H, W), (B, D // 2, H // 2, W // 2), (B, D // 4, H // 4, W // 4)
        st = stream_ptr()
        L = self.L
        _, gjb = self._act(gj, None, False)
        self._wgrad(S["yi"], gjb, L["j"], s0)
        g = self._dgrad(gjb, L["j"], s0)
        _, gib = self._act(g, S["yi"], True)
        self._wgrad(S["u0"], gib, L["i"], s0)
        gu0 = self._dgrad(gib, L["i"], s0)                       # 48 ch at s0
        gh_c = torch.empty(s1 + (32,), dtype=torch.float32, device=self.device)
        ge0_skip = torch.empty(s0 + (16,), dtype=torch.float32, device=self.device)
        _lib.call("fc_nn_upsample_concat_bwd", ptr(gu0), 32, 16, *s0, ptr(gh_c), ptr(ge0_skip), st)
        _, ghb = self._act(gh_c, S["yh"], True)
        self._wgrad(S["yg"], ghb, L["h"], s1)
        g = self._dgrad(ghb, L["h"], s1)
        _, ggb = self._act(g, S["yg"], True)
        self._wgrad(S["u1"], ggb, L["g"], s1)
        gu1 = self._dgrad(ggb, L["g"], s1)                       # 96 ch at s1
        gf_c = torch.empty(s2 + (64,), dtype=torch.float32, device=self.device)
        ge1_skip = torch.empty(s1 + (32,), dtype=torch.float32, device=self.device)
        _lib.call("fc_nn_upsample_concat_bwd", ptr(gu1), 64, 32, *s1, ptr(gf_c), ptr(ge1_skip), st)
        _, gfb = self._act(gf_c, S["yf"], True)
        self._wgrad(S["ye"], gfb, L["f"], s2)
        g = self._dgrad(gfb, L["f"], s2)
        _, geb = self._act(g, S["ye"], True)
        self._wgrad(S["p1"], geb, L["e"], s2)
        gp1 = self._dgrad(geb, L["e"], s2)                       # 32 ch at s2
        ge1_pool = torch.empty(s1 + (32,), dtype=torch.float32, device=self.device)
        _lib.call("fc_nn_avgpool2_bwd", ptr(gp1), *s1, 32, ptr(ge1_pool), st)
        _, gdb = self._act(ge1_skip, S["yd"], True, add=ge1_pool)
        self._wgrad(S["yc"], gdb, L["d"], s1)
        g = self._dgrad(gdb, L["d"], s1)
        _, gcb = self._act(g, S["yc"], True)
        self._wgrad(S["p0"], gcb, L["c"], s1)
        gp0 = self._dgrad(gcb, L["c"], s1)                       # 16 ch at s1
        ge0_pool = torch.empty(s0 + (16,), dtype=torch.float32, device=self.device)
        _lib.call("fc_nn_avgpool2_bwd", ptr(gp0), *s0, 16, ptr(ge0_pool), st)
        _, gbb = self._act(ge0_skip, S["yb"], True, add=ge0_pool)
        self._wgrad(S["ya"], gbb, L["b"], s0)
        g = self._dgrad(gbb, L["b"], s0)
        _, gab = self._act(g, S["ya"], True)
        self._wgrad(S["x"], gab, L["a"], s0)
        return [l.g[:, :27 * l.cin].reshape(l.cout, 27, l.cin) for l in self.layers]

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        st = stream_ptr()
        for l in self.layers:
            kvalid = 27 * (INPUT_REAL_CHANNELS if l.name == "a" else l.cin)
            if l.name == "a":
                # only the real input channels train; the padded ones stay zero
                g3 = l.g[:, :27 * l.cin].view(l.cout, 27, l.cin)
                g3[:, :, INPUT_REAL_CHANNELS:] = 0.0
                kvalid = 27 * l.cin
            _lib.call("fc_nn_adam", ptr(l.w), ptr(l.g), ptr(l.m), ptr(l.v), ptr(l.wb), l.w.numel(), l.kpad, kvalid,
                      float(lr), beta1, beta2, eps, self.step_count, 1.0, st)

    def check_device_error(self) -> int:
        return int(self.dev_err.item())


class LearnedPreconditioner:
    """Preconditioner callable (r64, z64) for fgmres_mg_f64 on a multigrid solver's fine level."""

    def __init__(self, net: UNetPreconditioner, mg_solver, k_field: torch.Tensor):
        self.net = net
        self.mg = mg_solver
        lv0 = mg_solver._levels[0]
        self.shape = lv0["shape"]
        self.mask = lv0["mask_f"]
        self.k = k_field.reshape((1,) + tuple(self.shape)).float().contiguous()
        self.r32 = torch.empty((1,) + tuple(self.shape), dtype=torch.float32, device=net.device)
        self.calls = 0

    def __call__(self, r64: torch.Tensor, z64: torch.Tensor) -> None:
        n = self.r32.numel()
        st = stream_ptr()
        _lib.call("fc_vec_convert", 1, ptr(self.r32), ptr(r64), n, ptr(self.mask), 1.0, st)
        z = self.net.forward(self.r32, self.k)
        _lib.call("fc_vec_convert", 0, ptr(z64), ptr(z), n, ptr(self.mask), 1.0, st)
        self.calls += 1


class LearnedCorrection:
    """Preconditioner callable (r64, z64) for fgmres_mg_f64: one plain V-cycle, then the network
    applied to what it leaves behind, then `post_smooth` damped-Jacobi sweeps of the fine level:
    z = S(v + N(r - A v)) with v = V(r).

    The V-cycle removes the oscillatory error; the network is trained (learned_bench,
    `correction=True` pairs) on the residual a V-cycle leaves and the exact error that goes with
    it, i.e. on the smooth, long-range part that geometric coarsening handles poorly across the
    conductivity jumps and along the flow.  Like the coarse correction of a two-grid cycle, the
    network's output carries some oscillatory error, which A = I + dt L (dt = 1000) turns into a
    large residual; the sweeps after it remove that part.  Every vector is zero on the Dirichlet
    rows."""

    def __init__(self, net: UNetPreconditioner, mg_solver, k_field: torch.Tensor, post_smooth: int = 0):
        self.net = net
        self.post_smooth = int(post_smooth)
        self.mg = mg_solver
        lv0 = mg_solver._levels[0]
        self.lv0 = lv0
        self.shape = lv0["shape"]
        self.mask = lv0["mask_f"]
        self.k = k_field.reshape((1,) + tuple(self.shape)).float().contiguous()
        self.r1 = torch.empty((1,) + tuple(self.shape), dtype=torch.float32, device=net.device)
        self.calls = 0

    def residual_after_vcycle(self, b32: torch.Tensor) -> torch.Tensor:
        """v = V(b) in lv0['x'] and r1 = b - A v (masked) in self.r1; b32 FP32 masked."""
        mg, lv0 = self.mg, self.lv0
        nx, ny, nz = self.shape
        st = stream_ptr()
        if b32.data_ptr() != lv0["b_buf"].data_ptr():
            lv0["b_buf"].copy_(b32.reshape(self.shape))
        mg._vcycle(0, zero_guess=True)
        _lib.call("fc_mg_mop_f32", ptr(lv0["x"]), *mg._cptrs(lv0), float(mg._dt_cache), nx, ny, nz, mg.ax,
                  lv0["out_idx"], ptr(lv0["b_buf"]), ptr(self.mask), ptr(self.r1), st)
        return self.r1

    def __call__(self, r64: torch.Tensor, z64: torch.Tensor) -> None:
        lv0 = self.lv0
        n = self.r1.numel()
        st = stream_ptr()
        _lib.call("fc_vec_convert", 1, ptr(lv0["b_buf"]), ptr(r64), n, ptr(self.mask), 1.0, st)
        r1 = self.residual_after_vcycle(lv0["b_buf"])
        y = self.net.forward(r1, self.k)
        # x += y (masked), smoothing sweeps on A x = r, then z = x in FP64
        _lib.call("fc_vec_axpby", 0, ptr(lv0["x"]), ptr(y), n, 1.0, None, None, 1.0, ptr(self.mask), st)
        if self.post_smooth > 0:
            self.mg._smooth_n(0, self.post_smooth)
        _lib.call("fc_vec_convert", 0, ptr(z64), ptr(lv0["x"]), n, ptr(self.mask), 1.0, st)
        self.calls += 1
