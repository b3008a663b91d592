"""tcgen05 implicit-GEMM convolutions and network glue against the float64 oracle.

Inputs are rounded to BF16 first, so the only differences are FP32 accumulation
order: tolerance 1e-4 relative (max-normalised)."""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import _lib
from fluxcore3d_gb300._torch import ptr, stream_ptr
from oracle import conv as oc

pytestmark = pytest.mark.gpu


def kpad_of(cin):
    return ((27 * cin + 63) // 64) * 64


def weights(cout, cin, rng):
    w = rng.standard_normal((cout, 27, cin)).astype(np.float32) * 0.1
    wb = oc.bf16(w)
    kp = kpad_of(cin)
    wt = np.zeros((cout, kp), np.float32)
    wt[:, :27 * cin] = wb.reshape(cout, 27 * cin)
    return wb, torch.tensor(wt, device="cuda").to(torch.bfloat16), kp


def err_rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("cin,cout,shape", [(8, 16, (1, 6, 8, 10)), (16, 32, (2, 8, 6, 12)), (32, 64, (1, 12, 10, 8)),
                                            (48, 16, (1, 8, 8, 8)), (16, 16, (1, 33, 5, 7))])
def test_conv_forward(cuda, cin, cout, shape):
    rng = np.random.default_rng(cin * 7 + cout)
    x = oc.bf16(rng.standard_normal(shape + (cin,)).astype(np.float32))
    wb, wt, kp = weights(cout, cin, rng)
    bias = rng.standard_normal(cout).astype(np.float32)
    X = torch.tensor(x, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    Y = torch.empty(shape + (cout,), device="cuda")
    Yb = torch.empty(shape + (cout,), device="cuda", dtype=torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("fc_conv3d_fwd", ptr(X), ptr(wt), ptr(torch.tensor(bias, device="cuda")), *shape, cin, cout, kp, 1,
              ptr(Y), ptr(Yb), ptr(err), stream_ptr())
    torch.cuda.synchronize()
    assert int(err) == 0
    ref = oc.conv_fwd(x, wb, bias, relu=True)
    assert err_rel(Y.cpu().numpy(), ref) < 1e-4
    assert err_rel(Yb.float().cpu().numpy(), ref) < 1e-2


@pytest.mark.parametrize("cin,cout,shape", [(16, 32, (1, 8, 6, 10)), (32, 16, (2, 6, 6, 6)), (96, 32, (1, 8, 8, 4))])
def test_conv_dgrad(cuda, cin, cout, shape):
    rng = np.random.default_rng(cin + 3 * cout)
    gy = oc.bf16(rng.standard_normal(shape + (cout,)).astype(np.float32))
    wb, wt, kp = weights(cout, cin, rng)
    GY = torch.tensor(gy, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    ws = torch.empty(int(_lib.call("fc_conv3d_dgrad_workspace_bytes", cin, cout)), dtype=torch.uint8, device="cuda")
    GX = torch.empty(shape + (cin,), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("fc_conv3d_dgrad", ptr(GY), ptr(wt), *shape, cin, cout, kp, ptr(ws), ws.numel(), ptr(GX), None,
              ptr(err), stream_ptr())
    torch.cuda.synchronize()
    assert int(err) == 0
    assert err_rel(GX.cpu().numpy(), oc.conv_dgrad(gy, wb)) < 1e-4


@pytest.mark.parametrize("cin,cout,shape,splits", [(8, 16, (1, 8, 8, 8), 3), (16, 32, (2, 6, 8, 10), 5),
                                                   (32, 64, (1, 8, 6, 8), 1)])
def test_conv_wgrad(cuda, cin, cout, shape, splits):
    rng = np.random.default_rng(cin + cout + splits)
    x = oc.bf16(rng.standard_normal(shape + (cin,)).astype(np.float32))
    gy = oc.bf16(rng.standard_normal(shape + (cout,)).astype(np.float32))
    kp = kpad_of(cin)
    X = torch.tensor(x, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    GY = torch.tensor(gy, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    nb = int(_lib.call("fc_conv3d_wgrad_workspace_bytes", *shape, cin, cout, splits))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    GW = torch.zeros((cout, kp), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("fc_conv3d_wgrad", ptr(X), ptr(GY), *shape, cin, cout, kp, splits, ptr(ws), nb, ptr(GW), ptr(err),
              stream_ptr())
    torch.cuda.synchronize()
    assert int(err) == 0
    ref = oc.conv_wgrad(x, gy).reshape(cout, 27 * cin)
    got = GW.cpu().numpy()
    assert err_rel(got[:, :27 * cin], ref) < 1e-4
    assert np.all(got[:, 27 * cin:] == 0)


def test_network_gradient_matches_finite_differences(cuda):
    """End-to-end gradient of the U-Net loss (GPU backward kernels) against central differences of
    the float64 oracle network on a tiny volume."""
    from fluxcore3d_gb300.learned import K_SCALE, K_SHIFT, SPEC, UNetPreconditioner
    net = UNetPreconditioner(device="cuda", seed=3)
    rng = np.random.default_rng(0)
    B, D = 1, 8
    r = rng.standard_normal((B, D, D, D)).astype(np.float32)
    k = np.exp(rng.standard_normal((B, D, D, D))).astype(np.float32)
    t = rng.standard_normal((B, D, D, D)).astype(np.float32)
    loss, grads = net.loss_and_grad(torch.tensor(r, device="cuda"), torch.tensor(k, device="cuda"),
                                    torch.tensor(t, device="cuda"))
    w64 = [oc.bf16(w.cpu().numpy()) for w in net.master_weights()]
    ref_loss = oc.unet_loss(SPEC, w64, r, k, t, K_SHIFT, K_SCALE)
    assert abs(loss - ref_loss) / abs(ref_loss) < 2e-2
    # directional derivative along a random direction in weight space
    dirs = [rng.standard_normal(w.shape) * 0.01 for w in w64]
    eps = 1e-3
    lp = oc.unet_loss(SPEC, [w + eps * d for w, d in zip(w64, dirs)], r, k, t, K_SHIFT, K_SCALE)
    lm = oc.unet_loss(SPEC, [w - eps * d for w, d in zip(w64, dirs)], r, k, t, K_SHIFT, K_SCALE)
    fd = (lp - lm) / (2 * eps)
    an = sum(float((g.cpu().numpy().astype(np.float64) * d).sum()) for g, d in zip(grads, dirs))
    assert abs(fd - an) / max(abs(fd), 1e-12) < 5e-2, (fd, an)


def test_learned_correction_is_certified_and_measured(cuda):
    """Train the network briefly on the residual a V-cycle leaves, then solve a held-out problem
    with FGMRES preconditioned by V-cycle + network (plain V-cycle fallback on stall) and by the
    V-cycle alone: both reach a 1e-8 FP64 residual, the learned solve is not pathologically longer
    (the fallback bounds it), and what one correction gains over the V-cycle is reported."""
    from fluxcore3d_gb300 import learned_bench as lb
    from fluxcore3d_gb300.learned import UNetPreconditioner
    dev = torch.device("cuda")
    data = lb.generate_pairs(16, 3, 2, 200, dev, correction=True)
    net = UNetPreconditioner(device=dev, seed=1)
    losses, _ = lb.train(net, data, 40)
    assert all(np.isfinite(losses))
    rows = lb.evaluate(net, 32, (2001,), dev, repeats=1, correction=True)
    r = rows[0]
    assert r["plain_res"] < 1e-8 and r["learned_res"] < 1e-8 and r["plain_bicgstab_res"] < 1e-8
    assert r["learned_it"] <= 2 * r["plain_it"] + 10
    q = lb.correction_quality(net, 32, (2001,), dev)[0]
    assert np.isfinite(q["vcycle_plus_net_rel_err"]) and q["vcycle_rel_err"] < 1.0
    print("learned correction:", r, q)
    assert net.check_device_error() == 0


def test_learned_correction_post_smoothing_and_stall_window(cuda):
    """LearnedCorrection(post_smooth=n) is the correction followed by n smoothing sweeps of the fine
    level on the same right-hand side, bit for bit; FGMRES with a windowed stall test converges and
    reports the iteration of its fallback (or None)."""
    from fluxcore3d_gb300 import learned_bench as lb
    from fluxcore3d_gb300.learned import LearnedCorrection, UNetPreconditioner
    from fluxcore3d_gb300.solver import mg_pcg
    dev = torch.device("cuda")
    mg, k, solid = lb.make_problem(16, 300, dev)
    b = lb.random_rhs(16, np.random.default_rng(3), dev, solid)
    net = UNetPreconditioner(device=dev, seed=2)
    lv0 = mg._levels[0]
    mask = lv0["mask_f"]
    r64 = (b.double() * mask.double()).contiguous()
    z0 = torch.zeros_like(r64)
    LearnedCorrection(net, mg, k, post_smooth=0)(r64, z0)
    mg._smooth_n(0, 2)                       # the same sweeps, on the state the correction left
    expect = (lv0["x"].double() * mask.double()).cpu().numpy()
    z2 = torch.zeros_like(r64)
    LearnedCorrection(net, mg, k, post_smooth=2)(r64, z2)
    assert np.array_equal(z2.cpu().numpy(), expect)
    assert not np.array_equal(z2.cpu().numpy(), z0.cpu().numpy())
    pc = LearnedCorrection(net, mg, k, post_smooth=2)
    _, info = mg_pcg.fgmres_mg_f64(mg, b, tol=1e-8, max_it=300, restart=30, precond=pc,
                                   stall_fallback=mg_pcg._vcycle_pc(mg), stall_window=5)
    assert info["converged"] and info["res_rel"] < 1e-8
    assert info["fell_back_at"] is None or info["fell_back_at"] >= 5
    assert info["fell_back"] == (info["fell_back_at"] is not None)
    assert net.check_device_error() == 0
