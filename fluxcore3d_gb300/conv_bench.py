"""Throughput of the tcgen05 implicit-GEMM 3-D convolution (fc_conv3d_fwd).

Each case is one forward launch of a 3x3x3 convolution, channels-last BF16
activations and weights, FP32 accumulation in TMEM, BF16 output with ReLU.
FLOPs per launch = 2 * 27 * C_in * C_out * voxels (the algorithmic count; the
padded K columns and the zero halo are not counted).  Device time is the mean
of back-to-back launches between CUDA events after warm-up; the inputs are
random and resident.  The shapes are the learned preconditioner's layers at its
64^3 evaluation size and one wider layer.
"""
from __future__ import annotations

import torch

from . import _lib
from ._torch import ptr, stream_ptr
from .learned import kpad_of

CASES = (
    ("64^3, 16 -> 16", (1, 64, 64, 64), 16, 16),
    ("32^3, 32 -> 64", (1, 32, 32, 32), 32, 64),
    ("64^3, 64 -> 64", (1, 64, 64, 64), 64, 64),
    ("64^3, 128 -> 128", (1, 64, 64, 64), 128, 128),
)


def run_case(dev, shape, cin, cout, iters=20):
    B, D, H, W = shape
    g = torch.Generator(device="cpu").manual_seed(cin * 1000 + cout)
    x = torch.randn((B, D, H, W, cin), generator=g).to(dev, torch.bfloat16).contiguous()
    kp = kpad_of(cin)
    w = torch.zeros((cout, kp), dtype=torch.float32)
    w[:, :27 * cin] = torch.randn((cout, 27 * cin), generator=g) * (2.0 / (27 * cin)) ** 0.5
    wb = w.to(dev, torch.bfloat16).contiguous()
    y = torch.empty((B, D, H, W, cout), dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)

    def launch():
        _lib.call("fc_conv3d_fwd", ptr(x), ptr(wb), None, B, D, H, W, cin, cout, kp, 1, None, ptr(y), ptr(err),
                  stream_ptr())

    for _ in range(3):
        launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        launch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    flops = 2.0 * 27 * cin * cout * B * D * H * W
    if int(err.item()) != 0:
        raise RuntimeError(f"fc_conv3d_fwd device error {int(err.item())}")
    return ms, flops


def run(dev, bf16_peak_tflops=None):
    out = []
    for name, shape, cin, cout in CASES:
        ms, flops = run_case(dev, shape, cin, cout)
        tf = flops / (ms / 1e3) / 1e12
        row = {"case": name, "ms": round(ms, 4), "tflops": round(tf, 1)}
        if bf16_peak_tflops:
            row["frac_of_bf16_peak"] = round(tf / bf16_peak_tflops, 4)
        out.append(row)
    return out


if __name__ == "__main__":
    import json
    from . import _build
    _build.build()
    print(json.dumps(run(torch.device("cuda"))))
