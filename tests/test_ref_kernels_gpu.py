"""The device plane kernels and the per-operation MRT-Smagorinsky collision against the
reference's own CUDA kernels (run on the host from their unmodified text by
oracle/build_ref.py; tests/golden/ref_lbm.npz from tests/golden/make_ref_fixtures.py):

  fc_lbm_zou_he_bc          vs lbm_zou_he_bc_kernel                (solver/lbm_kernels.cu:791-969)
  fc_lbm_convective_bc      vs lbm_convective_bc_reduce_kernel +
                               lbm_convective_mass_correct_kernel  (:1170-1344)
  fc_lbm_macro_collide_mrt_smag vs lbm_macro_collide_mrt_smag_kernel (:1018-1117)

Tolerance: 2e-6 of the largest value (FP32 rounding; the convective plane sum is FP64 in a
fixed order here and FP32 with per-block atomics in the reference)."""
import os

import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import _lib
from fluxcore3d_gb300._torch import ptr, stream_ptr

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_lbm.npz")
ZH_CASES = ("inlet_x_low", "outlet_x_high", "inlet_y_high", "outlet_y_low", "outlet_z_low", "inlet_z_low")
CV_CASES = ("x_high", "z_low", "x_high_two_blocks")


def _plane_cells(shape, axis, idx):
    i, j, k = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    flat = (i * shape[1] + j) * shape[2] + k
    return np.take(flat, idx, axis=axis).reshape(-1)


def _close(got, want, tol=2e-6):
    return float(np.abs(got.astype(np.float64) - want).max()) <= tol * float(np.abs(want).max())


@pytest.mark.parametrize("case", ZH_CASES)
def test_zou_he_matches_reference_kernel(cuda, case):
    d = np.load(FIX)
    a = d[f"zh_{case}_args"]
    shape = tuple(int(x) for x in a[:3])
    axis, plane, inter, bct = (int(x) for x in a[3:7])
    f_in = d[f"zh_{case}_in"]
    f = torch.tensor(f_in, device=cuda)
    solid = torch.tensor(d["solid_%dx%dx%d" % shape], device=cuda)
    _lib.call("fc_lbm_zou_he_bc", ptr(f), ptr(solid), *shape, axis, plane, inter, bct, float(a[7]), float(a[8]),
              int(a[9]), stream_ptr())
    got = f.cpu().numpy()
    pc = _plane_cells(shape, axis, plane)
    assert _close(got[:, pc], d[f"zh_{case}_plane"])
    assert np.array_equal(np.delete(got, pc, axis=1), np.delete(f_in, pc, axis=1))


@pytest.mark.parametrize("case", CV_CASES)
def test_convective_matches_reference_kernel(cuda, case):
    d = np.load(FIX)
    a = d[f"cv_{case}_args"]
    shape = tuple(int(x) for x in a[:3])
    axis, o, inter, ucax = (int(x) for x in a[3:7])
    n1, n2 = int(a[8]), int(a[9])
    f_in = d[f"cv_{case}_in"]
    f = torch.tensor(f_in, device=cuda)
    solid = torch.tensor(d["solid_%dx%dx%d" % shape], device=cuda)
    nb = int(_lib.call("fc_lbm_convective_workspace_bytes", n1, n2))
    ws = torch.empty(nb, dtype=torch.uint8, device=cuda)
    _lib.call("fc_lbm_convective_bc", ptr(f), ptr(solid), *shape, axis, o, inter, ucax, float(a[7]), n1, n2, ptr(ws),
              nb, stream_ptr())
    got = f.cpu().numpy()
    pc = _plane_cells(shape, axis, o)
    assert _close(got[:, pc], d[f"cv_{case}_plane"])
    assert np.array_equal(np.delete(got, pc, axis=1), np.delete(f_in, pc, axis=1))


def test_mrt_smagorinsky_matches_reference_kernel(cuda):
    d = np.load(FIX)
    shape = tuple(int(x) for x in d["smag_shape"])
    N = int(np.prod(shape))
    cs2, om0 = (float(x) for x in d["smag_params"])
    f = torch.tensor(d["smag_f"], device=cuda)
    fp = torch.empty_like(f)
    mac = torch.empty((4, N), device=cuda)
    solid = torch.tensor(d["solid_%dx%dx%d" % shape], device=cuda)
    S = torch.tensor(d["smag_S"], device=cuda)
    _lib.call("fc_lbm_macro_collide_mrt_smag", ptr(f), ptr(fp), ptr(mac[0]), ptr(mac[1]), ptr(mac[2]), ptr(mac[3]),
              ptr(solid), ptr(S), cs2, om0, N, stream_ptr())
    assert _close(fp.cpu().numpy(), d["smag_out_fp"])
    for got, want in zip(mac.cpu().numpy(), d["smag_out_macro"]):
        assert _close(got, want)
