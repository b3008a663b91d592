"""The allocation-free convective outlet entry point, called through the C ABI.

fc_lbm_convective_bc_noalloc serves callers that may not allocate device memory
once their time loop runs (a host that hands out all GPU memory from its own
pre-reserved arena, or a path where an allocation would synchronise the
device).  It must give the same plane, bit for bit, as fc_lbm_convective_bc with a caller
workspace (both run the same three kernels), on calls in a row that go from a
large plane to smaller ones, so that a later call finds the partial sums of an
earlier, larger plane left in the shared fixed array, and it must refuse planes
beyond its fixed capacity.
This file is collected last so a failing run has already run every other test.
"""
import numpy as np
import pytest
import torch

from fluxcore3d_gb300 import _lib
from fluxcore3d_gb300._torch import ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _plane_case(nx, ny, nz, seed):
    g = torch.Generator().manual_seed(seed)
    f = (torch.rand((19, nx * ny * nz), generator=g) * 0.05 + 0.02).cuda()
    solid = (torch.rand(nx * ny * nz, generator=g) < 0.15).to(torch.uint8).cuda()
    return f, solid


def _with_workspace(f, solid, nx, ny, nz, n1, n2):
    nb = int(_lib.call("fc_lbm_convective_workspace_bytes", n1, n2))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    _lib.call("fc_lbm_convective_bc", ptr(f), ptr(solid), nx, ny, nz, 0, nx - 1, nx - 2, -1, 1.0, n1, n2, ptr(ws),
              nb, stream_ptr())


def _no_alloc(f, solid, nx, ny, nz, n1, n2):
    return _lib.lib().fc_lbm_convective_bc_noalloc(ptr(f), ptr(solid), nx, ny, nz, 0, nx - 1, nx - 2, -1, 1.0, n1,
                                                   n2, stream_ptr())


def test_no_alloc_convective_matches_workspace_version_twice(cuda):
    # largest plane first: 18 blocks of partials, then 6, then 1 -- each later call reads only its own slots
    for call, (nx, ny, nz, seed) in enumerate(((9, 64, 70, 2), (12, 40, 36, 1), (5, 10, 12, 3))):
        f_ref, solid = _plane_case(nx, ny, nz, seed)
        f_new = f_ref.clone()
        _with_workspace(f_ref, solid, nx, ny, nz, ny, nz)
        rc = _no_alloc(f_new, solid, nx, ny, nz, ny, nz)
        torch.cuda.synchronize()
        assert rc == 0, f"call {call}: status {rc}"
        a, b = f_new.cpu().numpy(), f_ref.cpu().numpy()
        assert np.array_equal(a, b), f"call {call}: max diff {np.abs(a - b).max()}"
        assert not np.array_equal(b, _plane_case(nx, ny, nz, seed)[0].cpu().numpy())  # the BC changed the plane


def test_no_alloc_convective_rejects_planes_beyond_capacity(cuda):
    cap = int(_lib.lib().fc_lbm_convective_noalloc_max_plane())
    assert cap == 4096 * 256
    f = torch.zeros(19 * 4, device="cuda")
    solid = torch.zeros(4, dtype=torch.uint8, device="cuda")
    # a plane of 1025 x 1025 nodes (pointers are never dereferenced: the size check comes first)
    rc = _lib.lib().fc_lbm_convective_bc_noalloc(ptr(f), ptr(solid), 4, 1025, 1025, 0, 3, 2, -1, 1.0, 1025, 1025,
                                                 stream_ptr())
    assert rc == 4
