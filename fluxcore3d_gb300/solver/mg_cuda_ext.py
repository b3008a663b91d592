"""Drop-in replacement for the reference's solver/mg_cuda_ext.py (:24-66).

`MG_CUDA.mop_fused(T, aE, aW, aN, aS, aU, aD, diagL, Lo, dt, ax, out_idx) -> Lo`
and `MG_CUDA.jacobi_smooth(x, b, Lo, inv_diagM)` keep the reference signatures
(solver/mg_kernels.cu:133-205) and run the sm_103a kernels of
libfluxcore3d_gb300.so.  `MG_CUDA_AVAILABLE` is False only when the native
library or CUDA is missing, in which case every call raises.
"""
from __future__ import annotations

import torch

from .. import _lib
from .._torch import ptr, require, stream_ptr


class _MGKernels:
    def mop_fused(self, T, aE, aW, aN, aS, aU, aD, diagL, Lo, dt, ax, out_idx):
        require(T, "T", torch.float32)
        nx, ny, nz = T.shape
        for t, n in ((aE, "aE"), (aW, "aW"), (aN, "aN"), (aS, "aS"), (aU, "aU"), (aD, "aD"),
                     (diagL, "diagL"), (Lo, "Lo")):
            require(t, n, torch.float32, T.numel())
        _lib.call("fc_mg_mop", ptr(T), ptr(aE), ptr(aW), ptr(aN), ptr(aS), ptr(aU), ptr(aD), ptr(diagL), ptr(Lo),
                  float(dt), int(nx), int(ny), int(nz), int(ax), int(out_idx), stream_ptr())
        return Lo

    def jacobi_smooth(self, x, b, Lo, inv_diagM):
        require(x, "x", torch.float32)
        for t, n in ((b, "b"), (Lo, "Lo"), (inv_diagM, "inv_diagM")):
            require(t, n, torch.float32, x.numel())
        _lib.call("fc_mg_jacobi", ptr(x), ptr(b), ptr(Lo), ptr(inv_diagM), x.numel(), stream_ptr())


MG_CUDA = _MGKernels()
MG_CUDA_AVAILABLE = torch.cuda.is_available() and _lib.load_error() is None
