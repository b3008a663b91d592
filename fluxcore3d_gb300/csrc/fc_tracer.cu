// fc_tracer.cu -- passive scalar tracer advected by the lattice velocity.
//
// fc_tracer_step is one step of TracerField.step (pre_post/tracer_patch.py:55-82)
// in one pass: first-order upwind differences along each axis with periodic
// neighbours (torch.roll), phi - (u*ax + v*ay + w*az) clamped to [0, 1], scaled by
// the dissipation factor, zero in flow-solid cells.  Each operation is rounded as
// the reference's elementwise tensor operations are, so the field is the
// reference's bit for bit; the reference's ~20 tensor operations per step become
// one read of phi (7-point stencil, neighbours from cache), u, v, w and the flag
// byte and one write (21 B per cell).
// fc_tracer_inject sets phi = 1 on the injection cells (TracerField.inject, :51-53).
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

__global__ void __launch_bounds__(256)
k_tracer_step(const float* __restrict__ phi, float* __restrict__ out, const float* __restrict__ u,
              const float* __restrict__ v, const float* __restrict__ w, const uint8_t* __restrict__ solid, int nx,
              int ny, int nz, float diss) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= nz) return;
    const long long nyz = (long long)ny * nz;
    const long long c = (long long)i * nyz + (long long)j * nz + k;
    const float p = phi[c];
    const int im = i ? i - 1 : nx - 1, ip = i + 1 < nx ? i + 1 : 0;
    const int jm = j ? j - 1 : ny - 1, jp = j + 1 < ny ? j + 1 : 0;
    const int km = k ? k - 1 : nz - 1, kp = k + 1 < nz ? k + 1 : 0;
    const long long row = (long long)j * nz + k, col = (long long)i * nyz + k, pil = (long long)i * nyz + (long long)j * nz;
    const float uc = u[c], vc = v[c], wc = w[c];
    const float ax = uc >= 0.0f ? __fsub_rn(p, phi[im * nyz + row]) : __fsub_rn(phi[ip * nyz + row], p);
    const float ay = vc >= 0.0f ? __fsub_rn(p, phi[col + (long long)jm * nz]) : __fsub_rn(phi[col + (long long)jp * nz], p);
    const float az = wc >= 0.0f ? __fsub_rn(p, phi[pil + km]) : __fsub_rn(phi[pil + kp], p);
    const float s = __fadd_rn(__fadd_rn(__fmul_rn(uc, ax), __fmul_rn(vc, ay)), __fmul_rn(wc, az));
    float n = __fsub_rn(p, s);
    if (!isnan(n)) n = fminf(fmaxf(n, 0.0f), 1.0f);   // torch.clamp keeps NaN
    n = __fmul_rn(n, diss);
    out[c] = solid[c] ? 0.0f : n;
}

__global__ void __launch_bounds__(256) k_tracer_inject(float* __restrict__ phi, const uint8_t* __restrict__ mask,
                                                       long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride)
        if (mask[c]) phi[c] = 1.0f;
}

}  // namespace

extern "C" {

int fc_tracer_step(const float* phi, float* phi_out, const float* u, const float* v, const float* w,
                   const uint8_t* solid_flow, int nx, int ny, int nz, float dissipation, void* stream) {
    if (!phi || !phi_out || !u || !v || !w || !solid_flow || nx < 1 || ny < 1 || nz < 1 || phi == phi_out)
        return FC_ERR_ARG;
    if (ny > 65535 || nx > 65535) return FC_ERR_UNSUPPORTED;
    const dim3 grid((unsigned)((nz + 255) / 256), (unsigned)ny, (unsigned)nx);
    k_tracer_step<<<grid, 256, 0, (cudaStream_t)stream>>>(phi, phi_out, u, v, w, solid_flow, nx, ny, nz, dissipation);
    return launch_status();
}

int fc_tracer_inject(float* phi, const uint8_t* mask, long long n, void* stream) {
    if (!phi || !mask || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    long long b = (n + 255) / 256;
    if (b > 152LL * 32) b = 152LL * 32;
    k_tracer_inject<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(phi, mask, n);
    return launch_status();
}

}  // extern "C"
