// fc_nn.cu -- element-wise and pooling kernels around the tcgen05 convolutions of
// the learned thermal preconditioner (channels-last BF16 activations
// [B][D][H][W][C], FP32 gradients).  No counterpart in the reference.
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int BLOCK = 256;
inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }

// input volume: channel 0 = r * inv_scale[b], channel 1 = log(k) normalised, channels 2..7 = 0
__global__ void k_pack_input(const float* __restrict__ r, const float* __restrict__ kf, const float* __restrict__ inv_scale,
                             long long vox_per_b, long long nvox, float k_shift, float k_scale, __nv_bfloat16* __restrict__ out) {
    const long long v = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (v >= nvox) return;
    const long long b = v / vox_per_b;
    const float s = inv_scale ? inv_scale[b] : 1.f;
    __align__(16) __nv_bfloat16 e[8];
    e[0] = __float2bfloat16_rn(r[v] * s);
    e[1] = __float2bfloat16_rn((logf(fmaxf(kf[v], 1e-30f)) - k_shift) * k_scale);
#pragma unroll
    for (int c = 2; c < 8; ++c) e[c] = __float2bfloat16_rn(0.f);
    reinterpret_cast<uint4*>(out)[v] = *reinterpret_cast<uint4*>(e);
}

// 2x2x2 average pooling (even extents)
__global__ void k_avgpool(const __nv_bfloat16* __restrict__ x, int B, int D, int H, int W, int C,
                          __nv_bfloat16* __restrict__ y) {
    const int D2 = D / 2, H2 = H / 2, W2 = W / 2;
    const long long n = (long long)B * D2 * H2 * W2 * C;
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n) return;
    const int c = (int)(t % C);
    long long v = t / C;
    const int w = (int)(v % W2); v /= W2;
    const int h = (int)(v % H2); v /= H2;
    const int d = (int)(v % D2);
    const int b = (int)(v / D2);
    float s = 0.f;
    for (int a = 0; a < 8; ++a) {
        const int dd = 2 * d + (a >> 2), hh = 2 * h + ((a >> 1) & 1), ww = 2 * w + (a & 1);
        s += __bfloat162float(x[((((long long)b * D + dd) * H + hh) * W + ww) * C + c]);
    }
    y[t] = __float2bfloat16_rn(s * 0.125f);
}

__global__ void k_avgpool_bwd(const float* __restrict__ gy, int B, int D, int H, int W, int C, float* __restrict__ gx) {
    const long long n = (long long)B * D * H * W * C;
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n) return;
    const int c = (int)(t % C);
    long long v = t / C;
    const int w = (int)(v % W); v /= W;
    const int h = (int)(v % H); v /= H;
    const int d = (int)(v % D);
    const int b = (int)(v / D);
    const int D2 = D / 2, H2 = H / 2, W2 = W / 2;
    gx[t] = 0.125f * gy[((((long long)b * D2 + d / 2) * H2 + h / 2) * W2 + w / 2) * C + c];
}

// nearest 2x upsampling of x [B][D/2][H/2][W/2][Cx] into channels [0, Cx) of y [B][D][H][W][Cy]
// and copy of skip [B][D][H][W][Cs] into channels [Cx, Cx + Cs)
__global__ void k_upsample_concat(const __nv_bfloat16* __restrict__ x, int Cx, const __nv_bfloat16* __restrict__ skip,
                                  int Cs, int B, int D, int H, int W, __nv_bfloat16* __restrict__ y) {
    const int Cy = Cx + Cs;
    const long long n = (long long)B * D * H * W * Cy;
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n) return;
    const int c = (int)(t % Cy);
    const long long v = t / Cy;
    if (c >= Cx) {
        y[t] = skip[v * Cs + (c - Cx)];
        return;
    }
    long long u = v;
    const int w = (int)(u % W); u /= W;
    const int h = (int)(u % H); u /= H;
    const int d = (int)(u % D);
    const int b = (int)(u / D);
    y[t] = x[((((long long)b * (D / 2) + d / 2) * (H / 2) + h / 2) * (W / 2) + w / 2) * Cx + c];
}

// backward of k_upsample_concat: gx (coarse, Cx) = sum of the 8 fine children, gskip = slice
__global__ void k_upsample_concat_bwd(const float* __restrict__ gy, int Cx, int Cs, int B, int D, int H, int W,
                                      float* __restrict__ gx, float* __restrict__ gskip) {
    const int Cy = Cx + Cs;
    const int D2 = D / 2, H2 = H / 2, W2 = W / 2;
    const long long ncoarse = (long long)B * D2 * H2 * W2 * Cx;
    const long long nskip = (long long)B * D * H * W * Cs;
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t < ncoarse) {
        const int c = (int)(t % Cx);
        long long v = t / Cx;
        const int w = (int)(v % W2); v /= W2;
        const int h = (int)(v % H2); v /= H2;
        const int d = (int)(v % D2);
        const int b = (int)(v / D2);
        float s = 0.f;
        for (int a = 0; a < 8; ++a) {
            const int dd = 2 * d + (a >> 2), hh = 2 * h + ((a >> 1) & 1), ww = 2 * w + (a & 1);
            s += gy[((((long long)b * D + dd) * H + hh) * W + ww) * Cy + c];
        }
        gx[t] = s;
    }
    if (gskip && t < nskip) {
        const int c = (int)(t % Cs);
        const long long v = t / Cs;
        gskip[t] = gy[v * Cy + Cx + c];
    }
}

// g = (g + add) * [y > 0] for ReLU layers (relu = 0: plain sum), cast to BF16 for the GEMMs
__global__ void k_act_bwd(const float* __restrict__ g, const float* __restrict__ add, const __nv_bfloat16* __restrict__ y,
                          int relu, long long n, float* __restrict__ gout, __nv_bfloat16* __restrict__ gout_bf16) {
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n) return;
    float v = g[t];
    if (add) v += add[t];
    if (relu && !(__bfloat162float(y[t]) > 0.f)) v = 0.f;
    if (gout) gout[t] = v;
    if (gout_bf16) gout_bf16[t] = __float2bfloat16_rn(v);
}

// output channel 0 of y [nvox][C] times scale[b] into out [nvox] (FP32)
__global__ void k_take_channel0(const float* __restrict__ y, int C, const float* __restrict__ scale, long long vox_per_b,
                                long long nvox, const float* __restrict__ mask, float* __restrict__ out) {
    const long long v = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (v >= nvox) return;
    float o = y[v * C] * (scale ? scale[v / vox_per_b] : 1.f);
    if (mask) o *= mask[v];
    out[v] = o;
}

// MSE on channel 0: grad[v][0] = 2 (y - t) / nvox (masked), other channels 0; loss partials per block
__global__ void k_mse_grad(const float* __restrict__ y, int C, const float* __restrict__ target,
                           const float* __restrict__ mask, long long nvox, float* __restrict__ grad,
                           double* __restrict__ part) {
    __shared__ double sh[BLOCK];
    const long long v = (long long)blockIdx.x * BLOCK + threadIdx.x;
    double l = 0.0;
    if (v < nvox) {
        const float m = mask ? mask[v] : 1.f;   // per-voxel weight (0/1 mask or a relative-error scale)
        const float d = (y[v * C] - target[v]) * m;
        l = (double)d * d;
        for (int c = 0; c < C; ++c) grad[v * C + c] = c == 0 ? 2.f * d * m / (float)nvox : 0.f;
    }
    sh[threadIdx.x] = l;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam on FP32 master weights [rows][kpad] (columns >= kvalid stay zero), refreshes the BF16 copy
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ wb, long long n, int kpad, int kvalid, float lr, float b1, float b2,
                       float eps, float c1, float c2, float grad_scale) {
    const long long t = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (t >= n) return;
    if ((int)(t % kpad) >= kvalid) {
        wb[t] = __float2bfloat16_rn(0.f);
        return;
    }
    const float gr = g[t] * grad_scale;
    const float mm = b1 * m[t] + (1.f - b1) * gr;
    const float vv = b2 * v[t] + (1.f - b2) * gr * gr;
    m[t] = mm;
    v[t] = vv;
    const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    const float nw = w[t] - upd;
    w[t] = nw;
    wb[t] = __float2bfloat16_rn(nw);
}

}  // namespace

extern "C" {

int fc_nn_pack_input(const float* r, const float* k, const float* inv_scale, long long vox_per_b, long long nvox,
                     float k_shift, float k_scale, void* out, void* stream) {
    if (!r || !k || !out || nvox < 0 || vox_per_b < 1) return FC_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(out) & 15) return FC_ERR_ARG;
    if (nvox == 0) return FC_OK;
    k_pack_input<<<grid_for(nvox), BLOCK, 0, (cudaStream_t)stream>>>(r, k, inv_scale, vox_per_b, nvox, k_shift, k_scale,
                                                                     reinterpret_cast<__nv_bfloat16*>(out));
    return launch_status();
}

int fc_nn_avgpool2(const void* x, int B, int D, int H, int W, int C, void* y, void* stream) {
    if (!x || !y || (D | H | W) & 1 || C < 1) return FC_ERR_ARG;
    const long long n = (long long)B * (D / 2) * (H / 2) * (W / 2) * C;
    k_avgpool<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(reinterpret_cast<const __nv_bfloat16*>(x), B, D, H, W, C,
                                                              reinterpret_cast<__nv_bfloat16*>(y));
    return launch_status();
}

int fc_nn_avgpool2_bwd(const float* gy, int B, int D, int H, int W, int C, float* gx, void* stream) {
    if (!gy || !gx || (D | H | W) & 1) return FC_ERR_ARG;
    const long long n = (long long)B * D * H * W * C;
    k_avgpool_bwd<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(gy, B, D, H, W, C, gx);
    return launch_status();
}

int fc_nn_upsample_concat(const void* x, int Cx, const void* skip, int Cs, int B, int D, int H, int W, void* y,
                          void* stream) {
    if (!x || !y || (Cs > 0 && !skip) || (D | H | W) & 1) return FC_ERR_ARG;
    const long long n = (long long)B * D * H * W * (Cx + Cs);
    k_upsample_concat<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const __nv_bfloat16*>(x), Cx, reinterpret_cast<const __nv_bfloat16*>(skip), Cs, B, D, H, W,
        reinterpret_cast<__nv_bfloat16*>(y));
    return launch_status();
}

int fc_nn_upsample_concat_bwd(const float* gy, int Cx, int Cs, int B, int D, int H, int W, float* gx, float* gskip,
                              void* stream) {
    if (!gy || !gx || (D | H | W) & 1) return FC_ERR_ARG;
    const long long n1 = (long long)B * (D / 2) * (H / 2) * (W / 2) * Cx;
    const long long n2 = (long long)B * D * H * W * Cs;
    const long long n = n1 > n2 ? n1 : n2;
    k_upsample_concat_bwd<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(gy, Cx, Cs, B, D, H, W, gx, gskip);
    return launch_status();
}

int fc_nn_act_bwd(const float* g, const float* add, const void* y, int relu, long long n, float* gout,
                  void* gout_bf16, void* stream) {
    if (!g || (relu && !y) || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_act_bwd<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(g, add, reinterpret_cast<const __nv_bfloat16*>(y), relu,
                                                               n, gout, reinterpret_cast<__nv_bfloat16*>(gout_bf16));
    return launch_status();
}

int fc_nn_take_channel0(const float* y, int C, const float* scale, long long vox_per_b, long long nvox,
                        const float* mask, float* out, void* stream) {
    if (!y || !out || C < 1 || vox_per_b < 1) return FC_ERR_ARG;
    if (nvox == 0) return FC_OK;
    k_take_channel0<<<grid_for(nvox), BLOCK, 0, (cudaStream_t)stream>>>(y, C, scale, vox_per_b, nvox, mask, out);
    return launch_status();
}

long long fc_nn_mse_workspace_bytes(long long nvox) { return (long long)(grid_for(nvox) + 1) * 8; }

int fc_nn_mse_grad(const float* y, int C, const float* target, const float* mask, long long nvox, float* grad,
                   void* workspace, long long workspace_bytes, void* stream) {
    if (!y || !target || !grad || !workspace || nvox < 1) return FC_ERR_ARG;
    if (workspace_bytes < fc_nn_mse_workspace_bytes(nvox)) return FC_ERR_ARG;
    k_mse_grad<<<grid_for(nvox), BLOCK, 0, (cudaStream_t)stream>>>(y, C, target, mask, nvox, grad,
                                                                   reinterpret_cast<double*>(workspace));
    return launch_status();
}

int fc_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, int kpad, int kvalid,
               float lr, float beta1, float beta2, float eps, int step, float grad_scale, void* stream) {
    if (!w || !g || !m || !v || !w_bf16 || n < 0 || step < 1 || kpad < 1) return FC_ERR_ARG;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_adam<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(w, g, m, v, reinterpret_cast<__nv_bfloat16*>(w_bf16), n, kpad,
                                                            kvalid, lr, beta1, beta2, eps, c1, c2, grad_scale);
    return launch_status();
}

}  // extern "C"
