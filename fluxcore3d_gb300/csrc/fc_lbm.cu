// fc_lbm.cu -- D3Q19 lattice-Boltzmann kernels for sm_103a behind a C ABI.
//
// Two families live here.
//
// 1. The per-operation kernels with the reference module's call surface
//    (LBM_CUDA.* in solver/lbm_kernels.cu:1347-1386): macro_collide_{bgk,trt,
//    mrt,mrt_smag}, stream_pull, sponge, ibb, reset_solid, zou_he_bc and
//    convective_bc.  They operate on FP32 [19][N] tensors with the reference's
//    semantics and are what a caller that drives single operations binds.
//
// 2. The fused step used by the drop-in solver object: one pass per time step
//    that pulls post-collision populations from the previous step (periodic /
//    copy-self edges as stream_pull), applies interpolated bounce-back from a
//    per-cell link table, collides (BGK/TRT/MRT/MRT-Smagorinsky), applies the
//    outlet sponge and stores the next post-collision populations in FP32 or in
//    FP16/BF16 shifted (f - w_q) form.  Solid cells are never touched: their
//    populations are pinned to w_q in both ping-pong buffers, which is what
//    collide-then-reset produces in the reference every step.  Cells on
//    inlet/outlet planes export their post-stream populations to an FP32 [19][N]
//    tensor so the plane BC kernels can run on it in the reference order, after
//    which plane_collide finishes them.
#include "fc_common.cuh"
#include "fc_collide.cuh"
#include "fc_fused.cuh"
#include "../../include/fluxcore3d_gb300.h"

#include <mutex>

using namespace fc;

namespace {

constexpr int BLOCK = 256;

inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }

// ============================================================================
//  Family 1: per-operation kernels (reference call surface)
// ============================================================================

// The per-operation kernels are templates on the population type R: float
// serves the reference call surface, double the FP64 run of the plain method
// (fc_lbm64_*), which the reduced-precision runs are measured against.
template <int MODE, class R>
__global__ void __launch_bounds__(BLOCK) k_macro_collide(
    const R* __restrict__ f, R* __restrict__ f_post, R* __restrict__ rho,
    R* __restrict__ u, R* __restrict__ v, R* __restrict__ w,
    const uint8_t* __restrict__ solid, CollideParams p, const float* __restrict__ S_dev, long long N) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N) return;
    if (S_dev) {
#pragma unroll
        for (int q = 0; q < 19; ++q) p.S[q] = __ldg(S_dev + q);
    }
    if (solid[idx]) {
#pragma unroll
        for (int q = 0; q < 19; ++q) f_post[q * N + idx] = R(wq(q));
        rho[idx] = R(1); u[idx] = R(0); v[idx] = R(0); w[idx] = R(0);
        return;
    }
    R fi[19], feq[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) fi[q] = __ldg(f + q * N + idx);
    const MacroT<R> m = collide<MODE>(fi, feq, p);
    rho[idx] = m.rho; u[idx] = m.ux; v[idx] = m.uy; w[idx] = m.uz;
#pragma unroll
    for (int q = 0; q < 19; ++q) f_post[q * N + idx] = fi[q];
}

template <class R>
__global__ void __launch_bounds__(BLOCK) k_stream_pull(
    const R* __restrict__ fin, R* __restrict__ fout, int nx, int ny, int nz,
    int px, int py, int pz) {
    const long long N = (long long)nx * ny * nz;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N) return;
    const int nynz = ny * nz;
    const int i = (int)(idx / nynz);
    const int rem = (int)(idx - (long long)i * nynz);
    const int j = rem / nz;
    const int k = rem - j * nz;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        int si = i - cx(q), sj = j - cy(q), sk = k - cz(q);
        bool self = false;
        if (si < 0 || si >= nx) { if (px) si = (si + nx) % nx; else self = true; }
        if (sj < 0 || sj >= ny) { if (py) sj = (sj + ny) % ny; else self = true; }
        if (sk < 0 || sk >= nz) { if (pz) sk = (sk + nz) % nz; else self = true; }
        const long long src = self ? idx : ((long long)si * nynz + (long long)sj * nz + sk);
        fout[q * N + idx] = fin[q * N + src];
    }
}

template <class R>
__global__ void __launch_bounds__(BLOCK) k_sponge(
    R* __restrict__ f, const R* __restrict__ rho, const R* __restrict__ u,
    const R* __restrict__ v, const R* __restrict__ w, const float* __restrict__ sigma,
    long long N) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N) return;
    const R sg = R(sigma[idx]);
    if (sg <= R(0)) return;
    R feq[19];
    equilibrium(rho[idx], u[idx], v[idx], w[idx], feq);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const long long a = q * N + idx;
        f[a] = f[a] - sg * (f[a] - feq[q]);
    }
}

template <class R>
__global__ void __launch_bounds__(BLOCK) k_ibb_links(
    const R* __restrict__ fpost, R* __restrict__ fstream,
    const int* __restrict__ fluid_flat, const int* __restrict__ dir_i,
    const int* __restrict__ dir_opp, const float* __restrict__ w1,
    const float* __restrict__ w2, const uint8_t* __restrict__ q_ge_half,
    const int* __restrict__ ff_flat, const uint8_t* __restrict__ ff_valid,
    long long n_links, long long N, unsigned* __restrict__ dev_err) {
    const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_links) return;
    const long long xf = fluid_flat[l];
    const int qi = dir_i[l], qo = dir_opp[l];
    if (xf < 0 || xf >= N || qi < 0 || qi > 18 || qo < 0 || qo > 18) {
        if (dev_err) atomicOr(dev_err, DEV_ERR_INDEX);
        return;
    }
    const R a = fpost[qo * N + xf];
    R bb;
    if (q_ge_half[l]) {
        bb = R(w1[l]) * a + R(w2[l]) * fpost[qi * N + xf];
    } else if (ff_valid[l]) {
        const long long xff = ff_flat[l];
        if (xff < 0 || xff >= N) {
            if (dev_err) atomicOr(dev_err, DEV_ERR_INDEX);
            return;
        }
        bb = R(w1[l]) * a + R(w2[l]) * fpost[qo * N + xff];
    } else {
        bb = a;
    }
    fstream[qi * N + xf] = bb;
}

template <class R>
__global__ void __launch_bounds__(BLOCK) k_reset_solid(R* __restrict__ f, const uint8_t* __restrict__ solid,
                                                       long long N) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N || !solid[idx]) return;
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q * N + idx] = R(wq(q));
}

// plane node (a,b) -> flat index of plane `p` along `axis`
__device__ __forceinline__ long long plane_flat(int axis, int p, int a, int b, int ny, int nz) {
    if (axis == 0) return ((long long)p * ny + a) * nz + b;
    if (axis == 1) return ((long long)a * ny + p) * nz + b;
    return ((long long)a * ny + b) * nz + p;
}

// Regularized Zou/He on one plane (reference semantics: solver/lbm_kernels.cu:791-969).
// Second-order Hermite tensors Q = c c - I/3 use the reference's 8-digit literals.
__device__ __forceinline__ float q_diag(int c) { return c != 0 ? 0.66666667f : -0.33333333f; }

// The node's post-stream populations fi and, for a pressure outlet (bc_type 1,
// whose both branches read it), those of its interior neighbour fin, loaded
// by the caller so that every load of the node is in flight at once.  Writes
// the node's new populations to f and, when out is given, to out too.
template <class R>
__device__ __forceinline__ void zou_he_core(const R fi[19], const R fin[19], R* __restrict__ f,
                                            long long N, long long flat_bc, int axis, int plane_idx, int bc_type,
                                            R u_in, R rho_out, int sign, R* out) {
    const int unknown = (plane_idx == 0) ? 1 : -1;
    const int known = -unknown;
    R s0 = R(0), sk = R(0);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const int c = axis == 0 ? cx(q) : (axis == 1 ? cy(q) : cz(q));
        if (c == 0) s0 += fi[q];
        if (c == known) sk += fi[q];
    }
    R rho_bc, uax, ub = R(0), vb = R(0), wb = R(0);
    if (bc_type == 0) {
        uax = u_in;
        rho_bc = (s0 + R(2) * sk) / (R(1) - fabs(u_in) + R(1e-12));
        rho_bc = fmin(fmax(rho_bc, R(0.2)), R(5.0));
        if (axis == 0) ub = uax; else if (axis == 1) vb = uax; else wb = uax;
    } else {
        rho_bc = rho_out;
        uax = R(known) * ((s0 + R(2) * sk) / (rho_bc + R(1e-12)) - R(1));
        if (uax * R(sign) < R(0)) {
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                f[q * N + flat_bc] = fin[q];
                if (out) out[q] = fin[q];
            }
            return;
        }
        const MacroT<R> mi = macros_of(fin);
        if (axis == 0) { ub = uax; vb = mi.uy; wb = mi.uz; }
        else if (axis == 1) { ub = mi.ux; vb = uax; wb = mi.uz; }
        else { ub = mi.ux; vb = mi.uy; wb = uax; }
    }
    R feq[19];
    equilibrium(rho_bc, ub, vb, wb, feq);
    R g[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const int c = axis == 0 ? cx(q) : (axis == 1 ? cy(q) : cz(q));
        g[q] = (c == unknown) ? fi[opp(q)] + feq[q] - feq[opp(q)] : fi[q];
    }
    R Pxx = R(0), Pyy = R(0), Pzz = R(0), Pxy = R(0), Pxz = R(0), Pyz = R(0);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const R fn = g[q] - feq[q];
        Pxx += fn * R(q_diag(cx(q)));
        Pyy += fn * R(q_diag(cy(q)));
        Pzz += fn * R(q_diag(cz(q)));
        Pxy += fn * R(cx(q) * cy(q));
        Pxz += fn * R(cx(q) * cz(q));
        Pyz += fn * R(cy(q) * cz(q));
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const R sq = R(q_diag(cx(q))) * Pxx + R(q_diag(cy(q))) * Pyy + R(q_diag(cz(q))) * Pzz +
                     R(2) * (R(cx(q) * cy(q)) * Pxy + R(cx(q) * cz(q)) * Pxz + R(cy(q) * cz(q)) * Pyz);
        const R v = feq[q] + R(wq(q)) * sq * R(4.5);
        f[q * N + flat_bc] = v;
        if (out) out[q] = v;
    }
}

template <class R>
__device__ __forceinline__ void load_zou_he(const R* __restrict__ f, long long N, long long flat_bc,
                                            long long flat_in, int bc_type, R fi[19], R fin[19]) {
#pragma unroll
    for (int q = 0; q < 19; ++q) fi[q] = f[q * N + flat_bc];
    if (bc_type != 0) {
#pragma unroll
        for (int q = 0; q < 19; ++q) fin[q] = f[q * N + flat_in];
    }
}

template <class R>
__device__ void zou_he_node(R* __restrict__ f, long long N, long long flat_bc, long long flat_in,
                            int axis, int plane_idx, int bc_type, R u_in, R rho_out, int sign,
                            R* out = nullptr) {
    R fi[19], fin[19];
    load_zou_he(f, N, flat_bc, flat_in, bc_type, fi, fin);
    zou_he_core(fi, fin, f, N, flat_bc, axis, plane_idx, bc_type, u_in, rho_out, sign, out);
}

template <class R>
__global__ void __launch_bounds__(BLOCK) k_zou_he(
    R* __restrict__ f, const uint8_t* __restrict__ solid, int nx, int ny, int nz, int axis,
    int plane_idx, int interior_idx, int bc_type, R u_in, R rho_out, int sign, int n1, int n2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2) return;
    const int a = t / n2, b = t - (t / n2) * n2;
    const long long N = (long long)nx * ny * nz;
    const long long fb = plane_flat(axis, plane_idx, a, b, ny, nz);
    const long long fi = plane_flat(axis, interior_idx, a, b, ny, nz);
    if (solid[fb]) return;
    zou_he_node(f, N, fb, fi, axis, plane_idx, bc_type, u_in, rho_out, sign);
}

// Convective outlet, pass 1: zero-gradient copy of the incoming populations
// and per-block partial sums (FP64, fixed tree order => deterministic).
template <class R>
__global__ void __launch_bounds__(BLOCK) k_convective_pass1(
    R* __restrict__ f, const uint8_t* __restrict__ solid, int nx, int ny, int nz, int axis,
    int outlet_idx, int interior_idx, int unknown_cax, int n1, int n2,
    double* __restrict__ part_rho, int* __restrict__ part_cnt) {
    __shared__ double s_rho[BLOCK];
    __shared__ int s_cnt[BLOCK];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = (long long)nx * ny * nz;
    double r = 0.0;
    int c = 0;
    if (t < n1 * n2) {
        const int a = t / n2, b = t - (t / n2) * n2;
        const long long fo = plane_flat(axis, outlet_idx, a, b, ny, nz);
        const long long fi = plane_flat(axis, interior_idx, a, b, ny, nz);
        if (!solid[fo]) {
            R rn = R(0);
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const int cq = axis == 0 ? cx(q) : (axis == 1 ? cy(q) : cz(q));
                R val = f[q * N + fo];
                if (cq == unknown_cax) { val = f[q * N + fi]; f[q * N + fo] = val; }
                rn += val;
            }
            r = (double)rn;
            c = 1;
        }
    }
    s_rho[threadIdx.x] = r;
    s_cnt[threadIdx.x] = c;
    __syncthreads();
    for (int st = BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            s_rho[threadIdx.x] += s_rho[threadIdx.x + st];
            s_cnt[threadIdx.x] += s_cnt[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part_rho[blockIdx.x] = s_rho[0]; part_cnt[blockIdx.x] = s_cnt[0]; }
}

// Convective outlet, plane totals: one block reduces the per-block partials in a
// fixed order and leaves the sum of rho and the fluid count in slot 0 (every
// partial is read before the slot is written).
__global__ void __launch_bounds__(BLOCK) k_convective_total(double* __restrict__ part_rho, int* __restrict__ part_cnt,
                                                            int n_parts) {
    __shared__ double s_rho[BLOCK];
    __shared__ int s_cnt[BLOCK];
    double r = 0.0;
    int c = 0;
    for (int p = threadIdx.x; p < n_parts; p += BLOCK) { r += part_rho[p]; c += part_cnt[p]; }
    s_rho[threadIdx.x] = r;
    s_cnt[threadIdx.x] = c;
    __syncthreads();
    for (int st = BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            s_rho[threadIdx.x] += s_rho[threadIdx.x + st];
            s_cnt[threadIdx.x] += s_cnt[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part_rho[0] = s_rho[0];
        part_cnt[0] = s_cnt[0];
    }
}

// Convective outlet, pass 2: rescale the fluid outlet nodes by
// rho_out * count / sum(rho), the plane totals left in slot 0.
template <class R>
__global__ void __launch_bounds__(BLOCK) k_convective_pass2(
    R* __restrict__ f, const uint8_t* __restrict__ solid, int nx, int ny, int nz, int axis,
    int outlet_idx, double rho_out, int n1, int n2, const double* __restrict__ part_rho,
    const int* __restrict__ part_cnt) {
    const double sum = part_rho[0];
    const int cnt = part_cnt[0];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n1 * n2) return;
    if (cnt < 1 || sum < 1e-10) return;
    const R corr = (R)(rho_out * (double)cnt / sum);
    const int a = t / n2, b = t - (t / n2) * n2;
    const long long N = (long long)nx * ny * nz;
    const long long fo = plane_flat(axis, outlet_idx, a, b, ny, nz);
    if (solid[fo]) return;
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q * N + fo] *= corr;
}

// ============================================================================
//  Family 2: fused step
// ============================================================================

// Shared device code of the fused pass: fc_fused.cuh.

template <int KIND, int MODE, bool SKIP_LINKS>
__global__ void __launch_bounds__(TBX * TBY, 7) k_fused_step(const FusedArgs a) {
    int i, j, k, idx;
    if (!cell_of_thread(a.g, i, j, k, idx)) return;
    const uint8_t fl = __ldg(a.flags + idx);
    if (SKIP_LINKS && (fl & CF_LINK)) return;   // finished by k_link_cells
    if (fl & CF_SOLID) {
        if (fl & (CF_DEFER | CF_WRITE_S)) {
            float h[19];
            solid_cell<KIND>(a, idx, i, j, k, h);
            export_f(a, idx, h);
        }
        return;
    }
    float h[19];
    gather_cell<KIND>(a, idx, i, j, k, fl, h);
    if (fl & (CF_DEFER | CF_WRITE_S)) {
        export_f(a, idx, h);
        if (fl & CF_DEFER) return;
    }
    collide_store<KIND, MODE>(a, idx, i, j, k, h);
}

// Two cells per thread (rows j and j+1 of the same k): both cells' pulls are in
// flight before either collision, doubling the bytes a thread keeps in flight.
template <int KIND, int MODE>
__device__ __forceinline__ void finish_cell(const FusedArgs& a, int idx, int i, int j, int k, uint8_t fl,
                                            float h[19]) {
    if (fl & (CF_DEFER | CF_WRITE_S)) {
        export_f(a, idx, h);
        if (fl & CF_DEFER) return;
    }
    collide_store<KIND, MODE>(a, idx, i, j, k, h);
}

template <int KIND, int MODE>
__global__ void __launch_bounds__(TBX * TBY, 6) k_fused_step2(const FusedArgs a) {
    const int k = blockIdx.x * TBX + threadIdx.x;
    const int j0 = blockIdx.y * (2 * TBY) + 2 * threadIdx.y;
    const int i = blockIdx.z;
    if (k >= a.g.nz || j0 >= a.g.ny) return;
    const int j1 = j0 + 1;
    const bool has1 = j1 < a.g.ny;
    const int idx0 = (i * a.g.ny + j0) * a.g.nz + k;
    const int idx1 = idx0 + a.g.nz;
    const uint8_t fl0 = __ldg(a.flags + idx0);
    const uint8_t fl1 = has1 ? __ldg(a.flags + idx1) : (uint8_t)CF_SOLID;
    const bool live0 = !(fl0 & CF_SOLID), live1 = has1 && !(fl1 & CF_SOLID);
    if (!live0 && (fl0 & (CF_DEFER | CF_WRITE_S))) {
        float h[19];
        solid_cell<KIND>(a, idx0, i, j0, k, h);
        export_f(a, idx0, h);
    }
    if (has1 && !live1 && (fl1 & (CF_DEFER | CF_WRITE_S))) {
        float h[19];
        solid_cell<KIND>(a, idx1, i, j1, k, h);
        export_f(a, idx1, h);
    }
    float h0[19], h1[19];
    if (live0) gather_cell<KIND>(a, idx0, i, j0, k, fl0, h0);
    if (live1) gather_cell<KIND>(a, idx1, i, j1, k, fl1, h1);
    if (live0) finish_cell<KIND, MODE>(a, idx0, i, j0, k, fl0, h0);
    if (live1) finish_cell<KIND, MODE>(a, idx1, i, j1, k, fl1, h1);
}

// Cells that own interpolated-bounce-back links, one thread each, from a
// compacted ascending cell list: same work as k_fused_step for those cells.
template <int KIND, int MODE>
__global__ void __launch_bounds__(128) k_link_cells(const FusedArgs a, const int* __restrict__ cells, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int idx = __ldg(cells + t);
    if (idx < 0 || (long long)idx >= a.g.N) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    const uint8_t fl = __ldg(a.flags + idx);
    if (fl & CF_SOLID) return;
    const int i = idx / a.g.nynz;
    const int rem = idx - i * a.g.nynz;
    const int j = rem / a.g.nz, k = rem - (rem / a.g.nz) * a.g.nz;
    float h[19];
    gather_cell<KIND>(a, idx, i, j, k, fl, h);
    if (fl & (CF_DEFER | CF_WRITE_S)) {
        export_f(a, idx, h);
        if (fl & CF_DEFER) return;
    }
    collide_store<KIND, MODE>(a, idx, i, j, k, h);
}

// Per-step gather of every link's interpolated bounce-back value into link_val,
// one thread per link cell of the ascending link-cell list.
template <int KIND>
__global__ void __launch_bounds__(128) k_link_gather(const FusedArgs a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_link_cells) return;
    const int idx = __ldg(a.link_cells + t);
    const uint4 hd = __ldg(a.link_hdr + t);
    if (idx < 0 || (long long)idx >= a.g.N || (long long)hd.z + __popc(hd.x) > a.n_links) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    LinkGather<KIND, 1>::run(a, idx, hd);
}

// The same gather with one thread per link, from the precomputed element
// pairs: f1 = f_opp(d)(x_f), f2 = the second value; result w1 f1 + w2 f2 - w_d
// with the rounding of link_value, stored in storage form.
template <int KIND>
__global__ void __launch_bounds__(256) k_link_gather_links(const FusedArgs a, const int* __restrict__ subset,
                                                           long long n_subset, int skip_marked) {
    using T = typename Store<KIND>::T;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a.gather_order) t = (subset ? n_subset : a.n_links) - 1 - t;   // descending: negative past the end
    if (t < 0) return;
    if (subset) {
        if (t >= n_subset) return;
        t = __ldg(subset + t);
        if (t < 0 || t >= a.n_links) {
            if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
            return;
        }
    } else if (t >= a.n_links) {
        return;
    }
    const uint2 e = __ldg(a.link_src + t);
    if (skip_marked && (e.y >> 31)) return;
    const float2 wt = __ldg(a.link_w + t);
    const unsigned e1 = e.x & 0x7fffffffu, e2 = e.y & 0x7fffffffu;
    const long long lim = 19LL * a.g.N;
    if ((long long)e1 >= lim || (long long)e2 >= lim) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    const float w = (e.x >> 31) ? wq(7) : wq(1);
    const T* p = reinterpret_cast<const T*>(a.pin[0]);
    float f1, f2;
    if (KIND == ST_F32) {
        f1 = __ldg(reinterpret_cast<const float*>(p) + e1);
        f2 = __ldg(reinterpret_cast<const float*>(p) + e2);
    } else if (KIND == ST_F16S) {
        f1 = __fadd_rn(__half2float(__ldg(reinterpret_cast<const __half*>(p) + e1)), w);
        f2 = __fadd_rn(__half2float(__ldg(reinterpret_cast<const __half*>(p) + e2)), w);
    } else {
        f1 = __fadd_rn(__bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + e1)), w);
        f2 = __fadd_rn(__bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + e2)), w);
    }
    const float h = __fsub_rn(__fmaf_rn(wt.x, f1, __fmul_rn(wt.y, f2)), w);
    T out;
    if constexpr (KIND == ST_F32) out = __fadd_rn(h, w);
    else if constexpr (KIND == ST_F16S) out = __float2half_rn(h);
    else out = __float2bfloat16_rn(h);
    reinterpret_cast<T*>(a.link_val)[t] = out;
}

inline dim3 cell_grid(const Geo& g) {
    return dim3((unsigned)((g.nz + TBX - 1) / TBX), (unsigned)((g.ny + TBY - 1) / TBY), (unsigned)g.nx);
}
inline dim3 cell_grid2(const Geo& g) {
    return dim3((unsigned)((g.nz + TBX - 1) / TBX), (unsigned)((g.ny + 2 * TBY - 1) / (2 * TBY)), (unsigned)g.nx);
}

// Rebuild the post-stream FP32 populations (the reference's sim.f) of every
// cell not on a deferred plane from the previous post-collision buffer.
template <int KIND>
__global__ void __launch_bounds__(TBX * TBY) k_materialize(const FusedArgs a) {
    int i, j, k, idx;
    if (!cell_of_thread(a.g, i, j, k, idx)) return;
    const uint8_t fl = a.flags[idx];
    if (fl & CF_DEFER) return;
    float h[19];
    if (fl & CF_SOLID) solid_cell<KIND>(a, idx, i, j, k, h);
    else gather_cell<KIND>(a, idx, i, j, k, fl, h);
    export_f(a, idx, h);
}

// Collide cells straight from the FP32 post-stream tensor: the whole grid at
// start-up (prologue) or one inlet/outlet plane after its BC (plane mode).
template <int KIND, int MODE>
__global__ void __launch_bounds__(BLOCK) k_collide_from_f32(const FusedArgs a, int axis, int plane,
                                                            int n1, int n2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int idx;
    if (axis < 0) {
        if (t >= a.g.N) return;
        idx = (int)t;
    } else {
        if (t >= (long long)n1 * n2) return;
        const int pa = (int)(t / n2), pb = (int)(t - (t / n2) * n2);
        idx = (int)plane_flat(axis, plane, pa, pb, a.g.ny, a.g.nz);
    }
    if (a.flags[idx] & CF_SOLID) return;
    const int i = idx / a.g.nynz;
    const int rem = idx - i * a.g.nynz;
    const int j = rem / a.g.nz, k = rem - (rem / a.g.nz) * a.g.nz;
    float h[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) h[q] = a.f32[q * a.g.N + idx] - wq(q);
    collide_store<KIND, MODE>(a, idx, i, j, k, h);
}

// Zou/He and collision of every node of up to FC_MAX_PLANES disjoint planes of
// one axis: thread t -> plane p with start[p] <= t < start[p + 1].
struct PlaneSet {
    int n;
    fc_plane_bc p[FC_MAX_PLANES];
    int n1[FC_MAX_PLANES], n2[FC_MAX_PLANES];
    int start[FC_MAX_PLANES + 1];
};

constexpr int PLANE_BLOCK = 128;     // plane work is a few thousand warps: spread it over every SM

template <int KIND, int MODE>
__global__ void __launch_bounds__(PLANE_BLOCK) k_planes_zou_he_collide(const FusedArgs a, const PlaneSet ps) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ps.start[ps.n]) return;
    int p = 0;
    while (p + 1 < ps.n && t >= ps.start[p + 1]) ++p;
    const fc_plane_bc& pl = ps.p[p];
    const int u = t - ps.start[p];
    const int pa = u / ps.n2[p], pb = u - (u / ps.n2[p]) * ps.n2[p];
    const int idx = (int)plane_flat(pl.axis, pl.plane_idx, pa, pb, a.g.ny, a.g.nz);
    const long long fi = plane_flat(pl.axis, pl.interior_idx, pa, pb, a.g.ny, a.g.nz);
    // the flag byte and every population the node reads are requested together
    const uint8_t fl = a.flags[idx];
    float fb[19], fn[19];
    load_zou_he(a.f32, a.g.N, idx, fi, pl.bc_type, fb, fn);
    if (fl & CF_SOLID) return;
    float fv[19];
    zou_he_core(fb, fn, a.f32, a.g.N, idx, pl.axis, pl.plane_idx, pl.bc_type, pl.u_in_lat, pl.rho_out_lat, pl.sign,
                fv);
    const int i = idx / a.g.nynz;
    const int rem = idx - i * a.g.nynz;
    const int j = rem / a.g.nz, k = rem - (rem / a.g.nz) * a.g.nz;
    float h[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) h[q] = fv[q] - wq(q);
    collide_store<KIND, MODE>(a, idx, i, j, k, h);
}

template <int S, int M>
struct PlanesLauncher {
    static int go(const FusedArgs& a, cudaStream_t st, const PlaneSet& ps) {
        const unsigned nb = (unsigned)((ps.start[ps.n] + PLANE_BLOCK - 1) / PLANE_BLOCK);
        k_planes_zou_he_collide<S, M><<<nb, PLANE_BLOCK, 0, st>>>(a, ps);
        return launch_status();
    }
};

// Pin solid cells: populations w_q in the given buffer (shifted => 0), macros (1,0,0,0).
template <int KIND>
__global__ void __launch_bounds__(BLOCK) k_pin_solid(const FusedArgs a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.g.N) return;
    const int idx = (int)t;
    if (!(a.flags[idx] & CF_SOLID)) return;
#pragma unroll
    for (int q = 0; q < 19; ++q) out_h<KIND>(a, q, idx, 0.f);
    if (a.rho) { a.rho[idx] = 1.f; a.u[idx] = 0.f; a.v[idx] = 0.f; a.w[idx] = 0.f; }
}

int make_fused_args(const fc_lbm_step_args* s, FusedArgs& a) {
    if (!s) return FC_ERR_ARG;
    if (s->nx < 1 || s->ny < 1 || s->nz < 1) return FC_ERR_ARG;
    if (s->storage < 0 || s->storage > 2 || s->collision < 0 || s->collision > 3) return FC_ERR_ARG;
    a.g.nx = s->nx; a.g.ny = s->ny; a.g.nz = s->nz;
    a.g.px = s->periodic[0] != 0; a.g.py = s->periodic[1] != 0; a.g.pz = s->periodic[2] != 0;
    a.g.N = (long long)s->nx * s->ny * s->nz;
    if (a.g.N >= (1LL << 31)) return FC_ERR_UNSUPPORTED;  // cell indices are 32-bit
    a.g.nynz = s->ny * s->nz;
    {
        const size_t eb = s->storage == ST_F32 ? 4 : 2;
        for (int q = 0; q < 19; ++q) {
            a.pin[q] = s->pop_in ? (const void*)((const char*)s->pop_in + (size_t)q * (size_t)a.g.N * eb) : nullptr;
            a.pout[q] = s->pop_out ? (void*)((char*)s->pop_out + (size_t)q * (size_t)a.g.N * eb) : nullptr;
        }
    }
    a.f32 = s->f32;
    a.rho = s->rho; a.u = s->u; a.v = s->v; a.w = s->w;
    if (a.rho && (!a.u || !a.v || !a.w)) return FC_ERR_ARG;
    a.flags = s->cell_flags;
    a.link_off = s->link_off;
    a.link_hdr = reinterpret_cast<const uint4*>(s->link_hdr);
    a.link_w = reinterpret_cast<const float2*>(s->link_w);
    a.n_links = s->n_links;
    a.link_cells = s->link_cells;
    a.n_link_cells = s->n_link_cells;
    if (a.link_hdr && (reinterpret_cast<uintptr_t>(a.link_hdr) & 15)) return FC_ERR_ARG;
    a.link_val = s->link_val;
    a.n_link_val = s->n_link_val;
    if (a.link_val && (a.n_link_val < a.n_links + 8 || !a.link_cells || a.n_link_cells <= 0))
        a.link_val = nullptr;   // the gather needs the link-cell list and a padded buffer
    if (a.link_val && (reinterpret_cast<uintptr_t>(a.link_val) & 15)) return FC_ERR_ARG;
    a.tile_links = reinterpret_cast<const int4*>(s->tile_links);
    a.n_tile_links = s->n_tile_links;
    if (a.tile_links && (reinterpret_cast<uintptr_t>(a.tile_links) & 15)) return FC_ERR_ARG;
    a.link_pos = s->link_pos;
    a.n_link_pos = s->n_link_pos;
    if (a.link_pos && (a.n_link_pos < a.n_links + 8 || (reinterpret_cast<uintptr_t>(a.link_pos) & 15)))
        a.link_pos = nullptr;
    a.link_src = reinterpret_cast<const uint2*>(s->link_src);
    a.n_link_src = s->n_link_src;
    if (a.link_src && (a.n_link_src < a.n_links || (reinterpret_cast<uintptr_t>(a.link_src) & 7) ||
                       19LL * a.g.N >= (1LL << 31)))
        a.link_src = nullptr;
    a.sponge = s->sponge; a.sponge_axis = s->sponge_axis;
    if (a.sponge && (a.sponge_axis < 0 || a.sponge_axis > 2)) return FC_ERR_ARG;
    a.has_links = s->has_links;
    a.cp.omega = s->omega; a.cp.omega_plus = s->omega_plus; a.cp.omega_minus = s->omega_minus;
    for (int q = 0; q < 19; ++q) {
        a.cp.S[q] = s->S[q];
        a.cp.SN[q] = s->S[q] / mrt_row_norm2(q);
    }
    a.cp.Cs_dx2 = s->Cs_dx2; a.cp.omega0 = s->omega0;
    a.dev_err = s->dev_err;
    a.tr_in = s->tracer_in; a.tr_out = s->tracer_out;
    a.tr_u = s->tracer_u; a.tr_v = s->tracer_v; a.tr_w = s->tracer_w;
    a.tr_solid = s->tracer_solid; a.tr_diss = s->tracer_dissipation;
    a.tile_order = s->tile_order != 0;
    a.gather_order = s->gather_order != 0;
    if (a.tr_in && (!a.tr_out || !a.tr_u || !a.tr_v || !a.tr_w || !a.tr_solid || a.tr_in == a.tr_out))
        return FC_ERR_ARG;
    if (a.tr_in && a.u && (a.tr_u == a.u || a.tr_v == a.v || a.tr_w == a.w)) return FC_ERR_ARG;
    if (!a.flags) return FC_ERR_ARG;
    if (a.n_links > 0 && (!a.link_off || !a.link_hdr || !a.link_w || a.n_link_cells <= 0)) return FC_ERR_ARG;
    return FC_OK;
}

template <template <int, int> class Launcher>
int dispatch(int storage, int collision, const FusedArgs& a, cudaStream_t st, int x0, int x1, int x2, int x3) {
#define FC_CASE(S, M) \
    if (storage == S && collision == M) return Launcher<S, M>::go(a, st, x0, x1, x2, x3);
    FC_CASE(ST_F32, CM_BGK) FC_CASE(ST_F32, CM_TRT) FC_CASE(ST_F32, CM_MRT) FC_CASE(ST_F32, CM_MRT_SMAG)
    FC_CASE(ST_F16S, CM_BGK) FC_CASE(ST_F16S, CM_TRT) FC_CASE(ST_F16S, CM_MRT) FC_CASE(ST_F16S, CM_MRT_SMAG)
    FC_CASE(ST_BF16S, CM_BGK) FC_CASE(ST_BF16S, CM_TRT) FC_CASE(ST_BF16S, CM_MRT) FC_CASE(ST_BF16S, CM_MRT_SMAG)
#undef FC_CASE
    return FC_ERR_ARG;
}

template <int S, int M>
struct StepLauncher {
    static int go(const FusedArgs& a, cudaStream_t st, int skip_links, int cells_per_thread, int, int) {
        if (skip_links) k_fused_step<S, M, true><<<cell_grid(a.g), dim3(TBX, TBY), 0, st>>>(a);
        else if (cells_per_thread == 2) k_fused_step2<S, M><<<cell_grid2(a.g), dim3(TBX, TBY), 0, st>>>(a);
        else k_fused_step<S, M, false><<<cell_grid(a.g), dim3(TBX, TBY), 0, st>>>(a);
        return launch_status();
    }
};
template <int S, int M>
struct LinkCellLauncher {
    static int go(const FusedArgs& a, cudaStream_t st, int, int, int, int) {
        const int n = (int)a.n_link_cells;
        if (n <= 0) return FC_OK;
        k_link_cells<S, M><<<(n + 127) / 128, 128, 0, st>>>(a, a.link_cells, n);
        return launch_status();
    }
};
template <int S, int M>
struct CollideF32Launcher {
    static int go(const FusedArgs& a, cudaStream_t st, int axis, int plane, int n1, int n2) {
        const long long n = axis < 0 ? a.g.N : (long long)n1 * n2;
        k_collide_from_f32<S, M><<<grid_for(n), BLOCK, 0, st>>>(a, axis, plane, n1, n2);
        return launch_status();
    }
};

int launch_link_gather(const FusedArgs& a, int storage, cudaStream_t st, const int* subset = nullptr,
                       long long n_subset = 0, int skip_marked = 0) {
    if (!a.link_val || a.n_links <= 0) return FC_OK;
    if (subset && !a.link_src) return FC_ERR_ARG;
    if (a.link_src) {
        const long long n = subset ? n_subset : a.n_links;
        if (n <= 0) return FC_OK;
        const unsigned nb = (unsigned)((n + 255) / 256);
        switch (storage) {
            case ST_F32: k_link_gather_links<ST_F32><<<nb, 256, 0, st>>>(a, subset, n_subset, skip_marked); break;
            case ST_F16S: k_link_gather_links<ST_F16S><<<nb, 256, 0, st>>>(a, subset, n_subset, skip_marked); break;
            default: k_link_gather_links<ST_BF16S><<<nb, 256, 0, st>>>(a, subset, n_subset, skip_marked); break;
        }
    } else {
        const unsigned nb = (unsigned)((a.n_link_cells + 127) / 128);
        switch (storage) {
            case ST_F32: k_link_gather<ST_F32><<<nb, 128, 0, st>>>(a); break;
            case ST_F16S: k_link_gather<ST_F16S><<<nb, 128, 0, st>>>(a); break;
            default: k_link_gather<ST_BF16S><<<nb, 128, 0, st>>>(a); break;
        }
    }
    return launch_status();
}

template <int S, int M>
int planes_dispatch(const FusedArgs& a, cudaStream_t st, const PlaneSet& ps) {
    return PlanesLauncher<S, M>::go(a, st, ps);
}

}  // namespace

// ============================================================================
//  C ABI
// ============================================================================
extern "C" {

int fc_abi_version(void) { return FC_ABI_VERSION; }

long long fc_lbm_step_args_size(void) { return (long long)sizeof(fc_lbm_step_args); }

static int check_collide_ptrs(const float* f, float* fp, float* r, float* u, float* v, float* w,
                              const uint8_t* s, long long n) {
    if (!f || !fp || !r || !u || !v || !w || !s || n < 0) return FC_ERR_ARG;
    return FC_OK;
}

int fc_lbm_macro_collide_bgk(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, float omega, long long n_cells, void* stream) {
    int rc = check_collide_ptrs(f, f_post, rho, u, v, w, solid, n_cells);
    if (rc) return rc;
    if (n_cells == 0) return FC_OK;
    CollideParams p{}; p.omega = omega;
    const float* S_dev = nullptr;
    k_macro_collide<CM_BGK><<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells);
    return launch_status();
}

int fc_lbm_macro_collide_trt(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, float omega_plus, float omega_minus, long long n_cells,
                             void* stream) {
    int rc = check_collide_ptrs(f, f_post, rho, u, v, w, solid, n_cells);
    if (rc) return rc;
    if (n_cells == 0) return FC_OK;
    CollideParams p{}; p.omega_plus = omega_plus; p.omega_minus = omega_minus;
    const float* S_dev = nullptr;
    k_macro_collide<CM_TRT><<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells);
    return launch_status();
}

int fc_lbm_macro_collide_mrt(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, const float* S_dev, long long n_cells, void* stream) {
    int rc = check_collide_ptrs(f, f_post, rho, u, v, w, solid, n_cells);
    if (rc) return rc;
    if (!S_dev) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    CollideParams p{};
    k_macro_collide<CM_MRT><<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells);
    return launch_status();
}

int fc_lbm_macro_collide_mrt_smag(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                                  const uint8_t* solid, const float* S_dev, float Cs_dx2, float omega0,
                                  long long n_cells, void* stream) {
    int rc = check_collide_ptrs(f, f_post, rho, u, v, w, solid, n_cells);
    if (rc) return rc;
    if (!S_dev) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    CollideParams p{};
    p.Cs_dx2 = Cs_dx2; p.omega0 = omega0;
    k_macro_collide<CM_MRT_SMAG><<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells);
    return launch_status();
}

int fc_lbm_stream_pull(const float* f_in, float* f_out, int nx, int ny, int nz, int px, int py, int pz,
                       void* stream) {
    if (!f_in || !f_out || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    if (f_in == f_out) return FC_ERR_ARG;
    const long long N = (long long)nx * ny * nz;
    k_stream_pull<<<grid_for(N), BLOCK, 0, (cudaStream_t)stream>>>(f_in, f_out, nx, ny, nz, px, py, pz);
    return launch_status();
}

int fc_lbm_sponge(float* f, const float* rho, const float* u, const float* v, const float* w,
                  const float* sigma, long long n_cells, void* stream) {
    if (!f || !rho || !u || !v || !w || !sigma || n_cells < 0) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    k_sponge<<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, rho, u, v, w, sigma, n_cells);
    return launch_status();
}

int fc_lbm_ibb(const float* f_post, float* f_stream, const int32_t* fluid_flat, const int32_t* dir_i,
               const int32_t* dir_opp, const float* w1, const float* w2, const uint8_t* q_ge_half,
               const int32_t* ff_flat, const uint8_t* ff_valid, long long n_links, long long n_cells,
               unsigned* dev_err, void* stream) {
    if (n_links < 0 || n_cells < 0) return FC_ERR_ARG;
    if (n_links == 0) return FC_OK;
    if (!f_post || !f_stream || !fluid_flat || !dir_i || !dir_opp || !w1 || !w2 || !q_ge_half ||
        !ff_flat || !ff_valid)
        return FC_ERR_ARG;
    k_ibb_links<<<grid_for(n_links), BLOCK, 0, (cudaStream_t)stream>>>(
        f_post, f_stream, fluid_flat, dir_i, dir_opp, w1, w2, q_ge_half, ff_flat, ff_valid, n_links,
        n_cells, dev_err);
    return launch_status();
}

int fc_lbm_reset_solid(float* f, const uint8_t* solid, long long n_cells, void* stream) {
    if (!f || !solid || n_cells < 0) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    k_reset_solid<<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, solid, n_cells);
    return launch_status();
}

static int plane_dims(int axis, int nx, int ny, int nz, int* n1, int* n2) {
    if (axis == 0) { *n1 = ny; *n2 = nz; }
    else if (axis == 1) { *n1 = nx; *n2 = nz; }
    else if (axis == 2) { *n1 = nx; *n2 = ny; }
    else return FC_ERR_ARG;
    return FC_OK;
}

int fc_lbm_zou_he_bc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int plane_idx,
                     int interior_idx, int bc_type, float u_in_lat, float rho_out_lat, int sign, void* stream) {
    int n1, n2;
    if (!f || !solid || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    if (plane_dims(axis, nx, ny, nz, &n1, &n2)) return FC_ERR_ARG;
    const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (plane_idx < 0 || plane_idx >= na || interior_idx < 0 || interior_idx >= na) return FC_ERR_ARG;
    if (bc_type != 0 && bc_type != 1) return FC_ERR_ARG;
    k_zou_he<<<grid_for((long long)n1 * n2), BLOCK, 0, (cudaStream_t)stream>>>(
        f, solid, nx, ny, nz, axis, plane_idx, interior_idx, bc_type, u_in_lat, rho_out_lat, sign, n1, n2);
    return launch_status();
}

long long fc_lbm_convective_workspace_bytes(int n1, int n2) {
    if (n1 < 1 || n2 < 1) return -1;
    const long long nb = ((long long)n1 * n2 + BLOCK - 1) / BLOCK;
    return nb * (long long)(sizeof(double) + sizeof(int)) + 16;
}

int fc_lbm_convective_bc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                         int interior_idx, int unknown_cax, float rho_out_lat, int n1, int n2,
                         void* workspace, long long workspace_bytes, void* stream) {
    if (!f || !solid || !workspace || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    int e1, e2;
    if (plane_dims(axis, nx, ny, nz, &e1, &e2)) return FC_ERR_ARG;
    if (e1 != n1 || e2 != n2) return FC_ERR_ARG;
    const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (outlet_idx < 0 || outlet_idx >= na || interior_idx < 0 || interior_idx >= na) return FC_ERR_ARG;
    if (unknown_cax != 1 && unknown_cax != -1) return FC_ERR_ARG;
    if (workspace_bytes < fc_lbm_convective_workspace_bytes(n1, n2)) return FC_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(workspace) % 8 != 0) return FC_ERR_ARG;
    const int nb = (int)grid_for((long long)n1 * n2);
    double* part_rho = reinterpret_cast<double*>(workspace);
    int* part_cnt = reinterpret_cast<int*>(part_rho + nb);
    cudaStream_t st = (cudaStream_t)stream;
    k_convective_pass1<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, interior_idx, unknown_cax,
                                             n1, n2, part_rho, part_cnt);
    int rc = launch_status();
    if (rc) return rc;
    k_convective_total<<<1, BLOCK, 0, st>>>(part_rho, part_cnt, nb);
    rc = launch_status();
    if (rc) return rc;
    k_convective_pass2<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, rho_out_lat, n1, n2,
                                             part_rho, part_cnt);
    return launch_status();
}

// ---------------------------------------------------------------------------
// FP64 run of the plain method: the per-operation kernels above instantiated
// for double populations and macros (rates, sponge profile and link weights stay
// the reference's FP32 values, promoted).  Same argument meaning and checks as
// the FP32 entry points; collision selects BGK/TRT/MRT/MRT-Smagorinsky.
// ---------------------------------------------------------------------------
int fc_lbm64_macro_collide(int collision, const double* f, double* f_post, double* rho, double* u, double* v,
                           double* w, const uint8_t* solid, float omega, float omega_plus, float omega_minus,
                           const float* S_dev, float Cs_dx2, float omega0, long long n_cells, void* stream) {
    if (!f || !f_post || !rho || !u || !v || !w || !solid || n_cells < 0) return FC_ERR_ARG;
    if ((collision == CM_MRT || collision == CM_MRT_SMAG) && !S_dev) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    CollideParams p{};
    p.omega = omega; p.omega_plus = omega_plus; p.omega_minus = omega_minus;
    p.Cs_dx2 = Cs_dx2; p.omega0 = omega0;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned g = grid_for(n_cells);
    switch (collision) {
        case CM_BGK: k_macro_collide<CM_BGK><<<g, BLOCK, 0, st>>>(f, f_post, rho, u, v, w, solid, p, nullptr, n_cells); break;
        case CM_TRT: k_macro_collide<CM_TRT><<<g, BLOCK, 0, st>>>(f, f_post, rho, u, v, w, solid, p, nullptr, n_cells); break;
        case CM_MRT: k_macro_collide<CM_MRT><<<g, BLOCK, 0, st>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells); break;
        case CM_MRT_SMAG:
            k_macro_collide<CM_MRT_SMAG><<<g, BLOCK, 0, st>>>(f, f_post, rho, u, v, w, solid, p, S_dev, n_cells);
            break;
        default: return FC_ERR_ARG;
    }
    return launch_status();
}

int fc_lbm64_stream_pull(const double* f_in, double* f_out, int nx, int ny, int nz, int px, int py, int pz,
                         void* stream) {
    if (!f_in || !f_out || nx < 1 || ny < 1 || nz < 1 || f_in == f_out) return FC_ERR_ARG;
    const long long N = (long long)nx * ny * nz;
    k_stream_pull<<<grid_for(N), BLOCK, 0, (cudaStream_t)stream>>>(f_in, f_out, nx, ny, nz, px, py, pz);
    return launch_status();
}

int fc_lbm64_sponge(double* f, const double* rho, const double* u, const double* v, const double* w,
                    const float* sigma, long long n_cells, void* stream) {
    if (!f || !rho || !u || !v || !w || !sigma || n_cells < 0) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    k_sponge<<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, rho, u, v, w, sigma, n_cells);
    return launch_status();
}

int fc_lbm64_ibb(const double* f_post, double* f_stream, const int32_t* fluid_flat, const int32_t* dir_i,
                 const int32_t* dir_opp, const float* w1, const float* w2, const uint8_t* q_ge_half,
                 const int32_t* ff_flat, const uint8_t* ff_valid, long long n_links, long long n_cells,
                 unsigned* dev_err, void* stream) {
    if (n_links < 0 || n_cells < 0) return FC_ERR_ARG;
    if (n_links == 0) return FC_OK;
    if (!f_post || !f_stream || !fluid_flat || !dir_i || !dir_opp || !w1 || !w2 || !q_ge_half || !ff_flat ||
        !ff_valid)
        return FC_ERR_ARG;
    k_ibb_links<<<grid_for(n_links), BLOCK, 0, (cudaStream_t)stream>>>(
        f_post, f_stream, fluid_flat, dir_i, dir_opp, w1, w2, q_ge_half, ff_flat, ff_valid, n_links, n_cells,
        dev_err);
    return launch_status();
}

int fc_lbm64_reset_solid(double* f, const uint8_t* solid, long long n_cells, void* stream) {
    if (!f || !solid || n_cells < 0) return FC_ERR_ARG;
    if (n_cells == 0) return FC_OK;
    k_reset_solid<<<grid_for(n_cells), BLOCK, 0, (cudaStream_t)stream>>>(f, solid, n_cells);
    return launch_status();
}

int fc_lbm64_zou_he_bc(double* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int plane_idx,
                       int interior_idx, int bc_type, double u_in_lat, double rho_out_lat, int sign, void* stream) {
    int n1, n2;
    if (!f || !solid || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    if (plane_dims(axis, nx, ny, nz, &n1, &n2)) return FC_ERR_ARG;
    const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (plane_idx < 0 || plane_idx >= na || interior_idx < 0 || interior_idx >= na) return FC_ERR_ARG;
    if (bc_type != 0 && bc_type != 1) return FC_ERR_ARG;
    k_zou_he<<<grid_for((long long)n1 * n2), BLOCK, 0, (cudaStream_t)stream>>>(
        f, solid, nx, ny, nz, axis, plane_idx, interior_idx, bc_type, u_in_lat, rho_out_lat, sign, n1, n2);
    return launch_status();
}

int fc_lbm64_convective_bc(double* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                           int interior_idx, int unknown_cax, double rho_out_lat, int n1, int n2, void* workspace,
                           long long workspace_bytes, void* stream) {
    if (!f || !solid || !workspace || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    int e1, e2;
    if (plane_dims(axis, nx, ny, nz, &e1, &e2)) return FC_ERR_ARG;
    if (e1 != n1 || e2 != n2) return FC_ERR_ARG;
    const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (outlet_idx < 0 || outlet_idx >= na || interior_idx < 0 || interior_idx >= na) return FC_ERR_ARG;
    if (unknown_cax != 1 && unknown_cax != -1) return FC_ERR_ARG;
    if (workspace_bytes < fc_lbm_convective_workspace_bytes(n1, n2)) return FC_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(workspace) % 8 != 0) return FC_ERR_ARG;
    const int nb = (int)grid_for((long long)n1 * n2);
    double* part_rho = reinterpret_cast<double*>(workspace);
    int* part_cnt = reinterpret_cast<int*>(part_rho + nb);
    cudaStream_t st = (cudaStream_t)stream;
    k_convective_pass1<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, interior_idx, unknown_cax,
                                             n1, n2, part_rho, part_cnt);
    int rc = launch_status();
    if (rc) return rc;
    k_convective_total<<<1, BLOCK, 0, st>>>(part_rho, part_cnt, nb);
    rc = launch_status();
    if (rc) return rc;
    k_convective_pass2<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, rho_out_lat, n1, n2,
                                             part_rho, part_cnt);
    return launch_status();
}

// ---------------------------------------------------------------------------
// Convective outlet without any device allocation.
//
// Some callers cannot allocate device memory once their time loop runs: hosts
// that hand out all GPU memory from their own pre-reserved arena (a coupled
// solver driving this library from C or Fortran), or code paths where an
// allocation would have to synchronise the device.  For them this entry point
// keeps the plane-reduction partials in a fixed file-scope device array
// instead of a caller workspace.  Capacity: FC_NOALLOC_CONVECTIVE_MAX_BLOCKS
// partial slots, i.e. outlet planes of at most 4096 * 256 = 1,048,576 nodes
// (49,152 bytes, held by every GPU that loads the library until the process
// exits).  Larger planes are rejected with FC_ERR_TOO_LARGE.
//
// The device address of the array is looked up with cudaGetSymbolAddress on
// the first call made on each device (with that device current) and cached;
// make that first call before any stream capture.  All calls share the one
// array, so calls whose kernels overlap on the GPU (different streams without
// ordering) race on it.  Every slot the totals pass reads is written by the
// first pass of the same call, and the totals pass writes slot 0 that the last
// pass reads, so nothing has to be cleared between calls.
// ---------------------------------------------------------------------------
#define FC_NOALLOC_CONVECTIVE_MAX_BLOCKS 4096
static __device__ __align__(256) unsigned char g_noalloc_convective_scratch[FC_NOALLOC_CONVECTIVE_MAX_BLOCKS *
                                                                            (sizeof(double) + sizeof(int))];
static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FC_ERR_LAUNCH;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_convective_scratch) != cudaSuccess || !p) return FC_ERR_LAUNCH;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return FC_OK;
}

long long fc_lbm_convective_noalloc_max_plane(void) { return (long long)FC_NOALLOC_CONVECTIVE_MAX_BLOCKS * BLOCK; }

int fc_lbm_convective_bc_noalloc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                                 int interior_idx, int unknown_cax, float rho_out_lat, int n1, int n2, void* stream) {
    if (!f || !solid || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    int e1, e2;
    if (plane_dims(axis, nx, ny, nz, &e1, &e2)) return FC_ERR_ARG;
    if (e1 != n1 || e2 != n2) return FC_ERR_ARG;
    const int na = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (outlet_idx < 0 || outlet_idx >= na || interior_idx < 0 || interior_idx >= na) return FC_ERR_ARG;
    if (unknown_cax != 1 && unknown_cax != -1) return FC_ERR_ARG;
    const long long nbl = ((long long)n1 * n2 + BLOCK - 1) / BLOCK;
    if (nbl > FC_NOALLOC_CONVECTIVE_MAX_BLOCKS) return FC_ERR_TOO_LARGE;
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    const int nb = (int)nbl;
    double* part_rho = reinterpret_cast<double*>(scratch);
    int* part_cnt = reinterpret_cast<int*>(part_rho + FC_NOALLOC_CONVECTIVE_MAX_BLOCKS);
    cudaStream_t st = (cudaStream_t)stream;
    k_convective_pass1<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, interior_idx, unknown_cax,
                                             n1, n2, part_rho, part_cnt);
    rc = launch_status();
    if (rc) return rc;
    k_convective_total<<<1, BLOCK, 0, st>>>(part_rho, part_cnt, nb);
    rc = launch_status();
    if (rc) return rc;
    k_convective_pass2<<<nb, BLOCK, 0, st>>>(f, solid, nx, ny, nz, axis, outlet_idx, rho_out_lat, n1, n2,
                                             part_rho, part_cnt);
    return launch_status();
}

int fc_lbm_fused_step(const fc_lbm_step_args* args, void* stream) {
    FusedArgs a;
    int rc = make_fused_args(args, a);
    if (rc) return rc;
    if (!args->pop_in || !args->pop_out || args->pop_in == args->pop_out) return FC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int split = args->link_cells != nullptr && args->n_link_cells > 0 && args->separate_link_pass;
    const int phases = args->phase_mask ? args->phase_mask : 3;
    if (phases & 1) {
        if (!args->skip_link_gather) {
            rc = launch_link_gather(a, args->storage, st);
            if (rc) return rc;
        }
        rc = FC_ERR_UNSUPPORTED;
        bool tracer_done = false;
        if (!split && args->staging == 0 && args->cells_per_thread <= 1 && fused_tma_eligible(a, args->storage)) {
            // the staged pass reads and writes the tracer in cell pairs (8-byte words)
            FusedArgs am = a;
            const bool carry = a.tr_in && !((reinterpret_cast<uintptr_t>(a.tr_in) | reinterpret_cast<uintptr_t>(a.tr_out) |
                                             reinterpret_cast<uintptr_t>(a.tr_u) | reinterpret_cast<uintptr_t>(a.tr_v) |
                                             reinterpret_cast<uintptr_t>(a.tr_w)) & 7) &&
                               !(reinterpret_cast<uintptr_t>(a.tr_solid) & 1);
            if (!carry) am.tr_in = nullptr;
            rc = launch_fused_tma(am, args->storage, args->collision, st);
            tracer_done = rc == FC_OK && carry;
        }
        if (rc == FC_ERR_UNSUPPORTED)
            rc = dispatch<StepLauncher>(args->storage, args->collision, a, st, split, args->cells_per_thread, 0, 0);
        if (rc) return rc;
        if (a.tr_in && !tracer_done) {   // the direct pass does not carry the tracer
            rc = fc_tracer_step(a.tr_in, a.tr_out, a.tr_u, a.tr_v, a.tr_w, a.tr_solid, a.g.nx, a.g.ny, a.g.nz,
                                a.tr_diss, stream);
            if (rc) return rc;
        }
    }
    if (!split || !(phases & 2)) return FC_OK;
    return dispatch<LinkCellLauncher>(args->storage, args->collision, a, st, 0, 0, 0, 0);
}

long long fc_lbm_tile_links(const fc_lbm_step_args* args, int32_t* records, long long cap, uint16_t* link_pos,
                            long long pos_cap, uint32_t* link_src, long long src_cap, void* stream) {
    FusedArgs a;
    const int rc = make_fused_args(args, a);
    if (rc) return -rc;
    return tma_tile_links(a, reinterpret_cast<int4*>(records), cap, link_pos, pos_cap,
                          reinterpret_cast<uint2*>(link_src), src_cap, (cudaStream_t)stream);
}

int fc_lbm_link_gather(const fc_lbm_step_args* args, const int32_t* subset, long long n_subset, int skip_marked,
                       void* stream) {
    FusedArgs a;
    const int rc = make_fused_args(args, a);
    if (rc) return rc;
    if (!args->pop_in || n_subset < 0) return FC_ERR_ARG;
    return launch_link_gather(a, args->storage, (cudaStream_t)stream, subset, n_subset, skip_marked);
}

int fc_lbm_planes_zou_he_collide(const fc_lbm_step_args* args, const fc_plane_bc* planes, int n_planes,
                                 void* stream) {
    FusedArgs a;
    const int rc = make_fused_args(args, a);
    if (rc) return rc;
    if (!a.f32 || !args->pop_out || !planes || n_planes < 1 || n_planes > FC_MAX_PLANES) return FC_ERR_ARG;
    PlaneSet ps;
    ps.n = n_planes;
    ps.start[0] = 0;
    for (int p = 0; p < n_planes; ++p) {
        const fc_plane_bc& pl = planes[p];
        if (pl.axis != planes[0].axis) return FC_ERR_ARG;            // one axis ...
        for (int r = 0; r < p; ++r)
            if (planes[r].plane_idx == pl.plane_idx) return FC_ERR_ARG;   // ... distinct planes
        if (pl.bc_type != 0 && pl.bc_type != 1) return FC_ERR_ARG;
        if (plane_dims(pl.axis, a.g.nx, a.g.ny, a.g.nz, &ps.n1[p], &ps.n2[p])) return FC_ERR_ARG;
        const int na = pl.axis == 0 ? a.g.nx : (pl.axis == 1 ? a.g.ny : a.g.nz);
        if (pl.plane_idx < 0 || pl.plane_idx >= na || pl.interior_idx < 0 || pl.interior_idx >= na) return FC_ERR_ARG;
        ps.p[p] = pl;
        ps.start[p + 1] = ps.start[p] + ps.n1[p] * ps.n2[p];
    }
    // a plane whose condition reads a neighbour plane that another condition writes needs the
    // sequential order: not fused
    for (int p = 0; p < n_planes; ++p)
        for (int r = 0; r < n_planes; ++r)
            if (planes[p].interior_idx == planes[r].plane_idx) return FC_ERR_UNSUPPORTED;
#define FC_PCASE(S, M) \
    if (args->storage == S && args->collision == M) return planes_dispatch<S, M>(a, (cudaStream_t)stream, ps);
    FC_PCASE(ST_F32, CM_BGK) FC_PCASE(ST_F32, CM_TRT) FC_PCASE(ST_F32, CM_MRT) FC_PCASE(ST_F32, CM_MRT_SMAG)
    FC_PCASE(ST_F16S, CM_BGK) FC_PCASE(ST_F16S, CM_TRT) FC_PCASE(ST_F16S, CM_MRT) FC_PCASE(ST_F16S, CM_MRT_SMAG)
    FC_PCASE(ST_BF16S, CM_BGK) FC_PCASE(ST_BF16S, CM_TRT) FC_PCASE(ST_BF16S, CM_MRT) FC_PCASE(ST_BF16S, CM_MRT_SMAG)
#undef FC_PCASE
    return FC_ERR_ARG;
}

int fc_lbm_collide_from_f32(const fc_lbm_step_args* args, int axis, int plane_idx, void* stream) {
    FusedArgs a;
    int rc = make_fused_args(args, a);
    if (rc) return rc;
    if (!a.f32 || !args->pop_out) return FC_ERR_ARG;
    int n1 = 0, n2 = 0;
    if (axis >= 0) {
        if (plane_dims(axis, a.g.nx, a.g.ny, a.g.nz, &n1, &n2)) return FC_ERR_ARG;
        const int na = axis == 0 ? a.g.nx : (axis == 1 ? a.g.ny : a.g.nz);
        if (plane_idx < 0 || plane_idx >= na) return FC_ERR_ARG;
    }
    return dispatch<CollideF32Launcher>(args->storage, args->collision, a, (cudaStream_t)stream, axis,
                                        plane_idx, n1, n2);
}

int fc_lbm_materialize(const fc_lbm_step_args* args, void* stream) {
    FusedArgs a;
    int rc = make_fused_args(args, a);
    if (rc) return rc;
    a.link_val = nullptr;   // links evaluated from pop_in itself, independent of the last gather
    if (!a.f32 || !args->pop_in) return FC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    switch (args->storage) {
        case ST_F32: k_materialize<ST_F32><<<cell_grid(a.g), dim3(TBX, TBY), 0, st>>>(a); break;
        case ST_F16S: k_materialize<ST_F16S><<<cell_grid(a.g), dim3(TBX, TBY), 0, st>>>(a); break;
        default: k_materialize<ST_BF16S><<<cell_grid(a.g), dim3(TBX, TBY), 0, st>>>(a); break;
    }
    return launch_status();
}

int fc_lbm_pin_solid(const fc_lbm_step_args* args, void* stream) {
    FusedArgs a;
    int rc = make_fused_args(args, a);
    if (rc) return rc;
    if (!args->pop_out) return FC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    switch (args->storage) {
        case ST_F32: k_pin_solid<ST_F32><<<grid_for(a.g.N), BLOCK, 0, st>>>(a); break;
        case ST_F16S: k_pin_solid<ST_F16S><<<grid_for(a.g.N), BLOCK, 0, st>>>(a); break;
        default: k_pin_solid<ST_BF16S><<<grid_for(a.g.N), BLOCK, 0, st>>>(a); break;
    }
    return launch_status();
}

}  // extern "C"
