// fc_conv.cu -- BF16 implicit-GEMM 3-D convolutions on the 5th-generation tensor
// cores (tcgen05 + TMEM) for the learned thermal preconditioner.
//
// One engine, three loaders:
//   forward  Y[v][n]        = sum_{tap,c} X[v + o(tap)][c] W[n][tap][c]      (M = voxels, N = C_out)
//   data grad dX[v][c]      = sum_{tap,n} dY[v - o(tap)][n] W[n][tap][c]     (forward with flipped, transposed W)
//   weight grad dW[n][tap][c] = sum_v X[v + o(tap)][c] dY[v][n]             (M = 27 C_in, N = C_out, K = voxels, split-K)
// Activations are channels-last BF16 [B][D][H][W][C] (C a multiple of 8, zero
// padding outside each volume), weights BF16 [C_out][K_pad] with K = 27 C_in
// (tap-major) padded to a multiple of 64.
//
// Per CTA: a 128-row tile of D (M = 128) in TMEM (FP32, N columns); the K loop
// runs in 64-wide chunks through two shared-memory stages: all 128 threads
// gather the next chunk (16-byte rows of the canonical no-swizzle K-major
// layout: 8x16-byte core matrices) while the tensor core consumes the current
// one; one elected thread issues 4 x tcgen05.mma (K = 16 each) per chunk and
// commits them to the stage's mbarrier.  Every mbarrier wait is bounded: on
// timeout the CTA records an error bit, stops issuing and still releases TMEM.
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int TM = 128;       // rows per CTA tile
constexpr int KC = 64;        // K per chunk (4 MMAs of K = 16)
constexpr int NTHR = 128;
constexpr int STAGES = 2;     // shared-memory stages of the K loop (3 measured slower: fewer CTAs per SM)
constexpr unsigned SPIN_LIMIT = 1u << 26;

struct ConvGeom {
    int B, D, H, W;      // batch and volume extents (voxels = B*D*H*W)
    int cin, cout;       // channels (cin, cout multiples of 8)
    int kpad;            // padded K of the weights (multiple of 64)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version for tcgen05
    return d;                 // base offset 0, relative LBO, no swizzle
}

__device__ __forceinline__ uint32_t make_idesc(int M, int N) {
    return (1u << 4)                      // D: FP32
         | (1u << 7)                      // A: BF16
         | (1u << 10)                     // B: BF16
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16   (A, B K-major)
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned it = 0; it < SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity));
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// --------------------------------------------------------------------------
// operand loaders.  Each returns 8 consecutive K elements (one 16-byte row of
// a core matrix).  A loaders fill one tile row per thread (NTHR == TM): row()
// decodes the row once per tile and chunk() fills the row's 8 vectors of one
// 64-wide K chunk, so no chunk repeats the voxel decomposition.
// --------------------------------------------------------------------------
__device__ __forceinline__ void tap_offsets(int tap, int& dz, int& dy, int& dx) {
    dz = tap / 9 - 1;
    dy = (tap / 3) % 3 - 1;
    dx = tap % 3 - 1;
}

// forward / data-grad A: activations of the neighbour voxel v + o(tap), K = (tap, channel block)
struct LoadActA {
    const __nv_bfloat16* X;
    ConvGeom g;
    int cin;
    int nvox;
    struct Row {
        int v, d, h, w;
        bool ok;
    };
    __device__ Row row(int m) const {
        Row r;
        r.v = m;
        r.ok = m < nvox;
        r.w = m % g.W;
        r.h = (m / g.W) % g.H;
        r.d = (m / (g.W * g.H)) % g.D;
        return r;
    }
    __device__ void chunk(const Row& r, int k8_0, uint4 out[KC / 8]) const {
        const uint4 z = make_uint4(0, 0, 0, 0);
        const int cb = cin >> 3;
        int tap = k8_0 / cb;
        int cc = k8_0 - tap * cb;
        int dz, dy, dx;
        tap_offsets(tap, dz, dy, dx);
        bool in = r.ok && tap < 27 && (unsigned)(r.d + dz) < (unsigned)g.D && (unsigned)(r.h + dy) < (unsigned)g.H &&
                  (unsigned)(r.w + dx) < (unsigned)g.W;
        long long base = (long long)(r.v + (dz * g.H + dy) * g.W + dx) * cin;
#pragma unroll
        for (int kb = 0; kb < KC / 8; ++kb) {
            out[kb] = in ? __ldg(reinterpret_cast<const uint4*>(X + base + cc * 8)) : z;
            if (++cc == cb) {
                cc = 0;
                ++tap;
                tap_offsets(tap, dz, dy, dx);
                in = r.ok && tap < 27 && (unsigned)(r.d + dz) < (unsigned)g.D &&
                     (unsigned)(r.h + dy) < (unsigned)g.H && (unsigned)(r.w + dx) < (unsigned)g.W;
                base = (long long)(r.v + (dz * g.H + dy) * g.W + dx) * cin;
            }
        }
    }
};
// weights [rows][kpad]
struct LoadRowsB {
    const __nv_bfloat16* Wt;
    int rows, kpad;
    __device__ uint4 operator()(int n, int k8) const {
        if (n >= rows) return make_uint4(0, 0, 0, 0);
        return __ldg(reinterpret_cast<const uint4*>(Wt + (long long)n * kpad + k8 * 8));
    }
};
// weight-grad A: rows m = tap*cin + c, K = voxels
struct LoadWgradA {
    const __nv_bfloat16* X;
    ConvGeom g;
    int nvox;
    struct Row {
        int c, dz, dy, dx;
        bool ok;
    };
    __device__ Row row(int m) const {
        Row r;
        const int tap = m / g.cin;
        r.c = m - tap * g.cin;
        r.ok = tap < 27;
        tap_offsets(tap < 27 ? tap : 0, r.dz, r.dy, r.dx);
        return r;
    }
    // the 64 voxels k8_0*8 .. k8_0*8+63 in order: decode the first, then step w with carries
    __device__ void chunk(const Row& r, int k8_0, uint4 out[KC / 8]) const {
        int v = k8_0 * 8;
        int w = v % g.W, h = (v / g.W) % g.H, d = (v / (g.W * g.H)) % g.D;
        const int off = (r.dz * g.H + r.dy) * g.W + r.dx;
#pragma unroll
        for (int kb = 0; kb < KC / 8; ++kb) {
            __align__(16) __nv_bfloat16 e[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const bool in = r.ok && v < nvox && (unsigned)(d + r.dz) < (unsigned)g.D &&
                                (unsigned)(h + r.dy) < (unsigned)g.H && (unsigned)(w + r.dx) < (unsigned)g.W;
                e[t] = in ? X[(long long)(v + off) * g.cin + r.c] : __float2bfloat16(0.f);
                ++v;
                if (++w == g.W) {
                    w = 0;
                    if (++h == g.H) {
                        h = 0;
                        if (++d == g.D) d = 0;
                    }
                }
            }
            out[kb] = *reinterpret_cast<uint4*>(e);
        }
    }
};
// weight-grad B: rows n, K = voxels: dY[v][n]
struct LoadWgradB {
    const __nv_bfloat16* dY;
    int cout, nvox;
    __device__ uint4 operator()(int n, int k8) const {
        __align__(16) __nv_bfloat16 e[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int v = k8 * 8 + t;
            e[t] = (n < cout && v < nvox) ? dY[(long long)v * cout + n] : __float2bfloat16(0.f);
        }
        return *reinterpret_cast<uint4*>(e);
    }
};

// --------------------------------------------------------------------------
// engine
// --------------------------------------------------------------------------
struct Epi {
    float* out_f32;              // [rows][ldo] FP32 (or NULL)
    __nv_bfloat16* out_bf16;     // [rows][ldo] BF16 (or NULL)
    const float* bias;           // [N] or NULL
    int relu;
    int ldo;                     // leading dimension of the output rows
    int nvalid;                  // columns actually stored
    int rows;                    // rows actually stored
    long long row_offset;        // added to the row index (split-K partial slabs)
};

template <class LA, class LB>
__device__ void gemm_tile(const LA& la, const LB& lb, int m0, int N, int k8_begin, int nchunks, const Epi& ep,
                          unsigned* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // layout: STAGES x [A | B] then STAGES mbarriers + tmem slot
    const int a_bytes = TM * KC * 2;
    const int b_bytes = N * KC * 2;
    const int stage_bytes = a_bytes + b_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + STAGES);
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    int ncols = 32;
    while (ncols < N) ncols <<= 1;

    if (tid == 0) {
        for (int b = 0; b < STAGES; ++b) mbar_init(&bars[b], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = make_idesc(TM, N);
    static_assert(NTHR == TM, "one A row per thread");
    const typename LA::Row ra = la.row(m0 + tid);

    for (int c = 0; c < nchunks; ++c) {
        const int s = c % STAGES;
        unsigned char* As = smem + s * stage_bytes;
        unsigned char* Bs = As + a_bytes;
        if (c >= STAGES) {
            if (!mbar_wait(&bars[s], ((c - STAGES) / STAGES) & 1)) {
                if (err) atomicOr(err, 4u);
                s_abort = 1;
            }
        }
        __syncthreads();
        if (s_abort) break;
        // gather: A rows [TM] x 8 core columns; core (mb, kb) at kb*(TM/8)*128 + mb*128 + (row%8)*16;
        // thread tid fills row tid
        {
            uint4 v[KC / 8];
            la.chunk(ra, k8_begin + c * (KC / 8), v);
#pragma unroll
            for (int kb = 0; kb < KC / 8; ++kb)
                *reinterpret_cast<uint4*>(As + kb * (TM / 8) * 128 + (tid >> 3) * 128 + (tid & 7) * 16) = v[kb];
        }
        for (int t = tid; t < N * (KC / 8); t += NTHR) {
            const int row = t % N, kb = t / N;
            const uint4 v = lb(row, k8_begin + c * (KC / 8) + kb);
            *reinterpret_cast<uint4*>(Bs + kb * (N / 8) * 128 + (row >> 3) * 128 + (row & 7) * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a0 = smem_u32(As), b0 = smem_u32(Bs);
#pragma unroll
            for (int kk = 0; kk < KC / 16; ++kk) {
                // K = 16 spans two core columns: start at core column 2*kk
                const uint64_t da = make_desc(a0 + 2 * kk * (TM / 8) * 128, (TM / 8) * 128, 128);
                const uint64_t db = make_desc(b0 + 2 * kk * (N / 8) * 128, (N / 8) * 128, 128);
                mma_bf16(tmem, da, db, idesc, (c > 0 || kk > 0) ? 1 : 0);
            }
            mma_commit(&bars[s]);
        }
    }
    // wait for the last chunk's MMAs (commit covers all earlier ones)
    if (!s_abort && nchunks > 0) {
        const int c = nchunks - 1;
        if (!mbar_wait(&bars[c % STAGES], (c / STAGES) & 1)) {
            if (err) atomicOr(err, 4u);
            s_abort = 1;
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (!s_abort && nchunks > 0) {
        // epilogue: warp w owns TMEM lanes 32w..32w+31 == tile rows
        const int row = m0 + warp * 32 + (tid & 31);
        for (int n0 = 0; n0 < N; n0 += 8) {
            uint32_t r[8];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < ep.rows) {
                float v[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    v[t] = __uint_as_float(r[t]);
                    if (ep.bias && n0 + t < ep.nvalid) v[t] += ep.bias[n0 + t];
                    if (ep.relu) v[t] = fmaxf(v[t], 0.f);
                }
                const long long o = (ep.row_offset + row) * (long long)ep.ldo + n0;
                if (n0 + 8 <= ep.nvalid && (ep.ldo & 7) == 0) {
                    // 16-byte stores of whole 8-column groups (rows are 16-byte aligned)
                    if (ep.out_f32) {
                        *reinterpret_cast<float4*>(ep.out_f32 + o) = make_float4(v[0], v[1], v[2], v[3]);
                        *reinterpret_cast<float4*>(ep.out_f32 + o + 4) = make_float4(v[4], v[5], v[6], v[7]);
                    }
                    if (ep.out_bf16) {
                        __align__(16) __nv_bfloat162 b[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t) b[t] = __floats2bfloat162_rn(v[2 * t], v[2 * t + 1]);
                        *reinterpret_cast<uint4*>(ep.out_bf16 + o) = *reinterpret_cast<const uint4*>(b);
                    }
                } else {
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        if (n0 + t >= ep.nvalid) continue;
                        if (ep.out_f32) ep.out_f32[o + t] = v[t];
                        if (ep.out_bf16) ep.out_bf16[o + t] = __float2bfloat16_rn(v[t]);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
    }
}

__global__ void __launch_bounds__(NTHR) k_conv_fwd(LoadActA la, LoadRowsB lb, int N, int nchunks, Epi ep,
                                                   unsigned* err) {
    gemm_tile(la, lb, blockIdx.x * TM, N, 0, nchunks, ep, err);
}

__global__ void __launch_bounds__(NTHR) k_conv_wgrad(LoadWgradA la, LoadWgradB lb, int N, int chunks_per_split,
                                                     Epi ep, unsigned* err) {
    Epi e = ep;
    e.row_offset = (long long)blockIdx.y * e.rows;   // partial slab of this split
    gemm_tile(la, lb, blockIdx.x * TM, N, blockIdx.y * chunks_per_split * (KC / 8), chunks_per_split, e, err);
}

// dW[n][m] = sum_split partial[split][m][n]  (m < 27 cin), then cast to the padded BF16 K layout on demand
__global__ void k_wgrad_reduce(const float* __restrict__ part, int splits, int mrows, int mvalid, int n,
                               float* __restrict__ dW, int kpad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mvalid * n) return;
    const int m = t / n, c = t - (t / n) * n;
    float s = 0.f;
    for (int p = 0; p < splits; ++p) s += part[((long long)p * mrows + m) * n + c];
    dW[(long long)c * kpad + m] = s;
}

// W'[c][tap'][n] = W[n][26 - tap'][c]  (data-gradient weights)
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ W, __nv_bfloat16* __restrict__ Wf, int cout,
                               int cin, int kpad_in, int kpad_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cin * kpad_out) return;
    const int c = t / kpad_out, kk = t - c * kpad_out;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (kk < 27 * cout) {
        const int tap = kk / cout, n = kk - tap * cout;
        v = W[(long long)n * kpad_in + (26 - tap) * cin + c];
    }
    Wf[t] = v;
}

inline size_t smem_bytes(int N) {
    // the stages + barriers (+ 1 KB of slack).  Every operand read of the MMAs stays inside its
    // stage: an A read spans 15 SBO (128 B) + 1 LBO (2 KB) + 128 B from its start, the last one
    // ending at the stage's A size; B likewise ends at N x 128 B.  (A 32 KB slack, which held
    // residency to 2 CTAs per SM, measured 5-35 % slower.)
    size_t b = STAGES * (size_t)(TM * KC * 2 + N * KC * 2) + 8 * (STAGES + 1) + 1024;
    int ncols = 32;
    while (ncols < N) ncols <<= 1;
    // keep (CTAs per SM) x ncols <= 512 TMEM columns: make the smem footprint cap residency
    const size_t per_sm = 232448;
    const size_t max_ctas = 512 / ncols;
    const size_t need = per_sm / max_ctas + 1;
    return b > need ? b : need;
}

}  // namespace

extern "C" {

int fc_conv3d_fwd(const void* X, const void* Wt, const float* bias, int B, int D, int H, int W, int cin, int cout,
                  int kpad, int relu, float* Y_f32, void* Y_bf16, unsigned* dev_err, void* stream) {
    if (!X || !Wt || (!Y_f32 && !Y_bf16)) return FC_ERR_ARG;
    if (cin % 8 || cout % 16 || cout < 16 || cout > 256 || kpad % KC || kpad < 27 * cin) return FC_ERR_ARG;
    if (B < 1 || D < 1 || H < 1 || W < 1) return FC_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(Wt)) & 15) return FC_ERR_ARG;
    const long long nvox = (long long)B * D * H * W;
    if (nvox >= (1LL << 31)) return FC_ERR_UNSUPPORTED;
    ConvGeom g{B, D, H, W, cin, cout, kpad};
    LoadActA la{reinterpret_cast<const __nv_bfloat16*>(X), g, cin, (int)nvox};
    LoadRowsB lb{reinterpret_cast<const __nv_bfloat16*>(Wt), cout, kpad};
    Epi ep{Y_f32, reinterpret_cast<__nv_bfloat16*>(Y_bf16), bias, relu, cout, cout, (int)nvox, 0};
    const size_t sm = smem_bytes(cout);
    cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    const unsigned grid = (unsigned)((nvox + TM - 1) / TM);
    k_conv_fwd<<<grid, NTHR, sm, (cudaStream_t)stream>>>(la, lb, cout, kpad / KC, ep, dev_err);
    return launch_status();
}

// data gradient: dX[v][c] (FP32 and/or BF16) from dY[v][n] and W[n][kpad]; Wflip workspace: cin x kpad_t BF16
long long fc_conv3d_dgrad_workspace_bytes(int cin, int cout) {
    const long long kp = ((27LL * cout + KC - 1) / KC) * KC;
    return (long long)cin * kp * 2;
}

int fc_conv3d_dgrad(const void* dY, const void* Wt, int B, int D, int H, int W, int cin, int cout, int kpad,
                    void* workspace, long long workspace_bytes, float* dX_f32, void* dX_bf16, unsigned* dev_err,
                    void* stream) {
    if (!dY || !Wt || !workspace || (!dX_f32 && !dX_bf16)) return FC_ERR_ARG;
    if (cin % 16 || cin < 16 || cout % 8 || kpad < 27 * cin) return FC_ERR_ARG;
    if (workspace_bytes < fc_conv3d_dgrad_workspace_bytes(cin, cout)) return FC_ERR_ARG;
    const int kp_t = (int)(((27LL * cout + KC - 1) / KC) * KC);
    cudaStream_t st = (cudaStream_t)stream;
    __nv_bfloat16* Wf = reinterpret_cast<__nv_bfloat16*>(workspace);
    k_flip_weights<<<(cin * kp_t + 255) / 256, 256, 0, st>>>(reinterpret_cast<const __nv_bfloat16*>(Wt), Wf, cout,
                                                             cin, kpad, kp_t);
    int rc = launch_status();
    if (rc) return rc;
    const long long nvox = (long long)B * D * H * W;
    ConvGeom g{B, D, H, W, cout, cin, kp_t};
    LoadActA la{reinterpret_cast<const __nv_bfloat16*>(dY), g, cout, (int)nvox};
    // the flipped taps make the forward gather of dY at v + o(tap') equal dY at v - o(tap)
    LoadRowsB lb{Wf, cin, kp_t};
    Epi ep{dX_f32, reinterpret_cast<__nv_bfloat16*>(dX_bf16), nullptr, 0, cin, cin, (int)nvox, 0};
    const size_t sm = smem_bytes(cin);
    cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_conv_fwd<<<(unsigned)((nvox + TM - 1) / TM), NTHR, sm, st>>>(la, lb, cin, kp_t / KC, ep, dev_err);
    return launch_status();
}

long long fc_conv3d_wgrad_workspace_bytes(int B, int D, int H, int W, int cin, int cout, int splits) {
    const long long mrows = ((27LL * cin + TM - 1) / TM) * TM;
    return (long long)splits * mrows * cout * 4;
}

// weight gradient: dW[n][kpad] FP32 (columns >= 27 cin untouched) from X[v][cin], dY[v][cout]
int fc_conv3d_wgrad(const void* X, const void* dY, int B, int D, int H, int W, int cin, int cout, int kpad,
                    int splits, void* workspace, long long workspace_bytes, float* dW, unsigned* dev_err,
                    void* stream) {
    if (!X || !dY || !dW || !workspace || splits < 1) return FC_ERR_ARG;
    if (cin % 8 || cout % 16 || cout < 16 || cout > 256 || kpad < 27 * cin) return FC_ERR_ARG;
    if (workspace_bytes < fc_conv3d_wgrad_workspace_bytes(B, D, H, W, cin, cout, splits)) return FC_ERR_ARG;
    const long long nvox = (long long)B * D * H * W;
    const long long k8_total = (nvox + 7) / 8;
    const long long chunks = (k8_total + (KC / 8) - 1) / (KC / 8);
    const int cps = (int)((chunks + splits - 1) / splits);
    const int mrows = (int)(((27LL * cin + TM - 1) / TM) * TM);
    ConvGeom g{B, D, H, W, cin, cout, kpad};
    LoadWgradA la{reinterpret_cast<const __nv_bfloat16*>(X), g, (int)nvox};
    LoadWgradB lb{reinterpret_cast<const __nv_bfloat16*>(dY), cout, (int)nvox};
    float* part = reinterpret_cast<float*>(workspace);
    Epi ep{part, nullptr, nullptr, 0, cout, cout, mrows, 0};
    const size_t sm = smem_bytes(cout);
    cudaStream_t st = (cudaStream_t)stream;
    cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    dim3 grid(mrows / TM, splits);
    k_conv_wgrad<<<grid, NTHR, sm, st>>>(la, lb, cout, cps, ep, dev_err);
    int rc = launch_status();
    if (rc) return rc;
    const int mvalid = 27 * cin;
    k_wgrad_reduce<<<(mvalid * cout + 255) / 256, 256, 0, st>>>(part, splits, mrows, mvalid, cout, dW, kpad);
    return launch_status();
}

}  // extern "C"
