// fc_geom.cu -- geometry set-up for interpolated bounce-back, on the device.
//
//  * fc_geom_signed_edt: the signed Euclidean distance of a voxel mask
//    (positive in fluid, negative in solid, times the pitch), the field that
//    build_phi_from_voxel_mask_mm (pre_post/sdf_tracing.py:312-340) computes on
//    the host with scipy.ndimage.distance_transform_edt.
//  * fc_ibb_count_links / fc_ibb_build_links: the boundary-link list of
//    build_links_from_mask_gpu (sdf_tracing.py:20-85), in its order.
//  * fc_ibb_q_from_sdf: the Bouzidi fractions of bfl_q_from_sdf and
//    sdf_trilinear (sdf_tracing.py:89-184) and the weights of
//    bfl_weights_from_q (sdf_tracing.py:188-205), one thread per link.
//
// Distance transform.  The squared distance from a cell to the nearest cell of
// the other kind separates by axes:
//     D(i,j,k) = min_i' [ min_j' [ min_k' (k-k')^2 ] + (j-j')^2 ] + (i-i')^2
// over cells (i',j',k') of the other kind (Saito-Toriwaki).  The two transforms
// of the signed field -- fluid cells to the nearest solid cell, solid cells to
// the nearest fluid cell -- run together in one int32 per cell: after every
// pass a cell holds its own kind's value, and the other transform is 0 at that
// cell because the cell is one of its features.
//   pass z (contiguous rows): one warp per row.  Ballots of the two kinds,
//     32 cells at a time, give each lane the last and the next cell of the
//     other kind, so a row costs two sweeps over its 32-cell chunks.
//   passes y and x: a block stages KW columns of whole lines in shared memory;
//     each cell scans outward, r = 1, 2, ..., while r^2 is below the best value
//     found, which is exact (a farther cell adds at least r^2) and costs about
//     the distance found.
// Squared distances are exact integers.  The last pass takes their square
// root in FP64 and multiplies by the pitch in FP64 before rounding to FP32:
// numpy's sqrt of the exact integer sum, then the product, then the cast, as
// the host path does, so phi is the same FP32 value bit for bit.  When the mask
// holds no cell of the other kind at all, scipy's feature transform reports
// the point (-1, 0, 0) for every cell; the last pass reproduces that distance.
//
// Link order.  A link is a fluid cell x whose neighbour x + c_q (q = 1..18,
// no wrap) is solid.  The list is grouped by q and row-major inside each q.
// Blocks of 1024 cells count their links per q, a two-level scan turns the
// counts (q-major, so the offsets follow the list order) into offsets, and the
// write pass places every link at its block offset plus its rank inside the
// block (warp ballots).
//
// Fractions.  FP32, every operation rounded on its own as the reference's
// elementwise tensor operations are (no contraction).  sdf_trilinear's
// (x - origin) / dx divides a tensor by a host scalar: on a CUDA device torch
// multiplies by the scalar's FP32 reciprocal, on the CPU it divides.  true_div
// selects the CPU form; the default (0) is the CUDA form the reference's GPU
// run computes.  The two agree whenever dx is a power of two.
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int EDT_INF = 0x3fffffff;   // no cell of the other kind on the line so far
constexpr int EDT_FAR = 1 << 28;      // sentinel position for "none before / after"
constexpr int ROW_WARPS = 8;
constexpr int EDT_MAX_NZ = 4096;      // z pass: 128 chunks of ballots per warp in shared memory
constexpr int LINE_THREADS = 256;
constexpr int LINE_SMEM = 96 * 1024;  // y / x pass staging budget per block
constexpr int EDT_MAX_LINE = 4096;    // y / x lines: KW = 4 columns of 4096 cells fit the budget

// ---------------------------------------------------------------------------
// pass z: 1-D squared distance to the nearest cell of the other kind in the row
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(ROW_WARPS * 32)
k_edt_rows(const uint8_t* __restrict__ solid, int* __restrict__ g, long long nrows, int nz, int nch) {
    extern __shared__ unsigned edt_sh[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned* bS = edt_sh + (size_t)warp * 4 * nch;  // solid ballots per chunk
    unsigned* bF = bS + nch;                          // fluid ballots per chunk
    int* pS = (int*)(bF + nch);                       // last solid before the chunk
    int* pF = pS + nch;                               // last fluid before the chunk
    const long long stride = (long long)gridDim.x * ROW_WARPS;
    for (long long r = (long long)blockIdx.x * ROW_WARPS + warp; r < nrows; r += stride) {
        const uint8_t* row = solid + r * nz;
        int* out = g + r * nz;
        int lastS = -EDT_FAR, lastF = -EDT_FAR;
        for (int c = 0; c < nch; ++c) {
            const int k = c * 32 + lane;
            const bool in = k < nz;
            const bool s = in && row[k] != 0;
            const unsigned ws = __ballot_sync(FULL, s);
            const unsigned wf = __ballot_sync(FULL, in && !s);
            if (lane == 0) {
                bS[c] = ws;
                bF[c] = wf;
                pS[c] = lastS;
                pF[c] = lastF;
            }
            if (ws) lastS = c * 32 + 31 - __clz(ws);
            if (wf) lastF = c * 32 + 31 - __clz(wf);
        }
        __syncwarp();
        int nextS = EDT_FAR, nextF = EDT_FAR;
        for (int c = nch - 1; c >= 0; --c) {
            const unsigned ws = bS[c], wf = bF[c];
            const int k = c * 32 + lane;
            if (k < nz) {
                const bool s = (ws >> lane) & 1u;
                const unsigned other = s ? wf : ws;
                const unsigned le = other & (FULL >> (31 - lane));
                const unsigned ge = other & (FULL << lane);
                const int last = le ? c * 32 + 31 - __clz(le) : (s ? pF[c] : pS[c]);
                const int next = ge ? c * 32 + __ffs(ge) - 1 : (s ? nextF : nextS);
                int v = EDT_INF;
                if (last >= 0 || next < nz) {
                    const int d = min(k - last, next - k);
                    v = d * d;
                }
                out[k] = v;
            }
            if (ws) nextS = c * 32 + __ffs(ws) - 1;
            if (wf) nextF = c * 32 + __ffs(wf) - 1;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// passes y and x: min over the line of g(y) + (x - y)^2, in place; the x pass
// (FINAL) writes the signed FP32 distance instead.
//
// A cell first checks the cells within EDT_NEAR of it one by one, then walks
// outward block by block (EDT_BS cells): a block whose minimum value plus the
// squared distance to its nearest cell is not below the best so far is
// skipped whole, and the walk stops once that squared distance alone reaches
// it.  Both bounds are exact, so the result is the exact minimum; in open
// regions, where the values vary slowly along the line, a cell far from the
// wall costs a few block tests instead of a scan out to its distance.
// ---------------------------------------------------------------------------
constexpr int EDT_BS = 16;
constexpr int EDT_NEAR = 4;
constexpr int SQRT_TAB = 1 << 18;   // FP32 phi magnitudes of d^2 < 2^18 (distances below 512 cells)

__device__ __forceinline__ int g_of(unsigned w, unsigned kind) {
    return (w >> 31) != kind ? 0 : (int)(w & 0x7fffffffu);
}

__host__ __device__ constexpr long long line_smem_bytes(int L, int kw) {
    return 4LL * kw * ((long long)L + 2LL * ((L + EDT_BS - 1) / EDT_BS));
}

template <int KW, bool FINAL>
__global__ void __launch_bounds__(LINE_THREADS)
k_edt_lines(const uint8_t* __restrict__ solid, int* __restrict__ g, float* __restrict__ phi,
            const float* __restrict__ tab, int L, long long lstride, long long ostride, int nz, double pitch) {
    extern __shared__ unsigned edt_sh[];
    constexpr int RP = LINE_THREADS / KW;
    const int NB = (L + EDT_BS - 1) / EDT_BS;
    unsigned* sv = edt_sh;                          // [y][column]: value | kind << 31
    int* bm = (int*)(edt_sh + (size_t)L * KW);      // [kind][block][column]: block minima
    const int c = threadIdx.x % KW, xr = threadIdx.x / KW;
    const int k = blockIdx.x * KW + c;
    const bool col = k < nz;
    const long long base = (long long)blockIdx.y * ostride + k;
    if (col) {
        for (int x = xr; x < L; x += RP) {
            const long long cell = base + x * lstride;
            sv[x * KW + c] = (unsigned)g[cell] | (solid[cell] ? 0x80000000u : 0u);
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < NB * KW; p += LINE_THREADS) {
        const int b = p / KW, cc = p % KW;
        int m0 = EDT_INF, m1 = EDT_INF;
        if ((int)blockIdx.x * KW + cc < nz) {
            const int y1 = min(L, (b + 1) * EDT_BS);
            for (int y = b * EDT_BS; y < y1; ++y) {
                const unsigned w = sv[y * KW + cc];
                const int v = (int)(w & 0x7fffffffu);
                if (w >> 31) {
                    m0 = 0;
                    m1 = min(m1, v);
                } else {
                    m1 = 0;
                    m0 = min(m0, v);
                }
            }
        }
        bm[b * KW + cc] = m0;
        bm[(NB + b) * KW + cc] = m1;
    }
    __syncthreads();
    if (!col) return;
    for (int x = xr; x < L; x += RP) {
        const unsigned own = sv[x * KW + c];
        const unsigned kind = own >> 31;
        const int* bmk = bm + (size_t)kind * NB * KW + c;
        int best = (int)(own & 0x7fffffffu);
        for (int r = 1; r <= EDT_NEAR; ++r) {
            const int rr = r * r;
            if (rr >= best) break;
            if (x - r >= 0) best = min(best, g_of(sv[(x - r) * KW + c], kind) + rr);
            if (x + r < L) best = min(best, g_of(sv[(x + r) * KW + c], kind) + rr);
        }
        for (int yl = x - EDT_NEAR - 1; yl >= 0;) {
            const int d = x - yl;
            if (d * d >= best) break;
            const int y0 = (yl / EDT_BS) * EDT_BS;
            if (bmk[(yl / EDT_BS) * KW] + d * d < best) {
                for (int y = yl; y >= y0; --y) {
                    const int dd = (x - y) * (x - y);
                    if (dd >= best) break;
                    best = min(best, g_of(sv[y * KW + c], kind) + dd);
                }
            }
            yl = y0 - 1;
        }
        for (int yr = x + EDT_NEAR + 1; yr < L;) {
            const int d = yr - x;
            if (d * d >= best) break;
            const int y1 = min(L, (yr / EDT_BS + 1) * EDT_BS);
            if (bmk[(yr / EDT_BS) * KW] + d * d < best) {
                for (int y = yr; y < y1; ++y) {
                    const int dd = (y - x) * (y - x);
                    if (dd >= best) break;
                    best = min(best, g_of(sv[y * KW + c], kind) + dd);
                }
            }
            yr = y1;
        }
        const long long cell = base + x * lstride;
        if constexpr (FINAL) {
            // x pass: x is i, blockIdx.y is j
            float v;
            if (best < SQRT_TAB) {
                v = __ldg(tab + best);
            } else {
                double d2;
                if (best < EDT_INF) {
                    d2 = (double)best;
                } else {
                    const double a = (double)(x + 1), b = (double)blockIdx.y, e = (double)k;
                    d2 = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(e, e));
                }
                v = __double2float_rn(__dmul_rn(__dsqrt_rn(d2), pitch));
            }
            phi[cell] = kind ? -v : v;
        } else {
            g[cell] = best;
        }
    }
}

// tab[d2] = float(double(sqrt(d2)) * pitch): numpy's FP64 sqrt and product, then the cast
__global__ void __launch_bounds__(256) k_edt_sqrt_table(float* __restrict__ tab, double pitch) {
    const int d2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (d2 < SQRT_TAB) tab[d2] = __double2float_rn(__dmul_rn(__dsqrt_rn((double)d2), pitch));
}

template <bool FINAL>
int launch_lines(const uint8_t* solid, int* g, float* phi, const float* tab, int L, long long lstride,
                 long long ostride, int n_outer, int nz, double pitch, cudaStream_t st) {
    int kw = 32;
    while (kw > 4 && line_smem_bytes(L, kw) > LINE_SMEM) kw >>= 1;
    if (line_smem_bytes(L, kw) > LINE_SMEM) return FC_ERR_UNSUPPORTED;
    const size_t smem = (size_t)line_smem_bytes(L, kw);
    const dim3 grid((unsigned)((nz + kw - 1) / kw), (unsigned)n_outer);
    auto run = [&](auto kern) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, LINE_THREADS, smem, st>>>(solid, g, phi, tab, L, lstride, ostride, nz, pitch);
    };
    switch (kw) {
        case 32: run(k_edt_lines<32, FINAL>); break;
        case 16: run(k_edt_lines<16, FINAL>); break;
        case 8: run(k_edt_lines<8, FINAL>); break;
        default: run(k_edt_lines<4, FINAL>); break;
    }
    return launch_status();
}

// ---------------------------------------------------------------------------
// boundary links
// ---------------------------------------------------------------------------
constexpr int LB_THREADS = 256, LB_ROUNDS = 4, LB_CELLS = LB_THREADS * LB_ROUNDS;

struct Dims {
    int nx, ny, nz;
    long long nyz, N;
};

// bit q set: cell is fluid and its in-box neighbour along c_q is solid
__device__ __forceinline__ unsigned link_mask(const uint8_t* __restrict__ solid, const Dims& d, long long cell, int& i,
                                              int& j, int& k) {
    i = j = k = 0;
    if (cell >= d.N || solid[cell]) return 0u;
    i = (int)(cell / d.nyz);
    const int rem = (int)(cell - (long long)i * d.nyz);
    j = rem / d.nz;
    k = rem - j * d.nz;
    unsigned m = 0;
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        const int a = i + cx(q), b = j + cy(q), e = k + cz(q);
        if (a >= 0 && a < d.nx && b >= 0 && b < d.ny && e >= 0 && e < d.nz &&
            solid[cell + (long long)cx(q) * d.nyz + cy(q) * d.nz + cz(q)])
            m |= 1u << q;
    }
    return m;
}

__global__ void __launch_bounds__(LB_THREADS)
k_links_count(const uint8_t* __restrict__ solid, Dims d, unsigned* __restrict__ counts, int nblocks) {
    __shared__ unsigned cnt[19];
    if (threadIdx.x < 19) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int r = 0; r < LB_ROUNDS; ++r) {
        const long long cell = (long long)blockIdx.x * LB_CELLS + r * LB_THREADS + threadIdx.x;
        int i, j, k;
        const unsigned m = link_mask(solid, d, cell, i, j, k);
#pragma unroll
        for (int q = 1; q < 19; ++q) {
            const unsigned b = __ballot_sync(FULL, (m >> q) & 1u);
            if (lane == 0 && b) atomicAdd(&cnt[q], (unsigned)__popc(b));
        }
    }
    __syncthreads();
    if (threadIdx.x >= 1 && threadIdx.x < 19)
        counts[(long long)(threadIdx.x - 1) * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of the M per-(q, block) counts, in two levels: every block of
// 1024 threads scans a chunk of SCAN_CHUNK counts in place (local offsets), one
// block scans the chunk sums.  The offset of entry e is then
// counts[e] + chunk_off[e / SCAN_CHUNK].
constexpr int SCAN_THREADS = 1024, SCAN_PER_THREAD = 4, SCAN_CHUNK = SCAN_THREADS * SCAN_PER_THREAD;

template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* wsum, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(FULL, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    total = wsum[31];
    const T r = x - v + (warp ? wsum[warp - 1] : T(0));
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_chunks(unsigned* __restrict__ counts, long long M, long long* __restrict__ chunk_sum) {
    __shared__ unsigned wsum[32];
    const long long e0 = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_PER_THREAD;
    unsigned v[SCAN_PER_THREAD];
    unsigned s = 0;
#pragma unroll
    for (int t = 0; t < SCAN_PER_THREAD; ++t) {
        v[t] = e0 + t < M ? counts[e0 + t] : 0u;
        s += v[t];
    }
    unsigned total;
    unsigned run = block_exclusive_scan<unsigned>(s, wsum, total);
#pragma unroll
    for (int t = 0; t < SCAN_PER_THREAD; ++t) {
        if (e0 + t < M) counts[e0 + t] = run;
        run += v[t];
    }
    if (threadIdx.x == 0) chunk_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_totals(const long long* __restrict__ chunk_sum, long long nch, long long* __restrict__ chunk_off,
              long long* __restrict__ grand) {
    __shared__ long long wsum[32];
    long long carry = 0;
    for (long long b = 0; b < nch; b += SCAN_THREADS) {
        const long long e = b + threadIdx.x;
        const long long v = e < nch ? chunk_sum[e] : 0;
        long long total;
        const long long r = block_exclusive_scan<long long>(v, wsum, total);
        if (e < nch) chunk_off[e] = carry + r;
        carry += total;
    }
    if (threadIdx.x == 0 && grand) *grand = carry;
}

__global__ void __launch_bounds__(LB_THREADS)
k_links_write(const uint8_t* __restrict__ solid, Dims d, const unsigned* __restrict__ loc,
              const long long* __restrict__ chunk_off, int nblocks,
              long long n_links, long long* __restrict__ fluid_flat, long long* __restrict__ dir_i,
              long long* __restrict__ dir_opp, long long* __restrict__ ff_flat, uint8_t* __restrict__ ff_valid,
              unsigned* __restrict__ err) {
    constexpr int NW = LB_THREADS / 32;
    __shared__ long long base[19];
    __shared__ unsigned wc[19][NW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x >= 1 && threadIdx.x < 19) {
        const long long e = (long long)(threadIdx.x - 1) * nblocks + blockIdx.x;
        base[threadIdx.x] = (long long)loc[e] + chunk_off[e / SCAN_CHUNK];
    }
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < LB_ROUNDS; ++r) {
        const long long cell = (long long)blockIdx.x * LB_CELLS + r * LB_THREADS + threadIdx.x;
        int i, j, k;
        const unsigned m = link_mask(solid, d, cell, i, j, k);
        unsigned rank[19];
#pragma unroll
        for (int q = 1; q < 19; ++q) {
            const unsigned b = __ballot_sync(FULL, (m >> q) & 1u);
            rank[q] = __popc(b & lt);
            if (lane == 0) wc[q][warp] = __popc(b);
        }
        __syncthreads();
        if (m) {
#pragma unroll
            for (int q = 1; q < 19; ++q) {
                if (!((m >> q) & 1u)) continue;
                long long pos = base[q] + rank[q];
                for (int w = 0; w < warp; ++w) pos += wc[q][w];
                if (pos < 0 || pos >= n_links) {
                    atomicOr(err, DEV_ERR_INDEX);
                    continue;
                }
                const int a = i - cx(q), b = j - cy(q), e = k - cz(q);
                const bool inb = a >= 0 && a < d.nx && b >= 0 && b < d.ny && e >= 0 && e < d.nz;
                const long long ac = min(max(a, 0), d.nx - 1), bc = min(max(b, 0), d.ny - 1),
                                ec = min(max(e, 0), d.nz - 1);
                const long long ff = ac * d.nyz + bc * d.nz + ec;
                fluid_flat[pos] = cell;
                dir_i[pos] = q;
                dir_opp[pos] = opp(q);
                ff_flat[pos] = ff;
                ff_valid[pos] = (inb && !solid[ff]) ? 1 : 0;
            }
        }
        __syncthreads();
        if (threadIdx.x >= 1 && threadIdx.x < 19) {
            long long s = 0;
            for (int w = 0; w < NW; ++w) s += wc[threadIdx.x][w];
            base[threadIdx.x] += s;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Bouzidi fractions from the trilinear level set
// ---------------------------------------------------------------------------
struct QArgs {
    const float* phi;
    int nx, ny, nz;
    long long nyz;
    float ox, oy, oz;   // domain origin
    float pitch;        // FP32 pitch (the reference's float(pitch_mm) as an FP32 scalar)
    float hx, hy, hz;   // clamp bounds n - 1.001
    int true_div;       // 1: (x - origin) / dx rounded once; 0: times the FP32 reciprocal of dx
    const long long* fluid_flat;
    const long long* dir_i;
    long long n;
    float* q;
    uint8_t* ge;
    float* w1;
    float* w2;
    unsigned* err;
};

__device__ __forceinline__ float lerp_rn(float a, float b, float f) { return __fadd_rn(a, __fmul_rn(f, __fsub_rn(b, a))); }

// sdf_trilinear (sdf_tracing.py:89-125)
__device__ __forceinline__ float grid_coord(const QArgs& a, float inv_dx, float x, float o) {
    const float r = __fsub_rn(x, o);
    return a.true_div ? __fdiv_rn(r, a.pitch) : __fmul_rn(r, inv_dx);
}

__device__ float trilinear(const QArgs& a, float inv_dx, float x, float y, float z) {
    const float gx = fminf(fmaxf(grid_coord(a, inv_dx, x, a.ox), 0.0f), a.hx);
    const float gy = fminf(fmaxf(grid_coord(a, inv_dx, y, a.oy), 0.0f), a.hy);
    const float gz = fminf(fmaxf(grid_coord(a, inv_dx, z, a.oz), 0.0f), a.hz);
    int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    const float fx = __fsub_rn(gx, (float)i0), fy = __fsub_rn(gy, (float)j0), fz = __fsub_rn(gz, (float)k0);
    const int i1 = min(i0 + 1, a.nx - 1), j1 = min(j0 + 1, a.ny - 1), k1 = min(k0 + 1, a.nz - 1);
    // an axis of one cell clamps to n - 1.001 < 0, floor -1: torch indexing wraps -1 to the last cell
    if (i0 < 0) i0 += a.nx;
    if (j0 < 0) j0 += a.ny;
    if (k0 < 0) k0 += a.nz;
    const long long I0 = i0 * a.nyz, I1 = i1 * a.nyz;
    const long long J0 = (long long)j0 * a.nz, J1 = (long long)j1 * a.nz;
    const float* p = a.phi;
    const float c000 = __ldg(p + I0 + J0 + k0), c100 = __ldg(p + I1 + J0 + k0);
    const float c010 = __ldg(p + I0 + J1 + k0), c110 = __ldg(p + I1 + J1 + k0);
    const float c001 = __ldg(p + I0 + J0 + k1), c101 = __ldg(p + I1 + J0 + k1);
    const float c011 = __ldg(p + I0 + J1 + k1), c111 = __ldg(p + I1 + J1 + k1);
    const float x00 = lerp_rn(c000, c100, fx), x10 = lerp_rn(c010, c110, fx);
    const float x01 = lerp_rn(c001, c101, fx), x11 = lerp_rn(c011, c111, fx);
    const float y0 = lerp_rn(x00, x10, fy), y1 = lerp_rn(x01, x11, fy);
    return lerp_rn(y0, y1, fz);
}

// bfl_weights_from_q (sdf_tracing.py:188-205): q >= 1/2: w1 = 1/(2q), w2 = 1 - w1;
// else w1 = 2q, w2 = 1 - 2q
__device__ __forceinline__ void bfl_weights(float qv, uint8_t* ge, float* w1, float* w2) {
    const bool g = qv >= 0.5f;
    if (g) {
        const float a = __fdiv_rn(1.0f, __fmul_rn(2.0f, qv));
        *w1 = a;
        *w2 = __fsub_rn(1.0f, a);
    } else {
        *w1 = __fmul_rn(2.0f, qv);
        *w2 = __fsub_rn(1.0f, __fmul_rn(2.0f, qv));
    }
    *ge = g ? 1 : 0;
}

// bfl_q_from_sdf (sdf_tracing.py:128-184) with 6 coarse segments and 10
// bisections, then the weights
__global__ void __launch_bounds__(256) k_ibb_q(QArgs a) {
    const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= a.n) return;
    const long long cell = a.fluid_flat[l];
    const int q = (int)a.dir_i[l];
    if (cell < 0 || cell >= (long long)a.nx * a.nyz || q < 1 || q > 18) {
        atomicOr(a.err, DEV_ERR_INDEX);
        return;
    }
    const int i = (int)(cell / a.nyz);
    const int rem = (int)(cell - (long long)i * a.nyz);
    const int j = rem / a.nz, k = rem - j * a.nz;
    const float inv_dx = __fdiv_rn(1.0f, a.pitch);
    const float x0 = __fadd_rn(__fmul_rn((float)i, a.pitch), a.ox);
    const float y0 = __fadd_rn(__fmul_rn((float)j, a.pitch), a.oy);
    const float z0 = __fadd_rn(__fmul_rn((float)k, a.pitch), a.oz);
    // unit direction: c / (|c| + 1e-30) with |c| = 1 or sqrt(2)
    const int n_ax = (cx(q) != 0) + (cy(q) != 0) + (cz(q) != 0);
    const float cn = n_ax == 1 ? 1.0f : __fsqrt_rn(2.0f);
    const float den = __fadd_rn(cn, 1e-30f);
    const float dxv = __fdiv_rn((float)cx(q), den), dyv = __fdiv_rn((float)cy(q), den),
                dzv = __fdiv_rn((float)cz(q), den);
    const float L = __fmul_rn(a.pitch, cn);
    // torch.linspace(0, 1, 7): start + step*i below the midpoint, end - step*(6-i) from it
    const float step = __fdiv_rn(1.0f, 6.0f);
    float tv[7];
    tv[0] = 0.0f;
    tv[1] = step;
    tv[2] = __fmul_rn(step, 2.0f);
    tv[3] = __fsub_rn(1.0f, __fmul_rn(step, 3.0f));
    tv[4] = __fsub_rn(1.0f, __fmul_rn(step, 2.0f));
    tv[5] = __fsub_rn(1.0f, step);
    tv[6] = 1.0f;
    float t[7];
    bool pos[7];
#pragma unroll
    for (int s = 0; s < 7; ++s) {
        t[s] = __fmul_rn(tv[s], L);
        const float ph = trilinear(a, inv_dx, __fadd_rn(x0, __fmul_rn(t[s], dxv)), __fadd_rn(y0, __fmul_rn(t[s], dyv)),
                                   __fadd_rn(z0, __fmul_rn(t[s], dzv)));
        pos[s] = ph > 0.0f;
    }
    int idx = -1;
#pragma unroll
    for (int s = 5; s >= 0; --s)
        if (pos[s] && !pos[s + 1]) idx = s;
    float qv = 0.5f;
    if (idx >= 0) {
        float lo = t[idx], hi = t[idx + 1];
        for (int it = 0; it < 10; ++it) {
            const float mid = __fmul_rn(0.5f, __fadd_rn(lo, hi));
            const float pm = trilinear(a, inv_dx, __fadd_rn(x0, __fmul_rn(mid, dxv)), __fadd_rn(y0, __fmul_rn(mid, dyv)),
                                       __fadd_rn(z0, __fmul_rn(mid, dzv)));
            if (pm > 0.0f) lo = mid;
            else hi = mid;
        }
        qv = __fdiv_rn(hi, __fadd_rn(L, 1e-30f));
    }
    if (a.q) a.q[l] = qv;
    bfl_weights(qv, a.ge + l, a.w1 + l, a.w2 + l);
}

__global__ void __launch_bounds__(256)
k_ibb_weights(const float* __restrict__ q, long long n, uint8_t* ge, float* w1, float* w2) {
    const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l < n) bfl_weights(q[l], ge + l, w1 + l, w2 + l);
}

bool dims_ok(int nx, int ny, int nz) {
    return nx >= 1 && ny >= 1 && nz >= 1 && (long long)nx * ny * nz < (1LL << 40);
}

long long link_blocks(int nx, int ny, int nz) {
    return ((long long)nx * ny * nz + LB_CELLS - 1) / LB_CELLS;
}

long long align8(long long x) { return (x + 7) & ~7LL; }

}  // namespace

extern "C" {

long long fc_geom_edt_workspace_bytes(int nx, int ny, int nz) {
    if (!dims_ok(nx, ny, nz)) return -1;
    return (long long)nx * ny * nz * (long long)sizeof(int) + (long long)SQRT_TAB * (long long)sizeof(float);
}

int fc_geom_signed_edt(const uint8_t* solid, int nx, int ny, int nz, double pitch, float* phi, void* workspace,
                       long long workspace_bytes, void* stream) {
    if (!solid || !phi || !workspace || !dims_ok(nx, ny, nz)) return FC_ERR_ARG;
    if (workspace_bytes < fc_geom_edt_workspace_bytes(nx, ny, nz)) return FC_ERR_ARG;
    if (nz > EDT_MAX_NZ || ny > EDT_MAX_LINE || nx > EDT_MAX_LINE || ny > 65535 || nx > 65535)
        return FC_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    int* g = (int*)workspace;
    const long long nrows = (long long)nx * ny;
    const int nch = (nz + 31) / 32;
    const size_t rsmem = (size_t)ROW_WARPS * 4 * nch * sizeof(unsigned);
    const long long rblocks = (nrows + ROW_WARPS - 1) / ROW_WARPS;
    k_edt_rows<<<(unsigned)(rblocks < (1LL << 20) ? rblocks : (1LL << 20)), ROW_WARPS * 32, rsmem, st>>>(
        solid, g, nrows, nz, nch);
    int rc = launch_status();
    if (rc) return rc;
    float* tab = (float*)(g + (long long)nx * ny * nz);
    k_edt_sqrt_table<<<SQRT_TAB / 256, 256, 0, st>>>(tab, pitch);
    rc = launch_status();
    if (rc) return rc;
    // y pass: lines along j (stride nz), one block row per i
    rc = launch_lines<false>(solid, g, nullptr, nullptr, ny, nz, (long long)ny * nz, nx, nz, pitch, st);
    if (rc) return rc;
    // x pass: lines along i (stride ny*nz), one block row per j; writes phi
    return launch_lines<true>(solid, g, phi, tab, nx, (long long)ny * nz, nz, ny, nz, pitch, st);
}

long long fc_ibb_links_workspace_bytes(int nx, int ny, int nz) {
    if (!dims_ok(nx, ny, nz)) return -1;
    const long long M = 18 * link_blocks(nx, ny, nz);
    const long long nch = (M + SCAN_CHUNK - 1) / SCAN_CHUNK;
    return align8(M * 4) + 2 * nch * 8;
}

int fc_ibb_count_links(const uint8_t* solid, int nx, int ny, int nz, void* workspace, long long workspace_bytes,
                       long long* n_links, void* stream) {
    if (!solid || !workspace || !n_links || !dims_ok(nx, ny, nz)) return FC_ERR_ARG;
    if (workspace_bytes < fc_ibb_links_workspace_bytes(nx, ny, nz)) return FC_ERR_ARG;
    const long long nb = link_blocks(nx, ny, nz);
    if (nb > 0x7fffffffLL) return FC_ERR_UNSUPPORTED;
    const long long M = 18 * nb;
    const long long nch = (M + SCAN_CHUNK - 1) / SCAN_CHUNK;
    unsigned* counts = (unsigned*)workspace;
    long long* chunk_sum = (long long*)((char*)workspace + align8(M * 4));
    long long* chunk_off = chunk_sum + nch;
    Dims d{nx, ny, nz, (long long)ny * nz, (long long)nx * ny * nz};
    cudaStream_t st = (cudaStream_t)stream;
    k_links_count<<<(unsigned)nb, LB_THREADS, 0, st>>>(solid, d, counts, (int)nb);
    int rc = launch_status();
    if (rc) return rc;
    k_scan_chunks<<<(unsigned)nch, SCAN_THREADS, 0, st>>>(counts, M, chunk_sum);
    rc = launch_status();
    if (rc) return rc;
    k_scan_totals<<<1, SCAN_THREADS, 0, st>>>(chunk_sum, nch, chunk_off, n_links);
    return launch_status();
}

int fc_ibb_build_links(const uint8_t* solid, int nx, int ny, int nz, const void* workspace, long long workspace_bytes,
                       long long n_links, long long* fluid_flat, long long* dir_i, long long* dir_opp,
                       long long* ff_flat, uint8_t* ff_valid, unsigned* err, void* stream) {
    if (!solid || !workspace || !err || !dims_ok(nx, ny, nz) || n_links < 0) return FC_ERR_ARG;
    if (workspace_bytes < fc_ibb_links_workspace_bytes(nx, ny, nz)) return FC_ERR_ARG;
    if (n_links == 0) return FC_OK;
    if (!fluid_flat || !dir_i || !dir_opp || !ff_flat || !ff_valid) return FC_ERR_ARG;
    const long long nb = link_blocks(nx, ny, nz);
    if (nb > 0x7fffffffLL) return FC_ERR_UNSUPPORTED;
    const long long M = 18 * nb;
    const long long nch = (M + SCAN_CHUNK - 1) / SCAN_CHUNK;
    const unsigned* loc = (const unsigned*)workspace;
    const long long* chunk_off = (const long long*)((const char*)workspace + align8(M * 4)) + nch;
    Dims d{nx, ny, nz, (long long)ny * nz, (long long)nx * ny * nz};
    k_links_write<<<(unsigned)nb, LB_THREADS, 0, (cudaStream_t)stream>>>(solid, d, loc, chunk_off, (int)nb, n_links,
                                                                          fluid_flat, dir_i, dir_opp, ff_flat,
                                                                          ff_valid, err);
    return launch_status();
}

int fc_ibb_q_from_sdf(const float* phi, int nx, int ny, int nz, float origin_x, float origin_y, float origin_z,
                      double dx, int true_div, const long long* fluid_flat, const long long* dir_i, long long n_links,
                      float* q, uint8_t* q_ge_half, float* w_i, float* w_second, unsigned* err, void* stream) {
    if (!phi || !err || !dims_ok(nx, ny, nz) || n_links < 0 || !(dx > 0.0) || (true_div != 0 && true_div != 1))
        return FC_ERR_ARG;
    if (n_links == 0) return FC_OK;
    if (!fluid_flat || !dir_i || !q_ge_half || !w_i || !w_second) return FC_ERR_ARG;
    QArgs a;
    a.phi = phi;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.nyz = (long long)ny * nz;
    a.ox = origin_x;
    a.oy = origin_y;
    a.oz = origin_z;
    a.pitch = (float)dx;
    a.hx = (float)((double)nx - 1.001);
    a.hy = (float)((double)ny - 1.001);
    a.hz = (float)((double)nz - 1.001);
    a.true_div = true_div;
    a.fluid_flat = fluid_flat;
    a.dir_i = dir_i;
    a.n = n_links;
    a.q = q;
    a.ge = q_ge_half;
    a.w1 = w_i;
    a.w2 = w_second;
    a.err = err;
    k_ibb_q<<<(unsigned)((n_links + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a);
    return launch_status();
}

int fc_ibb_weights_from_q(const float* q, long long n_links, uint8_t* q_ge_half, float* w_i, float* w_second,
                          void* stream) {
    if (n_links < 0) return FC_ERR_ARG;
    if (n_links == 0) return FC_OK;
    if (!q || !q_ge_half || !w_i || !w_second) return FC_ERR_ARG;
    k_ibb_weights<<<(unsigned)((n_links + 255) / 256), 256, 0, (cudaStream_t)stream>>>(q, n_links, q_ge_half, w_i,
                                                                                       w_second);
    return launch_status();
}

}  // extern "C"
