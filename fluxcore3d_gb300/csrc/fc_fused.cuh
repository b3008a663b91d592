// fc_fused.cuh -- device code shared by the fused D3Q19 passes (direct-load
// pass in fc_lbm.cu, TMA-staged pass in fc_lbm_tma.cu).
#pragma once
#include "fc_common.cuh"
#include "fc_collide.cuh"

namespace fc {

struct Geo {
    int nx, ny, nz;
    int px, py, pz;
    long long N;   // population stride (cells); cell indices themselves fit in 32 bits
    int nynz;
};

// Threads map to cells as (k, j, i) = (x, y, z) launch coordinates: a warp
// covers 32 consecutive k of one row, so every population access of a warp is
// one contiguous (possibly one-element shifted) run, and i, j are warp-uniform.
constexpr int TBX = 32, TBY = 4;

__device__ __forceinline__ bool cell_of_thread(const Geo& g, int& i, int& j, int& k, int& idx) {
    k = blockIdx.x * TBX + threadIdx.x;
    j = blockIdx.y * TBY + threadIdx.y;
    i = blockIdx.z;
    if (k >= g.nz || j >= g.ny) return false;
    idx = (i * g.ny + j) * g.nz + k;
    return true;
}

// Source cell x - c_q of every population: periodic axes wrap, a non-periodic
// axis that leaves the box makes the cell its own source (stream_pull rule).
__device__ __forceinline__ void pull_sources(const Geo& g, int i, int j, int k, int idx, int src[19]) {
    const bool inner = (i > 0) & (i < g.nx - 1) & (j > 0) & (j < g.ny - 1);  // warp-uniform
    if (inner) {
        const bool zm_ok = (k > 0) | (g.pz != 0);
        const bool zp_ok = (k < g.nz - 1) | (g.pz != 0);
        const int dzm = k > 0 ? -1 : g.nz - 1;          // source k-1 (c_z = +1)
        const int dzp = k < g.nz - 1 ? 1 : -(g.nz - 1); // source k+1 (c_z = -1)
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int base = idx - cx(q) * g.nynz - cy(q) * g.nz;
            if (cz(q) == 0) src[q] = base;
            else if (cz(q) == 1) src[q] = zm_ok ? base + dzm : idx;
            else src[q] = zp_ok ? base + dzp : idx;
        }
        return;
    }
    const int im = i > 0 ? i - 1 : (g.px ? g.nx - 1 : -1);
    const int ip = i < g.nx - 1 ? i + 1 : (g.px ? 0 : -1);
    const int jm = j > 0 ? j - 1 : (g.py ? g.ny - 1 : -1);
    const int jp = j < g.ny - 1 ? j + 1 : (g.py ? 0 : -1);
    const int km = k > 0 ? k - 1 : (g.pz ? g.nz - 1 : -1);
    const int kp = k < g.nz - 1 ? k + 1 : (g.pz ? 0 : -1);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const int si = cx(q) == 1 ? im : (cx(q) == -1 ? ip : i);
        const int sj = cy(q) == 1 ? jm : (cy(q) == -1 ? jp : j);
        const int sk = cz(q) == 1 ? km : (cz(q) == -1 ? kp : k);
        src[q] = ((si | sj | sk) < 0) ? idx : (si * g.ny + sj) * g.nz + sk;
    }
}

struct FusedArgs {
    Geo g;
    const void* pin[19];   // population planes of the previous post-collision buffer
    void* pout[19];        // population planes of this step's buffer
    float* f32;
    float* rho;
    float* u;
    float* v;
    float* w;
    const uint8_t* flags;
    const int* link_off;      // per cell: link-cell ordinal (read where the link flag is set)
    const uint4* link_hdr;    // per link cell: (dir mask, second-node mask, weight offset, 0)
    const float2* link_w;
    long long n_links;
    const int* link_cells;    // optional list for the separate link pass
    long long n_link_cells;
    void* link_val;           // per link: this step's interpolated bounce-back value in storage form, or null
    long long n_link_val;     // capacity of link_val in elements
    const int4* tile_links;   // per tile of the staged pass: 2 x int4 record (ranges, chunk link offsets)
    long long n_tile_links;
    const uint16_t* link_pos; // per link: element of the staged tile its value replaces (0xffff: none)
    long long n_link_pos;
    const uint2* link_src;    // per link: population elements it blends (bit 31 of .x: edge direction)
    long long n_link_src;
    const float* sponge;
    int sponge_axis;
    int has_links;
    CollideParams cp;
    unsigned* dev_err;
    // passive tracer carried by the staged main pass (tr_in null: none)
    const float* tr_in;
    float* tr_out;
    const float* tr_u;
    const float* tr_v;
    const float* tr_w;
    const uint8_t* tr_solid;
    float tr_diss;
    int tile_order;     // staged pass: 0 tiles in ascending order, 1 descending
    int gather_order;   // link gather: 0 links in ascending order, 1 descending
};

// shifted value h = f - w_q of population q at `cell` of the input buffer
template <int KIND>
__device__ __forceinline__ float in_h(const FusedArgs& a, int q, int cell) {
    using T = typename Store<KIND>::T;
    const T* p = reinterpret_cast<const T*>(a.pin[q]) + cell;
    if (KIND == ST_F32) return __ldg(reinterpret_cast<const float*>(p)) - wq(q);
    if (KIND == ST_F16S) return __half2float(__ldg(reinterpret_cast<const __half*>(p)));
    return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p)));
}
template <int KIND>
__device__ __forceinline__ void out_h(const FusedArgs& a, int q, int cell, float h) {
    using T = typename Store<KIND>::T;
    T* p = reinterpret_cast<T*>(a.pout[q]) + cell;
    if (KIND == ST_F32) *reinterpret_cast<float*>(p) = h + wq(q);
    else if (KIND == ST_F16S) *reinterpret_cast<__half*>(p) = __float2half_rn(h);
    else *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(h);
}
// Unshifted value f_q of population q at `cell` of the input buffer.
template <int KIND>
__device__ __forceinline__ float in_f(const FusedArgs& a, int q, int cell) {
    using T = typename Store<KIND>::T;
    const T* p = reinterpret_cast<const T*>(a.pin[q]) + cell;
    if (KIND == ST_F32) return __ldg(reinterpret_cast<const float*>(p));
    if (KIND == ST_F16S) return __fadd_rn(__half2float(__ldg(reinterpret_cast<const __half*>(p))), wq(q));
    return __fadd_rn(__bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p))), wq(q));
}

// Interpolated bounce-back of one link cell (reference lbm_kernels.cu:542-588),
// evaluated from the previous post-collision buffer.  The cell's header (uint4)
// holds: x = mask of link directions (bit d), y = mask of links whose second
// term is the opposite population at x_f - c_d (q < 1/2 with a fluid second
// node) instead of population d at x_f, z = offset of the cell's (w1, w2)
// pairs, one per set bit of x in ascending d.  q < 1/2 links without a second
// node are stored as (w1, w2) = (1, 0).  The shifted post-stream value is
// w1 f_opp(d)(x_f) + w2 f_2 - w_d, rounded explicitly so that every kernel that
// evaluates it gets the same bits.  Directions are unrolled so every population
// index is a compile-time constant.
template <int KIND, int D>
__device__ __forceinline__ float link_value(const FusedArgs& a, int idx, uint4 hd) {
    constexpr int O = opp(D);
    const float2 wt = __ldg(a.link_w + hd.z + __popc(hd.x & ((1u << D) - 1u)));
    const float fo = in_f<KIND>(a, O, idx);
    const bool second_ff = (hd.y >> D) & 1u;
    const float f2 = second_ff ? in_f<KIND>(a, O, idx - (cx(D) * a.g.nynz + cy(D) * a.g.nz + cz(D)))
                               : in_f<KIND>(a, D, idx);
    return __fsub_rn(__fmaf_rn(wt.x, fo, __fmul_rn(wt.y, f2)), wq(D));
}

// h[d] <- link value, computed from the input buffer
template <int KIND, int D>
struct LinkDir {
    static __device__ __forceinline__ void run(const FusedArgs& a, int idx, uint4 hd, float h[19]) {
        if (hd.x & (1u << D)) h[D] = link_value<KIND, D>(a, idx, hd);
        LinkDir<KIND, D + 1>::run(a, idx, hd, h);
    }
};
template <int KIND>
struct LinkDir<KIND, 19> {
    static __device__ __forceinline__ void run(const FusedArgs&, int, uint4, float*) {}
};

// Storage form of a shifted value h of population q (what a population buffer
// holds) and back: FP32 keeps f = h + w_q, FP16/BF16 keep h rounded.
template <int KIND>
__device__ __forceinline__ typename Store<KIND>::T encode_h(float h, int q) {
    if constexpr (KIND == ST_F32) return __fadd_rn(h, wq(q));
    else if constexpr (KIND == ST_F16S) return __float2half_rn(h);
    else return __float2bfloat16_rn(h);
}
template <int KIND>
__device__ __forceinline__ float decode_h(typename Store<KIND>::T v, int q) {
    if constexpr (KIND == ST_F32) return __fsub_rn(v, wq(q));
    else if constexpr (KIND == ST_F16S) return __half2float(v);
    else return __bfloat162float(v);
}

// link_val[hd.z + rank(d)] <- link value in storage form (the per-step gather of k_link_gather)
template <int KIND, int D>
struct LinkGather {
    static __device__ __forceinline__ void run(const FusedArgs& a, int idx, uint4 hd) {
        using T = typename Store<KIND>::T;
        if (hd.x & (1u << D))
            reinterpret_cast<T*>(a.link_val)[hd.z + __popc(hd.x & ((1u << D) - 1u))] =
                encode_h<KIND>(link_value<KIND, D>(a, idx, hd), D);
        LinkGather<KIND, D + 1>::run(a, idx, hd);
    }
};
template <int KIND>
struct LinkGather<KIND, 19> {
    static __device__ __forceinline__ void run(const FusedArgs&, int, uint4) {}
};

// h[d] <- gathered link value (vals = the cell's values in storage form, one per set bit of mask)
template <int KIND, int D>
struct LinkTake {
    static __device__ __forceinline__ void run(unsigned mask, const typename Store<KIND>::T* vals, float h[19]) {
        if (mask & (1u << D)) h[D] = decode_h<KIND>(vals[__popc(mask & ((1u << D) - 1u))], D);
        LinkTake<KIND, D + 1>::run(mask, vals, h);
    }
};
template <int KIND>
struct LinkTake<KIND, 19> {
    static __device__ __forceinline__ void run(unsigned, const typename Store<KIND>::T*, float*) {}
};

// Interpolated bounce-back on the links of link cell `idx` whose link-cell
// ordinal `lc` was read from link_off (bad ordinals flag DEV_ERR_INDEX and leave
// the pulled values).  Uses this step's gathered values when link_val is set.
template <int KIND>
__device__ __forceinline__ void apply_links(const FusedArgs& a, int idx, int lc, float h[19]) {
    if (lc < 0 || (long long)lc >= a.n_link_cells) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    const uint4 hd = __ldg(a.link_hdr + lc);
    if ((long long)hd.z + __popc(hd.x) > a.n_links) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    if (a.link_val)
        LinkTake<KIND, 1>::run(hd.x, reinterpret_cast<const typename Store<KIND>::T*>(a.link_val) + hd.z, h);
    else LinkDir<KIND, 1>::run(a, idx, hd, h);
}

template <int KIND>
__device__ __forceinline__ void gather_cell(const FusedArgs& a, int idx, int i, int j, int k, uint8_t fl,
                                            float h[19]) {
    int lc = -1;
    if (fl & CF_LINK) lc = __ldg(a.link_off + idx);
    int src[19];
    pull_sources(a.g, i, j, k, idx, src);
#pragma unroll
    for (int q = 0; q < 19; ++q) h[q] = in_h<KIND>(a, q, src[q]);
    if (fl & CF_LINK) apply_links<KIND>(a, idx, lc, h);
}

// Post-stream populations (shifted) of a flow-solid cell as the reference leaves
// them: w_q after reset_solid when links exist, else the in-cell direction swap
// of the pulled values (LBM_CHT.py _bounce_back_post_stream).
template <int KIND>
__device__ __forceinline__ void solid_cell(const FusedArgs& a, int idx, int i, int j, int k, float h[19]) {
    if (a.has_links) {
#pragma unroll
        for (int q = 0; q < 19; ++q) h[q] = 0.f;
    } else {
        int src[19];
        pull_sources(a.g, i, j, k, idx, src);
        float t[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) t[q] = in_h<KIND>(a, q, src[q]);
#pragma unroll
        for (int q = 0; q < 19; ++q) h[q] = t[opp(q)];
    }
}

__device__ __forceinline__ void export_f(const FusedArgs& a, int idx, const float h[19]) {
#pragma unroll
    for (int q = 0; q < 19; ++q) a.f32[q * a.g.N + idx] = h[q] + wq(q);
}

template <int KIND, int MODE>
__device__ __forceinline__ void collide_store(const FusedArgs& a, int idx, int i, int j, int k, float hf[19]) {
    f1 h[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) h[q].v = hf[q];
    const MacroV<f1> m = collide_h<MODE>(h, a.cp);
    if (a.sponge) {
        const int c = a.sponge_axis == 0 ? i : (a.sponge_axis == 1 ? j : k);
        const float sg = __ldg(a.sponge + c);
        if (sg > 0.f) {
            f1 heq[19];
            equilibrium_h(m, heq);
#pragma unroll
            for (int q = 0; q < 19; ++q) h[q] = fma(-sg, h[q] - heq[q], h[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) out_h<KIND>(a, q, idx, h[q].v);
    if (a.rho) {
        a.rho[idx] = m.rho.v; a.u[idx] = m.ux.v; a.v[idx] = m.uy.v; a.w[idx] = m.uz.v;
    }
}

// TMA-staged persistent pass (fc_lbm_tma.cu).  Returns FC_ERR_UNSUPPORTED when
// the grid does not meet its tiling rules; the caller then uses the direct pass.
int launch_fused_tma(const FusedArgs& a, int storage, int collision, cudaStream_t st);
bool fused_tma_eligible(const FusedArgs& a, int storage);
// Tile count of the staged pass (0 if it does not apply); with out != null also
// fills the per-tile records (cap at most) and, with pos != null, the per-link
// staged-tile elements.  Negative on error.
long long tma_tile_links(const FusedArgs& a, int4* out, long long cap, uint16_t* pos, long long pos_cap,
                         uint2* src, long long src_cap, cudaStream_t st);

}  // namespace fc
