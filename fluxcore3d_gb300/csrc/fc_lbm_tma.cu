// fc_lbm_tma.cu -- TMA-staged persistent main pass of the fused D3Q19 step (sm_103a).
//
// The direct pass (k_fused_step) keeps its memory parallelism in registers: a
// thread holds 19 pulled populations while their loads are in flight, which
// caps residency at 28 warps per SM and leaves HBM under-subscribed.  This pass
// moves the pulls off the register file.
//
// Tiles.  The grid is cut into tiles of `tj` whole rows (fixed i, rows
// j0..j0+tj-1, every k; at most 512 cells and 8 chunks of 64 cells).  For each
// tile one thread issues 19 tensor copies (cp.async.bulk.tensor): population
// q's box starts at plane i - c_x(q), row j0 - c_y(q), so the box already holds
// exactly what the tile pulls along x and y and the k shift becomes an index
// offset inside a whole row.  A row longer than a box may be (256 elements) is
// seen through the tensor map as `nseg` segments of nz / nseg elements (a 5-D
// view: segment element, segment, row, plane, population), so one copy still
// brings whole rows.  One more tensor copy brings the tile's flag
// bytes, and two plain bulk copies bring the tile's slice of this step's
// gathered interpolated bounce-back values (storage form) and of the static
// table saying which staged element each of them replaces.  Link cells and
// links are stored in cell order, so a tile's links are one contiguous range;
// fc_lbm_tile_links precomputes it with the first link of every chunk.
// Persistent CTAs of 4 warps (4 per SM at 16-bit storage, 2 at FP32) take the
// tiles in ascending or, with tile_order, descending order (the step alternates,
// so each pass starts on the planes the previous one wrote last, still in L2) and
// rotate over 2 shared-memory stages
// tracked by mbarriers; warps run through the tiles independently and the last
// warp done with a stage refills it, so no CTA-wide barrier sits in the loop.
//
// Cells.  Before a warp reads its chunk it writes the chunk's link values into
// the slab elements its link cells pull (each element is pulled by exactly one
// cell and direction), so collision code never looks at links.  A lane then
// collides two neighbouring cells (k, k+1) with packed FP32 arithmetic (f2);
// every operation is explicitly rounded, so the results are bit-identical to
// the direct pass, which decodes the same stored link values.  Cells whose
// pulls leave the grid (i or j on the boundary, k on a non-periodic boundary),
// plane cells that export their post-stream state, and link cells of a tile
// whose link slice exceeds the stage's room take a path with direct global
// loads.
//
// Tracer.  When the arguments carry a passive tracer, every lane also advances
// it for its two cells (tracer_pair, all cells, solid ones included), so a step
// with a tracer needs no tracer launch of its own.
//
// Every mbarrier wait is bounded.  A CTA whose wait gives up sets
// DEV_ERR_TIMEOUT, waits (again bounded) for the copies it still has in flight
// and returns, so a lost copy never hangs the device.
#include "fc_fused.cuh"
#include "fc_tma.cuh"
#include "../../include/fluxcore3d_gb300.h"

#include <mutex>

namespace fc {
namespace {

constexpr int TS_THREADS = 128;
// CTAs of 4 warps per SM the register budget is set for: 4 at 16-bit storage
// (<= 128 registers a thread; 4 x 52.6 KB of stages fit the SM's shared memory),
// 3 at FP32 (whose 95 KB of stages allow 2 CTAs per SM anyway)
template <int KIND>
constexpr int ts_min_blocks() { return KIND == ST_F32 ? 3 : 4; }
constexpr int TS_WARPS = TS_THREADS / 32;
constexpr int TS_RANGE_CACHE = 64;         // per-CTA cache of the records of its first tiles
constexpr int TS_HEAD_BYTES = 128 + TS_RANGE_CACHE * 32;   // mbarriers, stage counters, record cache
constexpr unsigned TS_SPIN = 1u << 24;     // bound on mbarrier polls (seconds of waiting at most)
constexpr int TS_TILE_CELLS = 512;         // most cells of a tile (tj = 512 / nz rows)
constexpr int TS_PRE = 8;                  // at most 8 chunks (64 cells of a row) per tile
// room per stage for the tile's link values (the densest 512-cell tile of the
// pin-fin heat sink has 1217 links)
constexpr int TS_LK_CAP = 1280;

// Shared-memory layout of one stage, fixed per storage so that every slab
// offset is an immediate: 19 population slabs of TS_TILE_CELLS elements, the
// flag bytes, the tile record, and the tile's link slots and link values.
template <int KIND>
struct Layout {
    static constexpr uint32_t SB = KIND == ST_F32 ? 4u : 2u;
    static constexpr uint32_t Q = TS_TILE_CELLS * SB;
    static constexpr uint32_t FLAG = 19u * Q;
    static constexpr uint32_t INFO = FLAG + TS_TILE_CELLS;
    static constexpr uint32_t POS = INFO + 128u;
    static constexpr uint32_t VAL = POS + TS_LK_CAP * 2u;
    static constexpr uint32_t STAGE = VAL + TS_LK_CAP * SB;
    // 2 stages (a third one, which fits 3 CTAs at 16-bit storage, measured no faster)
    static constexpr int STAGES = 2;
    static_assert(STAGE % 128 == 0, "stage size keeps every stage 128-byte aligned");
};

struct TileGeo {
    int tj;              // rows per tile
    int tiles_j;         // tiles per plane
    int n_tiles;
    int kchunks;         // 64-cell chunks per row (a lane collides cells k, k+1)
    int kc_inv;          // ceil(65536 / kchunks): chunk -> row by multiply and shift
    uint32_t base_tx;    // bytes of the population and flag boxes of one tile
    int wrap_y;          // 1: the periodic y wrap of the first and last tile of a plane is staged
};

// Tensor maps of the population buffer: boxes of tj rows, of tj - 1 rows and of
// one row (the last two stage the periodic y wrap of a plane's edge tiles).
struct PopMaps {
    CUtensorMap full, shrt, row;
};

// Per-tile record (global, from fc_lbm_tile_links): link-cell range, link
// range, and the offset from the tile's first link of each chunk's first link.
struct TileRec {
    int lcb, lce, lb, le;
    unsigned short pre[TS_PRE];
};

// Per-stage record written by the issuing thread before it arms the stage.
struct TileInfo {
    int lb;      // first link of the tile
    int lb0;     // link held by staged slot 0 (lb rounded down to 8)
    int nl;      // links of the tile
    int staged;  // 1: link slots and values staged, 0: the tile has no links, -1: not staged
    unsigned short pre[TS_PRE];
    int wrap;    // 1: the rows this tile pulls across the periodic y boundary are staged
};

// Link slice of a tile as staged (16-byte aligned ends), or staged = -1 when
// it is absent, invalid or too large.
__device__ __forceinline__ TileInfo tile_info(const FusedArgs& a, const TileRec& r, int& n_st) {
    TileInfo ti;
    ti.lb = ti.lb0 = ti.nl = ti.staged = 0;
    n_st = 0;
#pragma unroll
    for (int c = 0; c < TS_PRE; ++c) ti.pre[c] = r.pre[c];
    if (a.n_links <= 0) return ti;
    if (!a.link_val || !a.tile_links || !a.link_pos) {
        ti.staged = -1;
        return ti;
    }
    const bool valid = r.lb >= 0 && r.lb <= r.le && (long long)r.le <= a.n_links;
    if (!valid) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        ti.staged = -1;
        return ti;
    }
    ti.lb = r.lb;
    ti.nl = r.le - r.lb;
    if (ti.nl == 0) return ti;
    ti.lb0 = r.lb & ~7;
    n_st = ((r.le - ti.lb0) + 7) & ~7;
    ti.staged = n_st <= TS_LK_CAP ? 1 : -1;
    if (ti.staged < 0) n_st = 0;
    return ti;
}

// One tile into one stage: 19 population boxes (segment-element and segment
// coordinates 0, so every copy starts on a 16-byte boundary), the tile's flag
// bytes, and its link slots and values.  A periodic x axis wraps the box's
// plane coordinate.  With tg.wrap_y, the boxes of the first and last tile of a
// plane that would reach row -1 or row ny are split into a box of tj - 1 rows
// and a one-row box of the wrapped row, landing in disjoint slab rows; other
// rows or planes outside the grid read as zero and are never used (those cells
// take the direct-load path).
// The staged link range ends at most 7 entries past the tile's last link;
// link_pos and link_val hold n_links + 8 entries, so the copies stay inside.
template <int KIND>
__device__ __forceinline__ void issue_tile(const FusedArgs& a, const PopMaps* tp, const CUtensorMap* tf,
                                           const TileGeo& tg, int tile, const TileRec& rec, unsigned char* stage,
                                           uint32_t bar) {
    using LY = Layout<KIND>;
    const int i = tile / tg.tiles_j;
    const int j0 = (tile - i * tg.tiles_j) * tg.tj;
    int n_st;
    TileInfo ti = tile_info(a, rec, n_st);
    const int ny = a.g.ny, nx = a.g.nx;
    const bool first = tg.wrap_y && j0 == 0, last = tg.wrap_y && j0 + tg.tj == ny;
    ti.wrap = first | last;
    *reinterpret_cast<TileInfo*>(stage + LY::INFO) = ti;
    const uint32_t tx = tg.base_tx + (uint32_t)n_st * (2u + LY::SB);
    bar_expect_tx(bar, tx);   // release: the info record is visible to whoever sees the phase complete
    const uint32_t st = su32(stage);
    const uint32_t row_bytes = (uint32_t)a.g.nz * LY::SB;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        int ii = i - cx(q);
        if (a.g.px) ii = ii < 0 ? nx - 1 : (ii >= nx ? 0 : ii);
        const uint32_t dst = st + q * LY::Q;
        if (cy(q) == 1 && first) {            // slab row 0 <- row ny - 1, rows 1.. <- rows 0..tj-2
            if (tg.tj > 1) tma_load_5d(dst + row_bytes, &tp->shrt, 0, 0, 0, ii, q, bar);
            tma_load_5d(dst, &tp->row, 0, 0, ny - 1, ii, q, bar);
        } else if (cy(q) == -1 && last) {     // rows 0..tj-2 <- rows j0+1.., slab row tj-1 <- row 0
            if (tg.tj > 1) tma_load_5d(dst, &tp->shrt, 0, 0, j0 + 1, ii, q, bar);
            tma_load_5d(dst + (uint32_t)(tg.tj - 1) * row_bytes, &tp->row, 0, 0, 0, ii, q, bar);
        } else {
            tma_load_5d(dst, &tp->full, 0, 0, j0 - cy(q), ii, q, bar);
        }
    }
    tma_load_4d(st + LY::FLAG, tf, 0, 0, j0, i, bar);
    if (n_st > 0) {
        bulk_load(st + LY::POS, a.link_pos + ti.lb0, (uint32_t)n_st * 2u, bar);
        bulk_load(st + LY::VAL, reinterpret_cast<const unsigned char*>(a.link_val) + (size_t)ti.lb0 * LY::SB,
                  (uint32_t)n_st * LY::SB, bar);
    }
}

// Shifted values of population q for the cell pair (k, k+1) of one slab row:
// elements e0, e0+1 when c_z(q) = 0 (one aligned 4- or 8-byte load), else the
// two elements at the given offsets.
template <int KIND>
__device__ __forceinline__ f2 slab_pair(const unsigned char* slab, int q, int e0, int e1, bool adjacent) {
    if (KIND == ST_F32) {
        const float* p = reinterpret_cast<const float*>(slab);
        const float2 v = adjacent ? *reinterpret_cast<const float2*>(p + e0) : make_float2(p[e0], p[e1]);
        return {make_float2(v.x - wq(q), v.y - wq(q))};
    } else if (KIND == ST_F16S) {
        const __half* p = reinterpret_cast<const __half*>(slab);
        if (adjacent) return {__half22float2(*reinterpret_cast<const __half2*>(p + e0))};
        return {make_float2(__half2float(p[e0]), __half2float(p[e1]))};
    } else {
        const __nv_bfloat16* p = reinterpret_cast<const __nv_bfloat16*>(slab);
        if (adjacent) return {__bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p + e0))};
        return {make_float2(__bfloat162float(p[e0]), __bfloat162float(p[e1]))};
    }
}

// Store population q of the pair at cells idx, idx+1 (idx even: one aligned
// store).  `keep` masks the packed 16-bit pair (0xffff per live cell), so a solid
// cell stores its pinned shifted 0 without a select per value; FP32 takes the
// values as given.
template <int KIND>
__device__ __forceinline__ void store_pair(const FusedArgs& a, int q, int idx, float x, float y, unsigned keep) {
    if (KIND == ST_F32) {
        *reinterpret_cast<float2*>(reinterpret_cast<float*>(a.pout[q]) + idx) = make_float2(x + wq(q), y + wq(q));
    } else if (KIND == ST_F16S) {
        const __half2 v = __floats2half2_rn(x, y);
        *reinterpret_cast<unsigned*>(reinterpret_cast<__half*>(a.pout[q]) + idx) =
            *reinterpret_cast<const unsigned*>(&v) & keep;
    } else {
        const __nv_bfloat162 v = __floats2bfloat162_rn(x, y);
        *reinterpret_cast<unsigned*>(reinterpret_cast<__nv_bfloat16*>(a.pout[q]) + idx) =
            *reinterpret_cast<const unsigned*>(&v) & keep;
    }
}

struct Pair19 {
    f2 h[19];
};

// Lanes that the packed path cannot finish: solid cells that export, pulls
// that leave the grid (direct loads, links included), link cells of a tile
// whose slice was not staged, and the post-stream export of plane cells.
// (Kept inline: as a called function its argument copies and the call's
// register constraints slowed the whole pass by a fifth.)
template <int KIND>
__device__ __forceinline__ Pair19 slow_lanes(const FusedArgs* ap, Pair19 p, uint8_t fa, uint8_t fb, bool ea, bool eb,
                                          bool staged_links, int idx, int i, int j, int k) {
    const FusedArgs& a = *ap;
#pragma unroll
    for (int L = 0; L < 2; ++L) {
        const uint8_t fl = L ? fb : fa;
        const bool edge = L ? eb : ea;
        const int cell = idx + L;
        float t[19];
        if (fl & CF_SOLID) {
            if (fl & (CF_DEFER | CF_WRITE_S)) {
                solid_cell<KIND>(a, cell, i, j, k + L, t);
                export_f(a, cell, t);
            }
            continue;
        }
        const bool relink = (fl & CF_LINK) && !staged_links;
        if (!(edge | relink | ((fl & (CF_DEFER | CF_WRITE_S)) != 0))) continue;
        if (edge) {
            gather_cell<KIND>(a, cell, i, j, k + L, fl, t);
        } else {
#pragma unroll
            for (int q = 0; q < 19; ++q) t[q] = lane(p.h[q], L);
            if (relink) apply_links<KIND>(a, cell, __ldg(a.link_off + cell), t);
        }
        if (fl & (CF_DEFER | CF_WRITE_S)) export_f(a, cell, t);
#pragma unroll
        for (int q = 0; q < 19; ++q) set_lane(p.h[q], L, t[q]);
    }
    return p;
}

// One step of the passive tracer for one cell: fc_tracer_step's arithmetic with
// the same roundings (first-order upwind differences, clamp to [0, 1] keeping
// NaN, dissipation, zero in flow-solid cells; tracer_patch.py:55-82).
__device__ __forceinline__ float tracer_cell(float p, float xm, float xp, float ym, float yp, float zm, float zp,
                                             float uc, float vc, float wc, bool solid, float diss) {
    const float ax = uc >= 0.0f ? __fsub_rn(p, xm) : __fsub_rn(xp, p);
    const float ay = vc >= 0.0f ? __fsub_rn(p, ym) : __fsub_rn(yp, p);
    const float az = wc >= 0.0f ? __fsub_rn(p, zm) : __fsub_rn(zp, p);
    const float s = __fadd_rn(__fadd_rn(__fmul_rn(uc, ax), __fmul_rn(vc, ay)), __fmul_rn(wc, az));
    float n = __fsub_rn(p, s);
    if (!isnan(n)) n = fminf(fmaxf(n, 0.0f), 1.0f);
    n = __fmul_rn(n, diss);
    return solid ? 0.0f : n;
}

// The tracer step of a lane's two cells (i, j, k) and (i, j, k + 1), k even: the
// field and the velocity are read as 8-byte pairs, the upwind neighbours from
// every axis with periodic wrap (the field's torch.roll), and the pair written
// to the other tracer buffer.  Neighbour rows and planes are being read by the
// warps and CTAs working next to this one, so most of those loads hit L2.
__device__ __forceinline__ void tracer_pair(const FusedArgs& a, int i, int j, int k, int idx) {
    const int nyz = a.g.nynz, nz = a.g.nz;
    const int dxm = (i > 0 ? -1 : a.g.nx - 1) * nyz, dxp = (i + 1 < a.g.nx ? 1 : 1 - a.g.nx) * nyz;
    const int dym = (j > 0 ? -1 : a.g.ny - 1) * nz, dyp = (j + 1 < a.g.ny ? 1 : 1 - a.g.ny) * nz;
    const float* ph = a.tr_in;
    const float2 p = __ldg(reinterpret_cast<const float2*>(ph + idx));
    const float2 xm = __ldg(reinterpret_cast<const float2*>(ph + idx + dxm));
    const float2 xp = __ldg(reinterpret_cast<const float2*>(ph + idx + dxp));
    const float2 ym = __ldg(reinterpret_cast<const float2*>(ph + idx + dym));
    const float2 yp = __ldg(reinterpret_cast<const float2*>(ph + idx + dyp));
    const float zm = __ldg(ph + idx + (k > 0 ? -1 : nz - 1));        // k - 1 of cell k
    const float zp = __ldg(ph + idx + (k + 2 < nz ? 2 : 2 - nz));    // k + 2 of cell k + 1
    const float2 u = __ldg(reinterpret_cast<const float2*>(a.tr_u + idx));
    const float2 v = __ldg(reinterpret_cast<const float2*>(a.tr_v + idx));
    const float2 w = __ldg(reinterpret_cast<const float2*>(a.tr_w + idx));
    const unsigned sd = __ldg(reinterpret_cast<const unsigned short*>(a.tr_solid + idx));
    const float oa = tracer_cell(p.x, xm.x, xp.x, ym.x, yp.x, zm, p.y, u.x, v.x, w.x, (sd & 0xffu) != 0, a.tr_diss);
    const float ob = tracer_cell(p.y, xm.y, xp.y, ym.y, yp.y, p.x, zp, u.y, v.y, w.y, (sd >> 8) != 0, a.tr_diss);
    *reinterpret_cast<float2*>(a.tr_out + idx) = make_float2(oa, ob);
}

// Tile taken at position q of the pass: q itself, or counted from the end when the
// pass runs in descending order (every tile is computed the same either way).
__device__ __forceinline__ int tile_at(const FusedArgs& a, const TileGeo& tg, int q) {
    return a.tile_order ? tg.n_tiles - 1 - q : q;
}

// Record of the CTA's m-th tile (from the shared cache for the first ones).
__device__ __forceinline__ TileRec tile_rec(const FusedArgs& a, const TileRec* cache, int m, int t) {
    TileRec r;
    if (!a.tile_links) {
        r.lcb = r.lce = r.lb = r.le = 0;
#pragma unroll
        for (int c = 0; c < TS_PRE; ++c) r.pre[c] = 0;
        return r;
    }
    if (m < TS_RANGE_CACHE) return cache[m];
    const int4* g = reinterpret_cast<const int4*>(a.tile_links) + 2 * (size_t)t;
    const int4 x = __ldg(g), y = __ldg(g + 1);
    r.lcb = x.x; r.lce = x.y; r.lb = x.z; r.le = x.w;
    const int w[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
    for (int c = 0; c < TS_PRE; ++c) r.pre[c] = (unsigned short)(((unsigned)w[c >> 1] >> (16 * (c & 1))) & 0xffffu);
    return r;
}

template <int KIND, int MODE>
__global__ void __launch_bounds__(TS_THREADS, ts_min_blocks<KIND>())
    k_fused_tma(const __grid_constant__ FusedArgs a, const __grid_constant__ PopMaps tm_pop,
                const __grid_constant__ CUtensorMap tm_flag, const TileGeo tg) {
    using LY = Layout<KIND>;
    constexpr int S = LY::STAGES;
    // [0, 64): full mbarriers | [64, 128): per-stage done counters | record cache | stages
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t bar0 = su32(smem);
    int* done = reinterpret_cast<int*>(smem + 64);
    TileRec* rcache = reinterpret_cast<TileRec*>(smem + 128);
    unsigned char* stages = smem + TS_HEAD_BYTES;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;

    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            bar_init(bar0 + 8 * s, 1);
            done[s] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (a.tile_links)
        for (int m = tid; m < TS_RANGE_CACHE; m += TS_THREADS) {
            const long long t = (long long)blockIdx.x + (long long)m * G;
            if (t < tg.n_tiles) rcache[m] = tile_rec(a, rcache, TS_RANGE_CACHE, tile_at(a, tg, (int)t));
        }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            const int q = blockIdx.x + s * G;
            if (q < tg.n_tiles) {
                const int t = tile_at(a, tg, q);
                issue_tile<KIND>(a, &tm_pop, &tm_flag, tg, t, tile_rec(a, rcache, s, t), stages + s * LY::STAGE,
                                 bar0 + 8 * s);
            }
        }
    }

    // Warps take the chunks of the CTA's tiles in order, chunk w, w + 4, w + 8, ... of
    // the concatenated sequence, so the work stays balanced whatever the chunk
    // count of a tile.  Each warp waits for a stage's copies itself, and the
    // warp that completes a tile's last chunk refills its stage.
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const int nch = tg.tj * tg.kchunks;
    const int my_tiles = (int)blockIdx.x < tg.n_tiles ? (tg.n_tiles - 1 - (int)blockIdx.x) / G + 1 : 0;
    const int touching = nch < TS_WARPS ? nch : TS_WARPS;   // warps that take chunks of any one tile
    int ready_it = -1;                                       // last tile whose stage this warp saw complete
    // (it, ch): tile iteration and chunk of this warp's current chunk, advanced by TS_WARPS chunks
    int it = warp / nch, ch = warp - (warp / nch) * nch;
    while (it < my_tiles) {
        const int t = tile_at(a, tg, blockIdx.x + it * G);
        const int s = it % S;
        const int i = t / tg.tiles_j;
        const int j0 = (t - i * tg.tiles_j) * tg.tj;
        const float sg_plane = (a.sponge && a.sponge_axis == 0) ? __ldg(a.sponge + i) : 0.f;
        if (it != ready_it && !__all_sync(0xffffffffu, bar_wait(bar0 + 8 * s, (unsigned)(it / S) & 1u))) {
            if (lane == 0) {
                if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_TIMEOUT);
                // let copies still in flight land before the CTA can retire (bounded)
                for (int m = it + 1; m < it + S; ++m)
                    if ((long long)blockIdx.x + (long long)m * G < tg.n_tiles)
                        bar_wait(bar0 + 8 * (m % S), (unsigned)(m / S) & 1u);
            }
            return;
        }
        ready_it = it;

        const unsigned char* sb = stages + s * LY::STAGE;
        const uint8_t* sflag = sb + LY::FLAG;
        const TileInfo& ti = *reinterpret_cast<const TileInfo*>(sb + LY::INFO);
        const int staged = ti.staged;
        const bool plane_edge = ((i == 0) | (i == nx - 1)) & (a.g.px == 0);   // a periodic x wraps in the box
        const bool wrapped = ti.wrap != 0;
        do {   // one chunk; `continue` leaves it
            const int r = (ch * tg.kc_inv) >> 16;
            const int k = (ch - r * tg.kchunks) * 64 + 2 * lane;   // cells k, k+1 (nz is even)
            const int j = j0 + r;
            const bool valid = (j < ny) & (k < nz);
            const int off = r * nz + k;
            // place this chunk's link values into the slab elements its link cells pull
            if (staged > 0) {
                const int lo = ti.pre[ch], hi = min(ch + 1 < TS_PRE ? (int)ti.pre[ch + 1] : ti.nl, ti.nl);
                if (lo < hi) {
                    using T = typename Store<KIND>::T;
                    const uint16_t* spos = reinterpret_cast<const uint16_t*>(sb + LY::POS);
                    const T* sval = reinterpret_cast<const T*>(sb + LY::VAL);
                    T* slab = reinterpret_cast<T*>(const_cast<unsigned char*>(sb));
                    const int d = ti.lb - ti.lb0;
                    for (int l = lo + lane; l < hi; l += 32) {
                        const unsigned pos = spos[d + l];
                        if (pos < 19u * TS_TILE_CELLS) slab[pos] = sval[d + l];
                    }
                    __syncwarp();
                }
            }
            const unsigned fl2 = valid ? (unsigned)*reinterpret_cast<const uint16_t*>(sflag + off)
                                       : (unsigned)(CF_SOLID | (CF_SOLID << 8));
            const uint8_t fa = (uint8_t)(fl2 & 0xffu), fb = (uint8_t)(fl2 >> 8);
            if (!valid) continue;
            const int idx = (i * ny + j) * nz + k;
            if (a.tr_in) tracer_pair(a, i, j, k, idx);
            if ((fa & fb & CF_SOLID) && !((fa | fb) & (CF_DEFER | CF_WRITE_S))) continue;
            f2 h[19];
            {
                const int om = r * nz + (k > 0 ? k - 1 : nz - 1);        // source of cell k for c_z = +1
                const int op = r * nz + (k + 2 < nz ? k + 2 : 0);        // source of cell k+1 for c_z = -1
#pragma unroll
                for (int q = 0; q < 19; ++q) {
                    const unsigned char* slab = sb + q * LY::Q;
                    if (cz(q) == 0) h[q] = slab_pair<KIND>(slab, q, off, off + 1, true);
                    else if (cz(q) == 1) h[q] = slab_pair<KIND>(slab, q, om, off, false);
                    else h[q] = slab_pair<KIND>(slab, q, off + 1, op, false);
                }
            }
            const bool live_a = !(fa & CF_SOLID), live_b = !(fb & CF_SOLID);
            // Direct loads where a pull leaves the staged boxes: rows across an unstaged y
            // boundary, cells on a non-periodic z boundary, and x-boundary cells that are not
            // inlet/outlet plane cells.  On an inlet/outlet plane the pulls that leave the
            // grid are exactly the plane's unknown directions, which the plane kernel
            // replaces before anything reads them (Zou/He rebuilds them, the convective
            // outlet copies them from the interior), so those cells keep the staged values.
            const bool edge_row = ((j == 0) | (j == ny - 1)) & !wrapped;
            const bool ea = live_a & (edge_row | (plane_edge & !(fa & CF_DEFER)) | ((a.g.pz == 0) & (k == 0)));
            const bool eb = live_b & (edge_row | (plane_edge & !(fb & CF_DEFER)) | ((a.g.pz == 0) & (k + 1 == nz - 1)));
            const bool link_a = live_a && (fa & CF_LINK), link_b = live_b && (fb & CF_LINK);
            const bool unstaged = staged < 0;
            if (ea | eb | (unstaged & (link_a | link_b)) | (((fa | fb) & (CF_DEFER | CF_WRITE_S)) != 0)) {
                Pair19 p;
#pragma unroll
                for (int q = 0; q < 19; ++q) p.h[q] = h[q];
                p = slow_lanes<KIND>(&a, p, fa, fb, ea, eb, !unstaged, idx, i, j, k);
#pragma unroll
                for (int q = 0; q < 19; ++q) h[q] = p.h[q];
            }
            const MacroV<f2> m = collide_h<MODE>(h, a.cp);
            if (a.sponge) {
                float sa = sg_plane, sbv = sg_plane;
                if (a.sponge_axis == 1) {
                    sa = sbv = __ldg(a.sponge + j);
                } else if (a.sponge_axis == 2) {
                    sa = __ldg(a.sponge + k);
                    sbv = __ldg(a.sponge + k + 1);
                }
                if ((sa > 0.f) | (sbv > 0.f)) {
                    f2 heq[19];
                    equilibrium_h(m, heq);
                    const f2 nsg = {make_float2(-sa, -sbv)};
                    if ((sa > 0.f) & (sbv > 0.f)) {
#pragma unroll
                        for (int q = 0; q < 19; ++q) h[q] = fma(nsg, h[q] - heq[q], h[q]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 19; ++q) {
                            const f2 hs = fma(nsg, h[q] - heq[q], h[q]);
                            h[q].v.x = sa > 0.f ? hs.v.x : h[q].v.x;
                            h[q].v.y = sbv > 0.f ? hs.v.y : h[q].v.y;
                        }
                    }
                }
            }
            // deferred cells are stored too: the plane pass overwrites them after the BCs.
            // Solid cells get their pinned state (shifted 0, macros 1,0,0,0).
            if constexpr (KIND == ST_F32) {
#pragma unroll
                for (int q = 0; q < 19; ++q)
                    store_pair<KIND>(a, q, idx, live_a ? h[q].v.x : 0.f, live_b ? h[q].v.y : 0.f, 0u);
            } else {
                const unsigned keep = (live_a ? 0x0000ffffu : 0u) | (live_b ? 0xffff0000u : 0u);
#pragma unroll
                for (int q = 0; q < 19; ++q) store_pair<KIND>(a, q, idx, h[q].v.x, h[q].v.y, keep);
            }
            if (a.rho) {
                *reinterpret_cast<float2*>(a.rho + idx) =
                    make_float2(live_a ? m.rho.v.x : 1.f, live_b ? m.rho.v.y : 1.f);
                *reinterpret_cast<float2*>(a.u + idx) = make_float2(live_a ? m.ux.v.x : 0.f, live_b ? m.ux.v.y : 0.f);
                *reinterpret_cast<float2*>(a.v + idx) = make_float2(live_a ? m.uy.v.x : 0.f, live_b ? m.uy.v.y : 0.f);
                *reinterpret_cast<float2*>(a.w + idx) = make_float2(live_a ? m.uz.v.x : 0.f, live_b ? m.uz.v.y : 0.f);
            }
        } while (false);
        // after its last chunk of a tile the warp is done with the stage; the last
        // warp done refills it with the tile S iterations ahead
        __syncwarp();
        if (lane == 0 && ch + TS_WARPS >= nch) {
            __threadfence_block();
            if (atomicAdd(done + s, 1) == touching - 1) {
                done[s] = 0;
                const int qn = blockIdx.x + (it + S) * G;
                if (qn < tg.n_tiles) {
                    const int tn = tile_at(a, tg, qn);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue_tile<KIND>(a, &tm_pop, &tm_flag, tg, tn, tile_rec(a, rcache, it + S, tn),
                                     stages + s * LY::STAGE, bar0 + 8 * s);
                }
            }
        }
        ch += TS_WARPS;
        while (ch >= nch) {
            ch -= nch;
            ++it;
        }
    }
}

// Per-tile link ranges: first link cell at or after the tile's first cell and
// first link cell at or after its end (binary search in the ascending list),
// with the matching link offsets from the headers.
__device__ __forceinline__ int lower_bound_cells(const int* cells, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cells + mid) < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int first_link_at(const FusedArgs& a, int cell) {
    const int n = (int)a.n_link_cells;
    const int lc = lower_bound_cells(a.link_cells, n, cell);
    return lc < n ? (int)__ldg(a.link_hdr + lc).z : (int)a.n_links;
}

__global__ void k_tile_links(const FusedArgs a, TileGeo tg, int4* out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tg.n_tiles) return;
    const int i = t / tg.tiles_j;
    const int j0 = (t - i * tg.tiles_j) * tg.tj;
    const int j1 = min(j0 + tg.tj, a.g.ny);
    const int c0 = (i * a.g.ny + j0) * a.g.nz, c1 = (i * a.g.ny + j1) * a.g.nz;
    const int n = (int)a.n_link_cells;
    const int lcb = lower_bound_cells(a.link_cells, n, c0);
    const int lce = lower_bound_cells(a.link_cells, n, c1);
    const int lb = lcb < n ? (int)__ldg(a.link_hdr + lcb).z : (int)a.n_links;
    const int le = lce < n ? (int)__ldg(a.link_hdr + lce).z : (int)a.n_links;
    // first link of each chunk (64 cells of a row, tile order), from the tile's first link
    unsigned short pre[TS_PRE];
    const int nch = tg.tj * tg.kchunks;
    for (int c = 0; c < TS_PRE; ++c) {
        int first = le;
        if (c < nch) {
            const int r = c / tg.kchunks, kc = (c - r * tg.kchunks) * 64;
            if (j0 + r < a.g.ny) first = first_link_at(a, (i * a.g.ny + j0 + r) * a.g.nz + kc);
        }
        pre[c] = (unsigned short)(first - lb);
    }
    out[2 * t] = make_int4(lcb, lce, lb, le);
    out[2 * t + 1] = make_int4((int)(pre[0] | ((unsigned)pre[1] << 16)), (int)(pre[2] | ((unsigned)pre[3] << 16)),
                               (int)(pre[4] | ((unsigned)pre[5] << 16)), (int)(pre[6] | ((unsigned)pre[7] << 16)));
}

// Staged-tile element that each link's value replaces: slab d at the element
// cell (r, k) pulls for direction d, (r, k - c_z(d)) with the row wrap of a
// periodic z axis; 0xffff where that leaves a non-periodic row (such cells
// take the direct-load path).
__global__ void k_link_pos(const FusedArgs a, TileGeo tg, uint16_t* pos) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_link_cells) return;
    const int idx = __ldg(a.link_cells + t);
    const uint4 hd = __ldg(a.link_hdr + t);
    if (idx < 0 || (long long)idx >= a.g.N || (long long)hd.z + __popc(hd.x) > a.n_links) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    const int nz = a.g.nz;
    const int k = idx % nz;
    const int j = (idx / nz) % a.g.ny;
    const int r = j - (j / tg.tj) * tg.tj;
    unsigned rank = 0;
    for (int d = 1; d < 19; ++d) {
        if (!(hd.x & (1u << d))) continue;
        int kk = k - cz(d);
        if (kk < 0 || kk >= nz) kk = a.g.pz ? (kk + nz) % nz : -1;
        pos[hd.z + rank] = kk < 0 ? (uint16_t)0xffffu : (uint16_t)(d * TS_TILE_CELLS + r * nz + kk);
        ++rank;
    }
}

// Per-link element pairs of the link gather: f_opp(d) at the link cell, and
// the second value (f_opp(d) at x_f - c_d, or f_d at x_f); bit 31 of the first
// marks an edge direction (lattice weight 1/36).
__global__ void k_link_src(const FusedArgs a, uint2* src) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n_link_cells) return;
    const int idx = __ldg(a.link_cells + t);
    const uint4 hd = __ldg(a.link_hdr + t);
    if (idx < 0 || (long long)idx >= a.g.N || (long long)hd.z + __popc(hd.x) > a.n_links) {
        if (a.dev_err) atomicOr(a.dev_err, DEV_ERR_INDEX);
        return;
    }
    const unsigned N = (unsigned)a.g.N;
    unsigned rank = 0;
    for (int d = 1; d < 19; ++d) {
        if (!(hd.x & (1u << d))) continue;
        const int o = opp(d);
        const bool second = (hd.y >> d) & 1u;
        const int off = cx(d) * a.g.nynz + cy(d) * a.g.nz + cz(d);
        const unsigned e1 = (unsigned)o * N + (unsigned)idx;
        const unsigned e2 = second ? (unsigned)o * N + (unsigned)(idx - off) : (unsigned)d * N + (unsigned)idx;
        src[hd.z + rank] = make_uint2(e1 | (d > 6 ? 0x80000000u : 0u), e2);
        ++rank;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int storage_bytes(int storage) { return storage == ST_F32 ? 4 : 2; }

TileGeo tile_geo(const Geo& g, int storage) {
    const int sb = storage_bytes(storage);
    TileGeo tg;
    tg.kchunks = (g.nz + 63) / 64;
    tg.tj = TS_TILE_CELLS / g.nz;                        // whole rows within 512 cells ...
    if (tg.tj > TS_PRE / tg.kchunks) tg.tj = TS_PRE / tg.kchunks;   // ... and within 8 chunks
    if (tg.tj > g.ny) tg.tj = g.ny;
    if (tg.tj < 1) tg.tj = 1;
    tg.tiles_j = (g.ny + tg.tj - 1) / tg.tj;
    tg.n_tiles = tg.tiles_j * g.nx;
    tg.kc_inv = (65536 + tg.kchunks - 1) / tg.kchunks;
    const int cells = tg.tj * g.nz;
    tg.base_tx = (uint32_t)(19 * cells * sb + cells);
    // the periodic y wrap is staged when every plane has a separate first and last tile of full
    // rows and a row boundary inside a slab keeps the 128-byte alignment of tensor-copy targets
    tg.wrap_y = (g.py != 0) && tg.tiles_j >= 2 && g.ny % tg.tj == 0 && (tg.tj == 1 || (g.nz * sb) % 128 == 0);
    return tg;
}

template <int KIND>
size_t smem_bytes() { return TS_HEAD_BYTES + (size_t)Layout<KIND>::STAGES * Layout<KIND>::STAGE; }

// a row is read as nseg box segments of at most 256 elements each
int row_segments(int nz) { return (nz + 255) / 256; }

bool grid_fits(const Geo& g) {
    // whole rows within a tile (at most 512 cells), segments of a multiple of
    // 16 elements (16-byte flag segments), int cell indices
    if (g.nz < 16 || g.nz > TS_TILE_CELLS || g.N >= (1LL << 31)) return false;
    return g.nz % (16 * row_segments(g.nz)) == 0;
}

template <int S, int M>
int launch_typed(const FusedArgs& a, const PopMaps& tp, const CUtensorMap& tf, const TileGeo& tg,
                 cudaStream_t st) {
    auto kern = k_fused_tma<S, M>;
    static int configured = 0;
    static std::once_flag once;
    std::call_once(once, [&] {
        configured = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
                         cudaSuccess &&
                     cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100) == cudaSuccess;
    });
    if (!configured) return FC_ERR_LAUNCH;
    const size_t smem = smem_bytes<S>();
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FC_ERR_LAUNCH;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FC_ERR_LAUNCH;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TS_THREADS, smem) != cudaSuccess ||
        per_sm < 1)
        return FC_ERR_LAUNCH;
    long long grid = (long long)sms * per_sm;
    if (grid > tg.n_tiles) grid = tg.n_tiles;
    kern<<<(unsigned)grid, TS_THREADS, smem, st>>>(a, tp, tf, tg);
    return launch_status();
}

// The pass's bounded mbarrier wait on its own: one warp waits on a barrier of
// arrival count 1.  With arrive == 0 nothing arrives, so the wait gives up after
// `polls` polls and the kernel records DEV_ERR_TIMEOUT and returns; with
// arrive == 1 lane 0 arrives first and the wait completes.
__global__ void k_wait_selftest(unsigned polls, int arrive, unsigned* status) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = su32(&bar);
    if (threadIdx.x == 0) {
        bar_init(b, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
    __syncwarp();
    const bool ok = __all_sync(0xffffffffu, bar_wait(b, 0u, polls));
    if (!ok && threadIdx.x == 0) atomicOr(status, DEV_ERR_TIMEOUT);
}

}  // namespace

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda link)
EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    });
    return fn;
}

bool fused_tma_eligible(const FusedArgs& a, int storage) {
    const Geo& g = a.g;
    if (!grid_fits(g)) return false;
    if (!encode_tiled()) return false;
    const uintptr_t pin = reinterpret_cast<uintptr_t>(a.pin[0]), fl = reinterpret_cast<uintptr_t>(a.flags);
    if ((pin & 15) || (fl & 15)) return false;
    if (a.link_val && (reinterpret_cast<uintptr_t>(a.link_val) & 15)) return false;
    const TileGeo tg = tile_geo(g, storage);
    if (a.tile_links && a.n_tile_links != tg.n_tiles) return false;
    return true;
}

long long tma_tile_links(const FusedArgs& a, int4* out, long long cap, uint16_t* pos, long long pos_cap,
                         uint2* src, long long src_cap, cudaStream_t st) {
    if (!grid_fits(a.g)) return 0;
    const TileGeo tg = tile_geo(a.g, ST_F32);
    if (!out) return tg.n_tiles;
    if (cap < tg.n_tiles) return -FC_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(out) & 15) return -FC_ERR_ARG;
    if (a.n_links > 0 && (!a.link_cells || !a.link_hdr || a.n_link_cells <= 0)) return -FC_ERR_ARG;
    if (pos && (pos_cap < a.n_links + 8 || (reinterpret_cast<uintptr_t>(pos) & 15))) return -FC_ERR_ARG;
    if (a.n_links <= 0) {
        if (cudaMemsetAsync(out, 0, 2 * sizeof(int4) * (size_t)tg.n_tiles, st) != cudaSuccess)
            return -FC_ERR_LAUNCH;
        return tg.n_tiles;
    }
    k_tile_links<<<(tg.n_tiles + 127) / 128, 128, 0, st>>>(a, tg, out);
    int rc = launch_status();
    if (rc) return -rc;
    if (pos) {
        if (cudaMemsetAsync(pos, 0xff, sizeof(uint16_t) * (size_t)pos_cap, st) != cudaSuccess) return -FC_ERR_LAUNCH;
        k_link_pos<<<(unsigned)((a.n_link_cells + 127) / 128), 128, 0, st>>>(a, tg, pos);
        rc = launch_status();
        if (rc) return -rc;
    }
    if (src) {
        if (src_cap < a.n_links + 8 || (reinterpret_cast<uintptr_t>(src) & 7) || 19LL * a.g.N >= (1LL << 31))
            return -FC_ERR_ARG;
        if (cudaMemsetAsync(src, 0, sizeof(uint2) * (size_t)src_cap, st) != cudaSuccess) return -FC_ERR_LAUNCH;
        k_link_src<<<(unsigned)((a.n_link_cells + 127) / 128), 128, 0, st>>>(a, src);
        rc = launch_status();
        if (rc) return -rc;
    }
    return tg.n_tiles;
}

int launch_fused_tma(const FusedArgs& a, int storage, int collision, cudaStream_t st) {
    if (!fused_tma_eligible(a, storage)) return FC_ERR_UNSUPPORTED;
    const Geo& g = a.g;
    const TileGeo tg = tile_geo(g, storage);
    const int sb = storage_bytes(storage);
    PopMaps tp;
    CUtensorMap tf;
    const int nseg = row_segments(g.nz), seg = g.nz / nseg;
    for (int m = 0; m < 3; ++m) {
        // box heights: tj rows, tj - 1 rows (at least 1), one row
        const int rows = m == 0 ? tg.tj : (m == 1 ? (tg.tj > 1 ? tg.tj - 1 : 1) : 1);
        CUtensorMap* map = m == 0 ? &tp.full : (m == 1 ? &tp.shrt : &tp.row);
        // (segment element, segment, row, plane, population): a row is nseg contiguous segments
        const cuuint64_t dims[5] = {(cuuint64_t)seg, (cuuint64_t)nseg, (cuuint64_t)g.ny, (cuuint64_t)g.nx, 19};
        const cuuint64_t strides[4] = {(cuuint64_t)seg * sb, (cuuint64_t)g.nz * sb, (cuuint64_t)g.nynz * sb,
                                       (cuuint64_t)g.N * sb};
        const cuuint32_t box[5] = {(cuuint32_t)seg, (cuuint32_t)nseg, (cuuint32_t)rows, 1, 1};
        const cuuint32_t es[5] = {1, 1, 1, 1, 1};
        const CUtensorMapDataType dt = storage == ST_F32    ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                       : storage == ST_F16S ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                            : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
        if (encode_tiled()(map, dt, 5, const_cast<void*>(a.pin[0]), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return FC_ERR_UNSUPPORTED;
    }
    {
        const cuuint64_t dims[4] = {(cuuint64_t)seg, (cuuint64_t)nseg, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
        const cuuint64_t strides[3] = {(cuuint64_t)seg, (cuuint64_t)g.nz, (cuuint64_t)g.nynz};
        const cuuint32_t box[4] = {(cuuint32_t)seg, (cuuint32_t)nseg, (cuuint32_t)tg.tj, 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        if (encode_tiled()(&tf, CU_TENSOR_MAP_DATA_TYPE_UINT8, 4, const_cast<uint8_t*>(a.flags), dims, strides, box,
                           es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return FC_ERR_UNSUPPORTED;
    }
#define FC_TMA_CASE(S, M) \
    if (storage == S && collision == M) return launch_typed<S, M>(a, tp, tf, tg, st);
    FC_TMA_CASE(ST_F32, CM_BGK) FC_TMA_CASE(ST_F32, CM_TRT) FC_TMA_CASE(ST_F32, CM_MRT)
    FC_TMA_CASE(ST_F32, CM_MRT_SMAG) FC_TMA_CASE(ST_F16S, CM_BGK) FC_TMA_CASE(ST_F16S, CM_TRT)
    FC_TMA_CASE(ST_F16S, CM_MRT) FC_TMA_CASE(ST_F16S, CM_MRT_SMAG) FC_TMA_CASE(ST_BF16S, CM_BGK)
    FC_TMA_CASE(ST_BF16S, CM_TRT) FC_TMA_CASE(ST_BF16S, CM_MRT) FC_TMA_CASE(ST_BF16S, CM_MRT_SMAG)
#undef FC_TMA_CASE
    return FC_ERR_ARG;
}

}  // namespace fc

extern "C" int fc_lbm_wait_selftest(unsigned polls, int arrive, unsigned* status, void* stream) {
    if (!status || polls < 1) return fc::FC_ERR_ARG;
    fc::k_wait_selftest<<<1, 32, 0, (cudaStream_t)stream>>>(polls, arrive, status);
    return fc::launch_status();
}
