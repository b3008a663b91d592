/*
 * fluxcore3d_gb300.h -- C ABI of libfluxcore3d_gb300.so (sm_103a kernels for the
 * conjugate-heat-transfer hot path: D3Q19 lattice Boltzmann, interpolated
 * bounce-back, multigrid / Krylov thermal solve).
 *
 * Conventions
 *   - Every pointer argument is a device pointer unless its name ends in _host.
 *   - Every function returns an int status: 0 ok, 1 bad argument, 2 launch
 *     failure, 3 unsupported combination, 4 size beyond a fixed capacity.  Nothing in this library allocates
 *     device memory behind the caller's back: scratch space is passed in as a
 *     workspace pointer whose size the matching *_workspace_bytes() reports.
 *   - `stream` is a cudaStream_t passed as void*; NULL is the legacy stream.
 *   - Populations are [19][N] row-major with N = nx*ny*nz and cell index
 *     flat = i*ny*nz + j*nz + k, direction order of the reference solver.
 *
 * Each declaration names the reference interface it replaces (file:line in
 * the fluxcore3D tree).
 */
#ifndef FLUXCORE3D_GB300_H
#define FLUXCORE3D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FC_ABI_VERSION 2

int fc_abi_version(void);

/* ---------------------------------------------------------------------------
 * Per-operation lattice kernels (the LBM_CUDA module surface)
 * ------------------------------------------------------------------------- */

/* replaces LBM_CUDA.macro_collide_bgk  (solver/lbm_kernels.cu:628-646) */
int fc_lbm_macro_collide_bgk(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, float omega, long long n_cells, void* stream);
/* replaces LBM_CUDA.macro_collide_trt  (solver/lbm_kernels.cu:649-668) */
int fc_lbm_macro_collide_trt(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, float omega_plus, float omega_minus, long long n_cells,
                             void* stream);
/* replaces LBM_CUDA.macro_collide_mrt  (solver/lbm_kernels.cu:671-692); S_dev: 19 floats on the device */
int fc_lbm_macro_collide_mrt(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                             const uint8_t* solid, const float* S_dev, long long n_cells, void* stream);
/* replaces LBM_CUDA.macro_collide_mrt_smag  (solver/lbm_kernels.cu:1120-1145) */
int fc_lbm_macro_collide_mrt_smag(const float* f, float* f_post, float* rho, float* u, float* v, float* w,
                                  const uint8_t* solid, const float* S_dev, float Cs_dx2, float omega0,
                                  long long n_cells, void* stream);
/* replaces LBM_CUDA.stream_pull  (solver/lbm_kernels.cu:695-708) */
int fc_lbm_stream_pull(const float* f_in, float* f_out, int nx, int ny, int nz, int px, int py, int pz,
                       void* stream);
/* replaces LBM_CUDA.sponge  (solver/lbm_kernels.cu:711-727) */
int fc_lbm_sponge(float* f, const float* rho, const float* u, const float* v, const float* w,
                  const float* sigma, long long n_cells, void* stream);
/* replaces LBM_CUDA.ibb  (solver/lbm_kernels.cu:730-754); dev_err may be NULL */
int fc_lbm_ibb(const float* f_post, float* f_stream, const int32_t* fluid_flat, const int32_t* dir_i,
               const int32_t* dir_opp, const float* w1, const float* w2, const uint8_t* q_ge_half,
               const int32_t* ff_flat, const uint8_t* ff_valid, long long n_links, long long n_cells,
               unsigned* dev_err, void* stream);
/* replaces LBM_CUDA.reset_solid  (solver/lbm_kernels.cu:757-764) */
int fc_lbm_reset_solid(float* f, const uint8_t* solid, long long n_cells, void* stream);
/* replaces LBM_CUDA.zou_he_bc  (solver/lbm_kernels.cu:975-996) */
int fc_lbm_zou_he_bc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int plane_idx,
                     int interior_idx, int bc_type, float u_in_lat, float rho_out_lat, int sign, void* stream);
/* replaces LBM_CUDA.convective_bc  (solver/lbm_kernels.cu:1299-1344).  The reference keeps two
 * process-global device scalars; here the caller passes a workspace of
 * fc_lbm_convective_workspace_bytes(n1, n2) bytes (8-byte aligned) and the
 * plane reduction is deterministic (fixed-order FP64 tree). */
long long fc_lbm_convective_workspace_bytes(int n1, int n2);
int fc_lbm_convective_bc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                         int interior_idx, int unknown_cax, float rho_out_lat, int n1, int n2,
                         void* workspace, long long workspace_bytes, void* stream);
/* FP64 run of the plain method: the per-operation kernels above on double populations and
 * macros, for reporting the error of the FP32 and FP16/BF16 runs against an FP64 run of the
 * same step sequence (no counterpart in the reference, which is FP32 only).  Rates, sponge
 * profile and link weights keep their FP32 values.  collision: 0 BGK, 1 TRT, 2 MRT, 3 MRT +
 * Smagorinsky; S_dev (19 floats on the device) is read for 2 and 3. */
int fc_lbm64_macro_collide(int collision, const double* f, double* f_post, double* rho, double* u, double* v,
                           double* w, const uint8_t* solid, float omega, float omega_plus, float omega_minus,
                           const float* S_dev, float Cs_dx2, float omega0, long long n_cells, void* stream);
int fc_lbm64_stream_pull(const double* f_in, double* f_out, int nx, int ny, int nz, int px, int py, int pz,
                         void* stream);
int fc_lbm64_sponge(double* f, const double* rho, const double* u, const double* v, const double* w,
                    const float* sigma, long long n_cells, void* stream);
int fc_lbm64_ibb(const double* f_post, double* f_stream, const int32_t* fluid_flat, const int32_t* dir_i,
                 const int32_t* dir_opp, const float* w1, const float* w2, const uint8_t* q_ge_half,
                 const int32_t* ff_flat, const uint8_t* ff_valid, long long n_links, long long n_cells,
                 unsigned* dev_err, void* stream);
int fc_lbm64_reset_solid(double* f, const uint8_t* solid, long long n_cells, void* stream);
int fc_lbm64_zou_he_bc(double* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int plane_idx,
                       int interior_idx, int bc_type, double u_in_lat, double rho_out_lat, int sign, void* stream);
int fc_lbm64_convective_bc(double* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                           int interior_idx, int unknown_cax, double rho_out_lat, int n1, int n2, void* workspace,
                           long long workspace_bytes, void* stream);
/* Convective outlet that allocates nothing: no counterpart in the reference.  For callers
 * that may not allocate device memory once their time loop runs (a host that hands out all
 * GPU memory from its own pre-reserved arena, or a path where an allocation would
 * synchronise the device).  Same result as fc_lbm_convective_bc, with the plane partials
 * kept in a fixed file-scope device array (49,152 bytes per GPU that loads the library,
 * held until exit): planes of at most fc_lbm_convective_noalloc_max_plane() = 1,048,576
 * nodes, larger ones return 4.  The first call on each device looks the array up and
 * caches its address; make it before any stream capture.  Calls share the array, so calls
 * that overlap on the GPU race on it. */
long long fc_lbm_convective_noalloc_max_plane(void);
int fc_lbm_convective_bc_noalloc(float* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx,
                                 int interior_idx, int unknown_cax, float rho_out_lat, int n1, int n2, void* stream);

/* ---------------------------------------------------------------------------
 * Fused step (replaces the collide -> sponge -> stream -> ibb -> reset_solid
 * launch sequence of LBMCUDAUpgrade._step_cuda, solver/lbm_cuda_ext.py:445-517)
 * ------------------------------------------------------------------------- */
typedef struct fc_lbm_step_args {
    int32_t storage;         /* 0 FP32, 1 FP16 shifted (f - w_q), 2 BF16 shifted */
    int32_t collision;       /* 0 BGK, 1 TRT, 2 MRT, 3 MRT + Smagorinsky */
    int32_t nx, ny, nz;
    int32_t periodic[3];     /* per-axis periodic streaming flags */
    const void* pop_in;      /* [19][N] post-collision populations of the previous step */
    void* pop_out;           /* [19][N] post-collision populations of this step */
    float* f32;              /* [19][N] FP32 post-stream export (cells flagged DEFER / WRITE_S) */
    float* rho;              /* [N] macro outputs, or NULL to skip the macro write */
    float* u;
    float* v;
    float* w;
    const uint8_t* cell_flags;   /* [N] bit0 solid, bit1 has links, bit2 deferred plane, bit3 export */
    const int32_t* link_off;     /* [N] link-cell ordinal of the cell (read only where bit1 is set) */
    const uint32_t* link_hdr;    /* [n_link_cells][4] (dir mask, second-node mask, first weight, 0); 16-B aligned */
    const float* link_w;         /* [n_links][2] (w1, w2) per link, cells in ordinal order, dirs ascending */
    long long n_links;
    const float* sponge;         /* sigma per plane along sponge_axis, or NULL */
    int32_t sponge_axis;
    int32_t has_links;           /* 0: solid cells export the in-cell swap (no-link bounce-back) */
    float omega, omega_plus, omega_minus;
    float S[19];
    float Cs_dx2, omega0;
    unsigned* dev_err;           /* device error word (bit0 index out of range), may be NULL */
    const int32_t* link_cells;   /* [n_link_cells] ascending cell list (ordinal order) */
    long long n_link_cells;
    int32_t phase_mask;          /* bit0 main pass, bit1 link-cell pass (0 is read as 3) */
    int32_t separate_link_pass;  /* 1: the main pass skips link cells and a second kernel runs them */
    int32_t cells_per_thread;    /* 1 or 2 (two rows per thread in the main pass); 0 is read as 1 */
    int32_t staging;             /* 0: main pass stages tiles of rows in shared memory with TMA when the
                                    grid allows it (16 <= nz <= 512, nz a multiple of 16 per 256-element
                                    row segment, no separate link pass, one cell per thread), 1: per-thread
                                    global loads always */
    void* link_val;              /* optional scratch of n_links + 8 elements of the population storage type:
                                    when set, each step first gathers every link's interpolated bounce-back
                                    value into it in storage form (one thread per link cell, needs
                                    link_cells) and both passes read those values */
    int64_t n_link_val;          /* capacity of link_val in elements */
    const int32_t* tile_links;   /* optional, from fc_lbm_tile_links: one 8 x int32 record per staged tile
                                    (link-cell range, link range, per-chunk link offsets); with link_pos it
                                    lets the staged pass place link values straight into its tiles */
    int64_t n_tile_links;        /* number of records in tile_links */
    const uint16_t* link_pos;    /* optional, from fc_lbm_tile_links: per link, the element of the staged
                                    tile that its value replaces (0xffff: none); n_links + 8 entries */
    int64_t n_link_pos;          /* capacity of link_pos in entries */
    const uint32_t* link_src;    /* optional, from fc_lbm_tile_links: per link two population element
                                    indices (q N + cell) of the values it blends, the first with bit 31 set
                                    for an edge direction (bit 31 of the second: caller's mark, see
                                    fc_lbm_link_gather); lets the gather run one thread per link */
    int64_t n_link_src;          /* capacity of link_src in links (2 entries each) */
    int32_t skip_link_gather;    /* 1: fc_lbm_fused_step does not run the link gather; the caller runs
                                    fc_lbm_link_gather for this step's input beforehand (e.g. on a second
                                    stream while the previous step's plane work runs) */
    /* Optional passive tracer carried by the main pass (tracer_in == NULL: none).  The step also
     * performs exactly one fc_tracer_step(tracer_in -> tracer_out, tracer_u/v/w, tracer_solid,
     * tracer_dissipation): inside the staged main pass when that pass runs, as its own launch
     * otherwise; the field is the same bit for bit either way.  tracer_u/v/w are the velocity the
     * tracer is advected by -- for the reference's wrapped step, the macros the lattice exposes
     * after this step, i.e. the ones the previous step wrote -- and must not be this step's macro
     * outputs.  Replaces the separate TracerField.step launch after each sim.step
     * (pre_post/tracer_patch.py:55-82, 100-124). */
    const float* tracer_in;
    float* tracer_out;
    const float* tracer_u;
    const float* tracer_v;
    const float* tracer_w;
    const uint8_t* tracer_solid;
    float tracer_dissipation;
    /* Order in which the staged main pass takes its tiles (0: ascending cells, 1: descending) and in
     * which the link gather takes its links.  The results do not depend on either; alternating the
     * pass order every step and running the gather opposite to the pass that wrote its input makes
     * both start on the cells written last, which are still in L2.  No reference counterpart. */
    int32_t tile_order;
    int32_t gather_order;
} fc_lbm_step_args;

/* One full time step for every non-deferred cell. */
int fc_lbm_fused_step(const fc_lbm_step_args* args, void* stream);
/* sizeof(fc_lbm_step_args) as compiled, so a binding can check its mirror of the struct.
 * No reference counterpart. */
long long fc_lbm_step_args_size(void);

/* Tiles of the TMA-staged main pass for this grid.  With records == NULL
 * returns the number of tiles (0 when the staged pass does not apply to the
 * grid).  Otherwise fills records[8 t .. 8 t + 7] for every tile t -- (first
 * link cell, end link cell, first link, end link) from link_cells / link_hdr,
 * then eight 16-bit offsets, from the tile's first link, of the first link of
 * each of its 64-cell chunks -- and, when link_pos is given (pos_cap >=
 * n_links + 8), the staged-tile element each link's value replaces; returns
 * the tile count (cap = records that fit), or a negative status.  With
 * link_src (src_cap >= n_links + 8 links, grid below 113 M cells) it also
 * fills the per-link element pairs of the link gather.  All of it depends
 * only on the geometry: compute it once after the link tables are built.
 * No reference counterpart (the reference has no staged pass). */
long long fc_lbm_tile_links(const fc_lbm_step_args* args, int32_t* records, long long cap, uint16_t* link_pos,
                            long long pos_cap, uint32_t* link_src, long long src_cap, void* stream);
/* The per-step link gather of fc_lbm_fused_step on its own: interpolated
 * bounce-back values from args->pop_in into args->link_val, for every link
 * (subset == NULL; with skip_marked, links whose link_src second index has
 * bit 31 set are left out) or for the n_subset links listed in subset.  A
 * caller marks the links that read cells of inlet/outlet planes, gathers the
 * rest concurrently with the previous step's plane work and the marked ones
 * after it.  No reference counterpart (the reference evaluates links inside
 * its IBB kernel). */
int fc_lbm_link_gather(const fc_lbm_step_args* args, const int32_t* subset, long long n_subset, int skip_marked,
                       void* stream);

/* Failure-detection check of the staged pass's bounded mbarrier wait (the
 * helper every wait of k_fused_tma uses), in a one-warp kernel: with arrive == 0
 * nothing arrives on the barrier, the wait gives up after `polls` polls, and the
 * kernel sets bit 4 (timeout) in *status and returns, leaving the context
 * usable; with arrive == 1 the phase completes and *status is not touched.
 * No reference counterpart (the reference has no bounded device waits). */
int fc_lbm_wait_selftest(unsigned polls, int arrive, unsigned* status, void* stream);

/* One inlet/outlet plane with a node-local (Zou/He) boundary condition. */
typedef struct {
    int32_t axis, plane_idx, interior_idx, bc_type;   /* bc_type 0 velocity, 1 pressure (as fc_lbm_zou_he_bc) */
    float u_in_lat, rho_out_lat;
    int32_t sign, pad;
} fc_plane_bc;
#define FC_MAX_PLANES 6
/* Zou/He on up to FC_MAX_PLANES planes of one axis (distinct plane indices),
 * each node's boundary condition on args->f32 followed by its collision into
 * args->pop_out: fc_lbm_zou_he_bc on every plane in order and then
 * fc_lbm_collide_from_f32 on every plane, in one launch (the conditions are
 * node-local and the planes disjoint, so the per-node order is the same).
 * Fusion of reference lbm_kernels.cu:791-969 with the plane collision. */
int fc_lbm_planes_zou_he_collide(const fc_lbm_step_args* args, const fc_plane_bc* planes, int n_planes,
                                 void* stream);

/* Collide cells straight from args->f32: axis < 0 => every fluid cell (start-up),
 * else the plane plane_idx along axis (after that plane's boundary condition). */
int fc_lbm_collide_from_f32(const fc_lbm_step_args* args, int axis, int plane_idx, void* stream);
/* Rebuild post-stream FP32 populations (the reference's sim.f) from args->pop_in
 * for every cell that is not on a deferred plane. */
int fc_lbm_materialize(const fc_lbm_step_args* args, void* stream);
/* Write rest populations w_q into args->pop_out (and macros 1,0,0,0) at solid cells. */
int fc_lbm_pin_solid(const fc_lbm_step_args* args, void* stream);

/* ---------------------------------------------------------------------------
 * Multigrid thermal operator (the MG_CUDA module surface plus fused V-cycle
 * kernels).  Fields are [nx][ny][nz] FP32; ax is the flow axis and out_idx the
 * outlet plane index on it (ghosting rule of solver/mg_kernels.cu:17-44).
 * ------------------------------------------------------------------------- */
/* replaces MG_CUDA.mop_fused  (solver/mg_kernels.cu:133-175): Lo = T + dt L(T) */
int fc_mg_mop(const float* T, const float* aE, const float* aW, const float* aN, const float* aS, const float* aU,
              const float* aD, const float* diagL, float* Lo, float dt, int nx, int ny, int nz, int ax, int out_idx,
              void* stream);
/* replaces MG_CUDA.jacobi_smooth  (solver/mg_kernels.cu:177-197): x += inv_diagM (b - Lo) */
int fc_mg_jacobi(float* x, const float* b, const float* Lo, const float* inv_diagM, long long n, void* stream);
/* replaces NLevelGeometricMGSolver.L_apply_fine  (solver/nlevel_mg_cuda.py:164-175): (M(T) - T) / dt */
int fc_mg_apply_L(const float* T, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, float* out, float dt, int nx, int ny, int nz,
                  int ax, int out_idx, void* stream);
/* replaces one mop_fused + jacobi_smooth pair of _vcycle (solver/nlevel_mg_cuda.py:285-287): x_out = x_in + invD (b - M x_in) */
int fc_mg_smooth(const float* x_in, float* x_out, const float* b, const float* inv_diagM, const float* aE,
                 const float* aW, const float* aN, const float* aS, const float* aU, const float* aD,
                 const float* diagL, float dt, int nx, int ny, int nz, int ax, int out_idx, void* stream);
/* the first sweep from a zero guess (nlevel_mg_cuda.py:297 zero + first smooth): x_out = invD b */
/* The first two damped-Jacobi sweeps from a zero guess in one pass (x1 = invD b
 * is formed on the fly for the cell and its neighbours): the pre-smoothing of
 * a V-cycle level entered with a zero guess (nlevel_mg_cuda.py:271-307,
 * n_pre = 2) in one launch instead of fc_mg_smooth_from_zero + fc_mg_smooth. */
int fc_mg_smooth_first2(float* x_out, const float* b, const float* inv_diagM, const float* aE, const float* aW,
                        const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                        float dt, int nx, int ny, int nz, int ax, int out_idx, void* stream);
/* All n_sweeps damped-Jacobi sweeps of a level of at most 6144 cells in one
 * single-CTA launch (the iterate stays in shared memory); the same arithmetic
 * as fc_mg_smooth_from_zero (from_zero) followed by fc_mg_smooth, so the
 * coarsest-level solve of the V-cycle (nlevel_mg_cuda.py:271-307, n_coarse
 * sweeps) is one launch instead of n_coarse.  Status 3 for a larger level. */
int fc_mg_smooth_small(float* x, const float* b, const float* inv_diagM, const float* aE, const float* aW,
                       const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                       float dt, int nx, int ny, int nz, int ax, int out_idx, int n_sweeps, int from_zero,
                       void* stream);
int fc_mg_smooth_from_zero(float* x_out, const float* b, const float* inv_diagM, long long n, void* stream);
/* replaces the residual + _restrict_into pair (nlevel_mg_cuda.py:289-295, :521-528); c* = n* / 2 */
int fc_mg_residual_restrict(const float* x, const float* b, const float* mask, const float* aE, const float* aW,
                            const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                            float dt, int nx, int ny, int nz, int ax, int out_idx, float* b_coarse, int cx, int cy,
                            int cz, void* stream);
/* replaces _prolong_2x + x.add_(e, alpha) + x.mul_(mask) (nlevel_mg_cuda.py:300-303, :531-537) */
int fc_mg_prolong_correct(float* x, const float* x_coarse, const float* mask, int nx, int ny, int nz, int cx,
                          int cy, int cz, float alpha, void* stream);
/* ||w (b - M x)||^2 in FP64 (w = mask, or 1 when mask is NULL), replaces the residual
 * norm of NLevelGeometricMGSolver.solve (nlevel_mg_cuda.py:132-135).  r_out (optional)
 * receives the FP32 residual.  result: one device double. */
long long fc_mg_reduce_workspace_bytes(long long n);
int fc_mg_residual_norm2(const float* x, const float* b, const float* mask, const float* aE, const float* aW,
                         const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                         float dt, int nx, int ny, int nz, int ax, int out_idx, float* r_out, void* workspace,
                         long long workspace_bytes, double* result, void* stream);
/* replaces NLevelGeometricMGSolver._build_coeffs_full  (solver/nlevel_mg_cuda.py:417-507) */
int fc_mg_build_coeffs(const float* k, const float* rho_cp, const float* u, const float* v, const float* w, int nx,
                       int ny, int nz, int ax, int out_idx, float dx, float s, float* aE, float* aW, float* aN,
                       float* aS, float* aU, float* aD, float* diagL, void* stream);
/* replaces _restrict_2x (solver/nlevel_mg_cuda.py:511-519); as_mask thresholds the mean at 0.999 (:255) */
int fc_mg_restrict_mean(const float* src, int nx, int ny, int nz, float* dst, int as_mask, void* stream);
/* FP64 exact solve of the coarsest multigrid level (no counterpart in the reference, which
 * gives the coarsest level n_coarse damped-Jacobi sweeps in FP32, solver/nlevel_mg_cuda.py:271-307).
 * build: A = I + dt L of the level (7-point couplings, operator ghosting, flux-form diagonal
 * 1 + dt sum_n a_n, identity rows where mask == 0; diagL is not read) assembled in FP64 and
 * inverted in place by Gauss-Jordan elimination (A is strictly diagonally dominant by rows: no
 * pivoting), into `inv` of fc_mg_coarse_dense_bytes() bytes (the n x n inverse followed by 4 n
 * work doubles); levels of at most 4096 cells (-1 / status 4 beyond).
 * apply: x = mask * inv (mask * b), accumulated in FP64, one warp per row. */
long long fc_mg_coarse_dense_bytes(int nx, int ny, int nz);
int fc_mg_coarse_dense_build(const float* aE, const float* aW, const float* aN, const float* aS, const float* aU,
                             const float* aD, const float* diagL, const float* mask, float dt, int nx, int ny, int nz,
                             int ax, int out_idx, double* inv, long long inv_bytes, void* stream);
int fc_mg_coarse_dense_apply(const double* inv, const float* b, const float* mask, float* x, int n, void* stream);
/* replaces _update_inv_diag  (solver/nlevel_mg_cuda.py:262-267) */
int fc_mg_inv_diag(const float* diagL, const float* mask, float* inv_diagM, float dt, float omega, long long n,
                   void* stream);

/* ---------------------------------------------------------------------------
 * Krylov vector kernels (replace the torch.dot / Tensor.norm / axpy calls of
 * solver/mg_pcg.py:25-187 with FP64-accumulated, deterministic versions)
 * ------------------------------------------------------------------------- */
long long fc_vec_workspace_bytes(long long n);
/* kind 0 (f64,f64), 1 (f32,f32), 2 (f64,f32); weight optional; result: device double */
int fc_vec_dot(int kind, const void* x, const void* y, long long n, const float* weight, void* workspace,
               long long workspace_bytes, double* result, void* stream);
/* y = alpha x + beta y, alpha = alpha_host * (*alpha_num / *alpha_den) when alpha_num is set; then * mask */
int fc_vec_axpby(int is_f64, void* y, const void* x, long long n, double alpha_host, const double* alpha_num,
                 const double* alpha_den, double beta, const float* mask, void* stream);
/* dst = scale * src (* mask); kind 0 f32->f64, 1 f64->f32, 2 f32->f32, 3 f64->f64 */
int fc_vec_convert(int kind, void* dst, const void* src, long long n, const float* mask, double scale, void* stream);
/* y = M(x) or y = b - M(x) in FP64 with the FP32 fine-level coefficients; optional mask */
/* Fused steps of BiCGSTAB (bicgstab_mg_f64 with FP64 vectors, the inner solve of
 * bicgstab_mg_mixed with FP32 vectors: is_f64) with the recurrence scalars in
 * device memory, so an iteration needs no host round trip (the reference's
 * bicgstab_mg, mg_pcg.py:103-175, reads every scalar on the host).
 * scalars[9] (FP64): 0 rho_new, 1 rho_old, 2 alpha, 3 omega, 4 (r_hat, v),
 * 5 (t, s), 6 (t, t), 7 (r, r), 8 beta.
 *   fc_bicgstab_p:  beta = (rho_new/rho_old)(alpha/omega); p = r + beta (p - omega v)
 *   fc_bicgstab_xr: stage 0: alpha = rho_new/(r_hat, v); r -= alpha w; x += alpha u
 *                   stage 1: omega = (t, s)/(t, t); rho_old = rho_new; x += omega u;
 *                            r -= omega w; scalars[7] = (r, r)
 *   fc_vec_dot2:    result2[0] = (x, y1), result2[1] = (x, y2) in one pass (FP64) */
long long fc_vec_dot2_workspace_bytes(long long n);
int fc_vec_dot2(int is_f64, const void* x, const void* y1, const void* y2, long long n, void* workspace,
                long long workspace_bytes, double* result2, void* stream);
int fc_bicgstab_p(int is_f64, void* p, const void* r, const void* v, long long n, double* scalars, void* stream);
int fc_bicgstab_xr(int is_f64, void* x, void* r, const void* u, const void* w, long long n, double* scalars,
                   int stage, void* workspace, long long workspace_bytes, void* stream);
int fc_mg_mop_f64(const double* x, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, double dt, int nx, int ny, int nz, int ax,
                  int out_idx, const double* b, const float* mask, double* y, void* stream);
/* fc_mg_mop_f64 on FP32 vectors (FP32 arithmetic): the operator of the inner
 * FP32 BiCGSTAB of bicgstab_mg_mixed. */
int fc_mg_mop_f32(const float* x, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, float dt, int nx, int ny, int nz, int ax,
                  int out_idx, const float* b, const float* mask, float* y, void* stream);
/* y = M^T (mask * x): the transpose of the operator of fc_mg_mop_f32 (same coefficients and
 * boundary ghosting), applied to the masked vector, FP32, accumulated with atomics (summation order
 * not fixed).  For the residual-norm loss of the learned correction, whose gradient is
 * -2 M^T (b - M y).  No reference counterpart. */
int fc_mg_mop_transpose_f32(const float* x, const float* aE, const float* aW, const float* aN, const float* aS,
                            const float* aU, const float* aD, float dt, int nx, int ny, int nz, int ax,
                            int out_idx, const float* mask, float* y, void* stream);

/* ---------------------------------------------------------------------------
 * Thermal pseudo-time step (the THERMAL_CUDA module surface)
 * ------------------------------------------------------------------------- */
/* replaces THERMAL_CUDA.thermal_rhs  (solver/thermal_kernels.cu:198-210) */
int fc_thermal_rhs(const float* T_old, const float* T0, const float* src_step, const float* LT0, const float* mask_f,
                   float* rhs, float* theta0, float dt, long long n, void* stream);
/* replaces THERMAL_CUDA.thermal_reconstruct  (solver/thermal_kernels.cu:212-224); caller owns T_new */
int fc_thermal_reconstruct(const float* T0, const float* theta, float* T_new, int nx, int ny, int nz, int ax,
                           int out_idx, void* stream);
long long fc_thermal_workspace_bytes(long long n);
/* replaces THERMAL_CUDA.convergence_metrics  (solver/thermal_kernels.cu:226-247); result: 2 device floats */
int fc_thermal_convergence_metrics(const float* T_new, const float* T_old, const uint8_t* solid, long long n,
                                   void* workspace, long long workspace_bytes, float* result, void* stream);
/* replaces THERMAL_CUDA.physics_check  (solver/thermal_kernels.cu:249-256); caller zeroes *flag */
int fc_thermal_physics_check(const float* T, int* flag, float T_min, float T_max, long long n, void* stream);
/* steady residual of _temperature_step_mg (LBM_CHT.py:2690-2699); result: 2 device floats (r_inf, src_inf) */
int fc_thermal_steady_residual(const float* T, const float* aE, const float* aW, const float* aN, const float* aS,
                               const float* aU, const float* aD, const float* diagL, const float* src_step,
                               const float* mask, float dt, int nx, int ny, int nz, int ax, int out_idx,
                               void* workspace, long long workspace_bytes, float* result, void* stream);

/* ---------------------------------------------------------------------------
 * BF16 implicit-GEMM 3-D convolutions on tcgen05 (learned preconditioner;
 * no counterpart in the reference).  Activations channels-last BF16
 * [B][D][H][W][C] (16-byte aligned), weights BF16 [C_out][kpad] with
 * K = 27 C_in tap-major (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)), kpad a multiple
 * of 64 >= 27 C_in, zero padding outside each volume.  dev_err bit2 = a
 * bounded mbarrier wait timed out.
 * ------------------------------------------------------------------------- */
/* Y = act(conv(X, W) + bias); C_in % 8 == 0, C_out % 16 == 0, 16 <= C_out <= 256 */
int fc_conv3d_fwd(const void* X, const void* Wt, const float* bias, int B, int D, int H, int W, int cin, int cout,
                  int kpad, int relu, float* Y_f32, void* Y_bf16, unsigned* dev_err, void* stream);
long long fc_conv3d_dgrad_workspace_bytes(int cin, int cout);
/* dX = conv^T(dY, W); C_in % 16 == 0 */
int fc_conv3d_dgrad(const void* dY, const void* Wt, int B, int D, int H, int W, int cin, int cout, int kpad,
                    void* workspace, long long workspace_bytes, float* dX_f32, void* dX_bf16, unsigned* dev_err,
                    void* stream);
long long fc_conv3d_wgrad_workspace_bytes(int B, int D, int H, int W, int cin, int cout, int splits);
/* dW[n][k] (FP32, k < 27 C_in written) = sum over voxels of X (x) dY, split-K over `splits` CTAs columns */
int fc_conv3d_wgrad(const void* X, const void* dY, int B, int D, int H, int W, int cin, int cout, int kpad,
                    int splits, void* workspace, long long workspace_bytes, float* dW, unsigned* dev_err,
                    void* stream);

/* ---------------------------------------------------------------------------
 * Learned-preconditioner network glue (no counterpart in the reference):
 * channels-last BF16 activations, FP32 gradients.
 * ------------------------------------------------------------------------- */
/* 8-channel BF16 input: c0 = r * inv_scale[b], c1 = (log k - k_shift) * k_scale, c2..7 = 0 */
int fc_nn_pack_input(const float* r, const float* k, const float* inv_scale, long long vox_per_b, long long nvox,
                     float k_shift, float k_scale, void* out, void* stream);
int fc_nn_avgpool2(const void* x, int B, int D, int H, int W, int C, void* y, void* stream);
int fc_nn_avgpool2_bwd(const float* gy, int B, int D, int H, int W, int C, float* gx, void* stream);
/* y[..., 0:Cx] = nearest-2x-upsampled x, y[..., Cx:Cx+Cs] = skip (D, H, W: fine extents) */
int fc_nn_upsample_concat(const void* x, int Cx, const void* skip, int Cs, int B, int D, int H, int W, void* y,
                          void* stream);
int fc_nn_upsample_concat_bwd(const float* gy, int Cx, int Cs, int B, int D, int H, int W, float* gx, float* gskip,
                              void* stream);
/* gout = (g + add) * [y > 0] (ReLU) or g + add, FP32 and/or BF16 */
int fc_nn_act_bwd(const float* g, const float* add, const void* y, int relu, long long n, float* gout,
                  void* gout_bf16, void* stream);
int fc_nn_take_channel0(const float* y, int C, const float* scale, long long vox_per_b, long long nvox,
                        const float* mask, float* out, void* stream);
long long fc_nn_mse_workspace_bytes(long long nvox);
int fc_nn_mse_grad(const float* y, int C, const float* target, const float* mask, long long nvox, float* grad,
                   void* workspace, long long workspace_bytes, void* stream);
int fc_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, int kpad, int kvalid,
               float lr, float beta1, float beta2, float eps, int step, float grad_scale, void* stream);

/* ---------------------------------------------------------------------------
 * Geometry set-up for interpolated bounce-back (device side).
 * solid: uint8 0/1 per cell, flat = i*ny*nz + j*nz + k.
 * ------------------------------------------------------------------------- */
/* Signed Euclidean distance of a voxel mask, positive in fluid, times pitch:
 * replaces build_phi_from_voxel_mask_mm (pre_post/sdf_tracing.py:312-340), which
 * runs scipy.ndimage.distance_transform_edt on the host.  phi equals
 * float32(scipy distance * pitch) bit for bit.  Workspace: one int32 per cell.
 * Limits: nx, ny, nz <= 4096 (status 3 beyond). */
long long fc_geom_edt_workspace_bytes(int nx, int ny, int nz);
int fc_geom_signed_edt(const uint8_t* solid, int nx, int ny, int nz, double pitch, float* phi, void* workspace,
                       long long workspace_bytes, void* stream);
/* Boundary links of build_links_from_mask_gpu (sdf_tracing.py:20-85), same order
 * (grouped by q = 1..18, row-major inside each q).  Two calls: count writes the
 * total to the DEVICE word *n_links (and per-block offsets to the workspace);
 * build fills the five arrays (n_links entries each) from the same workspace. */
long long fc_ibb_links_workspace_bytes(int nx, int ny, int nz);
int fc_ibb_count_links(const uint8_t* solid, int nx, int ny, int nz, void* workspace, long long workspace_bytes,
                       long long* n_links, void* stream);
int fc_ibb_build_links(const uint8_t* solid, int nx, int ny, int nz, const void* workspace, long long workspace_bytes,
                       long long n_links, long long* fluid_flat, long long* dir_i, long long* dir_opp,
                       long long* ff_flat, uint8_t* ff_valid, unsigned* err, void* stream);
/* Bouzidi fraction per link from the trilinear level set phi (bfl_q_from_sdf +
 * sdf_trilinear, sdf_tracing.py:89-184; 6 coarse samples, 10 bisections; the
 * fluid cell at origin + pitch*(i,j,k)) and the weights of bfl_weights_from_q
 * (:188-205).  true_div = 0: (x - origin)/dx as torch evaluates it on a CUDA
 * device (times the FP32 reciprocal); 1: as on the CPU (one division).
 * q may be NULL.  err: device word, DEV_ERR_INDEX on a bad link. */
int fc_ibb_q_from_sdf(const float* phi, int nx, int ny, int nz, float origin_x, float origin_y, float origin_z,
                      double dx, int true_div, const long long* fluid_flat, const long long* dir_i, long long n_links,
                      float* q, uint8_t* q_ge_half, float* w_i, float* w_second, unsigned* err, void* stream);
/* bfl_weights_from_q (sdf_tracing.py:188-205) alone, for fractions computed elsewhere */
int fc_ibb_weights_from_q(const float* q, long long n_links, uint8_t* q_ge_half, float* w_i, float* w_second,
                          void* stream);

/* ---------------------------------------------------------------------------
 * Snapshot and checkpoint I/O (device side)
 * ------------------------------------------------------------------------- */
/* One frame of _save_snapshot (LBM_CHT.py:2749-2769) in one pass: the fields
 * selected by `fields` (bit 0 u, 1 v, 2 w, 3 speed = sqrt(u*u + v*v + w*w) rounded
 * as torch rounds it, 4 rho, 5 T) written to out in that order, n floats each. */
int fc_snapshot_pack(const float* rho, const float* u, const float* v, const float* w, const float* T, long long n,
                     int fields, float* out, void* stream);
/* out[r*m + j] = src[r*ld + idx[j]] (no reference counterpart: the populations
 * of the inlet/outlet plane cells a checkpoint carries); scatter is the inverse.
 * err: device word, DEV_ERR_INDEX for an index outside [0, ld). */
int fc_columns_gather(const float* src, int rows, long long ld, const long long* idx, long long m, float* out,
                      unsigned* err, void* stream);
int fc_columns_scatter(float* dst, int rows, long long ld, const long long* idx, long long m, const float* cols,
                       unsigned* err, void* stream);

/* ---------------------------------------------------------------------------
 * STL voxelization and body stamping (device side)
 * ------------------------------------------------------------------------- */
/* gpu_voxelize_mesh (pre_post/gpu_voxelizer.py:81-170), in two calls.
 * prepare: tri = n_tri x 3 vertices x (x,y,z) FP32; prep = fc_vox_prepared_floats(n_tri)
 * floats (16-byte aligned); z0 = FP32 grid origin z.
 * parity: +z rays from (origin_x + i*pitch + perturb_x, origin_y + j*pitch + perturb_y)
 * (FP64, then FP32), cell centres origin_z + (k + 0.5)*pitch; voxels[(i*ny + j)*nz + k]
 * = 1 where an odd number of triangles is pierced below the centre.  nz <= 4096. */
long long fc_vox_prepared_floats(long long n_tri);
int fc_vox_prepare_triangles(const float* tri, long long n_tri, float z0, float* prep, void* stream);
int fc_vox_parity_z(const float* prep, long long n_tri, int nx, int ny, int nz, double origin_x, double origin_y,
                    double origin_z, double pitch, double perturb_x, double perturb_y, uint8_t* voxels,
                    void* stream);
/* LBMCHT3D_Torch.add_solid_body's stamp (LBM_CHT.py:959-1023): voxels (gx,gy,gz) placed
 * with voxel (0,0,0) at domain cell (i0,j0,k0), clamped to the domain; solid |= voxel,
 * k_field / rho_cp_field (may be NULL) set where the voxel is solid; body_mask (may be
 * NULL, caller-zeroed) = cells this body added (SolidAssembly.stamp's per-body mask,
 * pre_post/solid_assembly.py:164-184); *stamped (device, may be NULL) += solid voxels
 * placed. */
int fc_geom_stamp_body(const uint8_t* vox, int gx, int gy, int gz, int i0, int j0, int k0, int nx, int ny, int nz,
                       uint8_t* solid, float* k_field, float* rho_cp_field, float k_val, float rho_cp_val,
                       uint8_t* body_mask, unsigned long long* stamped, void* stream);

/* ---------------------------------------------------------------------------
 * Passive tracer (device side)
 * ------------------------------------------------------------------------- */
/* One TracerField.step (pre_post/tracer_patch.py:55-82): upwind advection of phi by
 * (u, v, w) with periodic neighbours, clamp to [0, 1], times dissipation, 0 where
 * solid_flow != 0; phi_out must not alias phi.  nx, ny <= 65535. */
int fc_tracer_step(const float* phi, float* phi_out, const float* u, const float* v, const float* w,
                   const uint8_t* solid_flow, int nx, int ny, int nz, float dissipation, void* stream);
/* TracerField.inject (:51-53): phi = 1 where mask != 0 */
int fc_tracer_inject(float* phi, const uint8_t* mask, long long n, void* stream);

/* ---------------------------------------------------------------------------
 * FP64 conservation integrals (no reference counterpart: the reference tracks
 * mass change and heat in FP32 torch reductions or not at all)
 * ------------------------------------------------------------------------- */
/* mass = sum over cells with flag bit CF_SOLID clear (flags may be NULL: all
 * cells) of sum_q f_q, populations [19][n] in storage `storage` (0 FP32, 1 FP16
 * shifted, 2 BF16 shifted), decoded and summed in FP64; *result is device memory. */
long long fc_lbm_mass_workspace_bytes(void);
int fc_lbm_mass(const void* pop, int storage, const uint8_t* flags, long long n_cells, void* workspace,
                long long workspace_bytes, double* result, void* stream);
/* Heat balance of the thermal operator over the cells with mask != 0, in FP64:
 * result3 = { sum src, sum L(T), sum T } with L the operator of the multigrid
 * level's coefficients (L(T) summed is the net heat leaving through the
 * boundaries, Dirichlet planes included); src may be NULL (0). */
long long fc_mg_heat_balance_workspace_bytes(long long n);
int fc_mg_heat_balance(const float* T, const float* src, const float* mask, const float* aE, const float* aW,
                       const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL, int nx,
                       int ny, int nz, int ax, int out_idx, void* workspace, long long workspace_bytes,
                       double* result3, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FLUXCORE3D_GB300_H */
