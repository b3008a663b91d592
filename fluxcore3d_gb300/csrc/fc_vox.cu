// fc_vox.cu -- STL voxelization and body stamping on the device.
//
//  * fc_vox_prepare_triangles + fc_vox_parity_z: gpu_voxelize_mesh
//    (pre_post/gpu_voxelizer.py:81-170).  One ray per (i, j) column along +z,
//    Moller-Trumbore against every triangle, and a cell is solid when an odd
//    number of surfaces is pierced below its centre.  The ray origins, the cell
//    centres and every operation of the intersection test are rounded as the
//    reference's tensor expressions are (FP64 numpy for the origins and centres,
//    then FP32; FP32 elementwise for the test, no contraction), so the voxel grid
//    is the reference's bit for bit.  The per-triangle terms that do not depend
//    on the ray (edges, determinant, its reciprocal, the z offsets) are computed
//    once by the prepare kernel.  A block stages 512 prepared triangles at a
//    time in shared memory; each thread walks them for its ray and, for every
//    hit, toggles a bit at the first cell centre above the hit (binary search in
//    the centre table); a prefix XOR over the bits gives the parity column, and
//    the block writes its columns (one contiguous byte range) with 16-byte stores.
//    Every triangle is tested against every ray, as in the reference: a bounding
//    box cull would be exact only with an error bound that sliver triangles
//    (tiny determinant, huge reciprocal) do not have.
//  * fc_geom_stamp_body: LBMCHT3D_Torch.add_solid_body's stamp
//    (LBM_CHT.py:959-1023): solid |= voxels in the clamped box, k and rho_cp set
//    where the voxels are solid, and the per-body mask of SolidAssembly.stamp
//    (pre_post/solid_assembly.py:164-184: cells this body added).
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int VOX_RAYS = 128;       // rays (threads) per block
constexpr int VOX_CHUNK = 512;      // prepared triangles staged per round
constexpr int VOX_MAX_NZ = 4096;
constexpr int PREP_FLOATS = 16;     // per prepared triangle (float4 x 4)

// prepared triangle: v0x v0y e1x e1y | e1z e2x e2y e2z | hx hy inv_det szt_e1y | szt_e1x valid - -
__global__ void __launch_bounds__(256) k_vox_prepare(const float* __restrict__ tri, long long T, float z0,
                                                     float4* __restrict__ prep) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float* p = tri + t * 9;
    const float v0x = p[0], v0y = p[1], v0z = p[2];
    const float e1x = __fsub_rn(p[3], v0x), e1y = __fsub_rn(p[4], v0y), e1z = __fsub_rn(p[5], v0z);
    const float e2x = __fsub_rn(p[6], v0x), e2y = __fsub_rn(p[7], v0y), e2z = __fsub_rn(p[8], v0z);
    const float hx = -e2y, hy = e2x;                      // h = (0,0,1) x e2
    const float det = __fadd_rn(__fmul_rn(e1x, hx), __fmul_rn(e1y, hy));
    const bool valid = fabsf(det) > 1e-7f;
    const float inv = valid ? __fdiv_rn(1.0f, det) : 0.0f;
    const float szt = __fsub_rn(z0, v0z);
    float4* o = prep + t * 4;
    o[0] = make_float4(v0x, v0y, e1x, e1y);
    o[1] = make_float4(e1z, e2x, e2y, e2z);
    o[2] = make_float4(hx, hy, inv, __fmul_rn(szt, e1y));
    o[3] = make_float4(__fmul_rn(szt, e1x), valid ? 1.0f : 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(VOX_RAYS)
k_vox_parity(const float4* __restrict__ prep, long long T, int nx, int ny, int nz, double ox0, double oy0,
             double pitch, double pert_x, double pert_y, double z0d, float z0, uint8_t* __restrict__ out) {
    extern __shared__ float4 vox_sh[];
    float4* tri = vox_sh;                                           // VOX_CHUNK x 4
    float* zc = (float*)(vox_sh + VOX_CHUNK * 4);                   // nz cell centres
    const int nw = (nz + 31) / 32;
    unsigned* bits = (unsigned*)(zc + ((nz + 3) & ~3));             // [word][ray]
    const long long nrays = (long long)nx * ny;
    const long long r = (long long)blockIdx.x * VOX_RAYS + threadIdx.x;
    const bool active = r < nrays;
    const int ix = active ? (int)(r / ny) : 0, iy = active ? (int)(r - (long long)ix * ny) : 0;
    // origins: float32(origin + i*pitch + perturbation) from FP64, as numpy forms them
    const float ox = __double2float_rn(__dadd_rn(__dadd_rn(ox0, __dmul_rn((double)ix, pitch)), pert_x));
    const float oy = __double2float_rn(__dadd_rn(__dadd_rn(oy0, __dmul_rn((double)iy, pitch)), pert_y));
    for (int k = threadIdx.x; k < nz; k += VOX_RAYS)
        zc[k] = __double2float_rn(__dadd_rn(z0d, __dmul_rn((double)k + 0.5, pitch)));
    for (int w = 0; w < nw; ++w) bits[w * VOX_RAYS + threadIdx.x] = 0u;
    for (long long base = 0; base < T; base += VOX_CHUNK) {
        const int cnt = (int)min((long long)VOX_CHUNK, T - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt * 4; e += VOX_RAYS) tri[e] = prep[base * 4 + e];
        __syncthreads();
        if (!active) continue;
        for (int j = 0; j < cnt; ++j) {
            const float4 a = tri[4 * j], b = tri[4 * j + 1], c = tri[4 * j + 2], d = tri[4 * j + 3];
            // a: v0x v0y e1x e1y  b: e1z e2x e2y e2z  c: hx hy inv szt*e1y  d: szt*e1x valid
            const float sx = __fsub_rn(ox, a.x), sy = __fsub_rn(oy, a.y);
            const float u = __fmul_rn(__fadd_rn(__fmul_rn(sx, c.x), __fmul_rn(sy, c.y)), c.z);
            if (!(u >= 0.0f && u <= 1.0f) || d.y == 0.0f) continue;
            const float qz = __fsub_rn(__fmul_rn(sx, a.w), __fmul_rn(sy, a.z));
            const float v = __fmul_rn(qz, c.z);
            if (!(v >= 0.0f && __fadd_rn(u, v) <= 1.0f)) continue;
            const float qx = __fsub_rn(__fmul_rn(sy, b.x), c.w);
            const float qy = __fsub_rn(d.x, __fmul_rn(sx, b.x));
            const float t = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(b.y, qx), __fmul_rn(b.z, qy)), __fmul_rn(b.w, qz)),
                                      c.z);
            if (!(t >= 0.0f)) continue;
            const float hz = __fadd_rn(z0, t);
            // first centre strictly above the hit
            int lo = 0, hi = nz;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (hz < zc[mid]) hi = mid;
                else lo = mid + 1;
            }
            if (lo < nz) bits[(lo >> 5) * VOX_RAYS + threadIdx.x] ^= 1u << (lo & 31);
        }
    }
    // flip bits -> parity bits (prefix XOR along the column), in place
    if (active) {
        unsigned carry = 0u;
        for (int w = 0; w < nw; ++w) {
            unsigned p = bits[w * VOX_RAYS + threadIdx.x];
            p ^= p << 1;
            p ^= p << 2;
            p ^= p << 4;
            p ^= p << 8;
            p ^= p << 16;
            if (carry) p = ~p;
            carry = p >> 31;
            bits[w * VOX_RAYS + threadIdx.x] = p;
        }
    }
    __syncthreads();
    // the block's columns are one contiguous byte range: write it with 16-byte stores
    const long long r0 = (long long)blockIdx.x * VOX_RAYS;
    const long long nr = min((long long)VOX_RAYS, nrays - r0);
    const long long nbytes = nr * nz;
    uint8_t* dst = out + r0 * nz;       // r0 * nz is a multiple of 128
    const long long nchunk = nbytes >> 4;
    for (long long c = threadIdx.x; c < nchunk; c += VOX_RAYS) {
        const long long b0 = c << 4;
        int ray = (int)(b0 / nz), k = (int)(b0 - (long long)ray * nz);
        unsigned wd[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const unsigned bit = (bits[(k >> 5) * VOX_RAYS + ray] >> (k & 31)) & 1u;
            wd[i >> 2] |= bit << ((i & 3) * 8);
            if (++k == nz) {
                k = 0;
                ++ray;
            }
        }
        *reinterpret_cast<uint4*>(dst + b0) = make_uint4(wd[0], wd[1], wd[2], wd[3]);
    }
    for (long long b = (nchunk << 4) + threadIdx.x; b < nbytes; b += VOX_RAYS) {
        const int ray = (int)(b / nz), k = (int)(b - (long long)ray * nz);
        dst[b] = (uint8_t)((bits[(k >> 5) * VOX_RAYS + ray] >> (k & 31)) & 1u);
    }
}

__global__ void __launch_bounds__(256)
k_stamp(const uint8_t* __restrict__ vox, int gx, int gy, int gz, int i0, int j0, int k0, int di0, int dj0, int dk0,
        int bx, int by, int bz, int ny, int nz, uint8_t* __restrict__ solid, float* __restrict__ kf,
        float* __restrict__ rcp, float k_val, float rho_cp_val, uint8_t* __restrict__ body,
        unsigned long long* __restrict__ count) {
    const long long n = (long long)bx * by * bz;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mine = 0;
    if (t < n) {
        const int a = (int)(t / ((long long)by * bz));
        const int rem = (int)(t - (long long)a * by * bz);
        const int b = rem / bz, c = rem - b * bz;
        const int i = di0 + a, j = dj0 + b, k = dk0 + c;
        const long long s = ((long long)(i - i0) * gy + (j - j0)) * gz + (k - k0);
        if (vox[s]) {
            const long long cell = ((long long)i * ny + j) * nz + k;
            if (body && !solid[cell]) body[cell] = 1;
            solid[cell] = 1;
            if (kf) kf[cell] = k_val;
            if (rcp) rcp[cell] = rho_cp_val;
            mine = 1;
        }
    }
    if (count) {
        const unsigned long long w = __reduce_add_sync(0xffffffffu, (unsigned)mine);
        if ((threadIdx.x & 31) == 0 && w) atomicAdd(count, w);
    }
}

}  // namespace

extern "C" {

int fc_vox_prepare_triangles(const float* tri, long long n_tri, float z0, float* prep, void* stream) {
    if (n_tri < 0 || (n_tri > 0 && (!tri || !prep))) return FC_ERR_ARG;
    if (n_tri == 0) return FC_OK;
    k_vox_prepare<<<(unsigned)((n_tri + 255) / 256), 256, 0, (cudaStream_t)stream>>>(tri, n_tri, z0, (float4*)prep);
    return launch_status();
}

long long fc_vox_prepared_floats(long long n_tri) { return n_tri < 0 ? -1 : n_tri * PREP_FLOATS; }

int fc_vox_parity_z(const float* prep, long long n_tri, int nx, int ny, int nz, double origin_x, double origin_y,
                    double origin_z, double pitch, double perturb_x, double perturb_y, uint8_t* voxels,
                    void* stream) {
    if (!voxels || n_tri < 0 || (n_tri > 0 && !prep) || nx < 1 || ny < 1 || nz < 1 || !(pitch > 0.0))
        return FC_ERR_ARG;
    if (nz > VOX_MAX_NZ) return FC_ERR_UNSUPPORTED;
    const long long nrays = (long long)nx * ny;
    const long long blocks = (nrays + VOX_RAYS - 1) / VOX_RAYS;
    if (blocks > 0x7fffffffLL) return FC_ERR_UNSUPPORTED;
    const int nw = (nz + 31) / 32;
    const size_t smem = (size_t)VOX_CHUNK * 4 * sizeof(float4) + (size_t)((nz + 3) & ~3) * sizeof(float) +
                        (size_t)nw * VOX_RAYS * sizeof(unsigned);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_vox_parity, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const float z0 = (float)origin_z;
    k_vox_parity<<<(unsigned)blocks, VOX_RAYS, smem, (cudaStream_t)stream>>>(
        (const float4*)prep, n_tri, nx, ny, nz, origin_x, origin_y, pitch, perturb_x, perturb_y, (double)z0, z0,
        voxels);
    return launch_status();
}

int fc_geom_stamp_body(const uint8_t* vox, int gx, int gy, int gz, int i0, int j0, int k0, int nx, int ny, int nz,
                       uint8_t* solid, float* k_field, float* rho_cp_field, float k_val, float rho_cp_val,
                       uint8_t* body_mask, unsigned long long* stamped, void* stream) {
    if (!vox || !solid || gx < 1 || gy < 1 || gz < 1 || nx < 1 || ny < 1 || nz < 1) return FC_ERR_ARG;
    const int di0 = i0 > 0 ? i0 : 0, di1 = (i0 + gx) < nx ? (i0 + gx) : nx;
    const int dj0 = j0 > 0 ? j0 : 0, dj1 = (j0 + gy) < ny ? (j0 + gy) : ny;
    const int dk0 = k0 > 0 ? k0 : 0, dk1 = (k0 + gz) < nz ? (k0 + gz) : nz;
    if (di1 <= di0 || dj1 <= dj0 || dk1 <= dk0) return FC_OK;     // entirely outside the domain
    const int bx = di1 - di0, by = dj1 - dj0, bz = dk1 - dk0;
    const long long n = (long long)bx * by * bz;
    k_stamp<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        vox, gx, gy, gz, i0, j0, k0, di0, dj0, dk0, bx, by, bz, ny, nz, solid, k_field, rho_cp_field, k_val,
        rho_cp_val, body_mask, stamped);
    return launch_status();
}

}  // extern "C"
