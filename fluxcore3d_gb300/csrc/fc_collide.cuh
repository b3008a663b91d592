// fc_collide.cuh -- D3Q19 single-cell collision operators in FP32 registers.
//
// Semantics follow the reference kernels (solver/lbm_kernels.cu):
//   macroscopic sums          lbm_kernels.cu:286-299 (q-order sums, inv_rho = 1/(rho+1e-12))
//   equilibrium               lbm_kernels.cu:77-113
//   BGK                       lbm_kernels.cu:305-307
//   TRT (even/odd parts)      lbm_kernels.cu:355-364
//   MRT  f* = f - M^-1 S (m - m_eq)            lbm_kernels.cu:413-435
//   MRT + Smagorinsky omega on channels 9,11,13,14,15   lbm_kernels.cu:1058-1116
// The moment transform is written here as M (f - f_eq) followed by the inverse
// of M built from its row-orthogonality (M^-1 = M^T diag(1/|M_k|^2)); this is
// the same linear map as the reference's literal M^-1 table, evaluated with
// integer row coefficients.
#pragma once
#include "fc_common.cuh"

namespace fc {

enum CollisionMode : int { CM_BGK = 0, CM_TRT = 1, CM_MRT = 2, CM_MRT_SMAG = 3 };

struct CollideParams {
    float omega;        // BGK rate
    float omega_plus;   // TRT even rate
    float omega_minus;  // TRT odd rate
    float S[19];        // MRT rates (channels 0,3,5,7 ignored: conserved)
    float Cs_dx2;       // (Cs*dx)^2 for Smagorinsky
    float omega0;       // base viscous rate for Smagorinsky
};

struct Macro {
    float rho, ux, uy, uz, inv_rho;
};

__device__ __forceinline__ Macro macros_of(const float f[19]) {
    Macro m;
    float rho = 0.f;
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += f[q];
    // momentum sums in direction order (c components are +-1 or 0)
    float jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        if (cx(q) == 1) jx += f[q];
        if (cx(q) == -1) jx -= f[q];
        if (cy(q) == 1) jy += f[q];
        if (cy(q) == -1) jy -= f[q];
        if (cz(q) == 1) jz += f[q];
        if (cz(q) == -1) jz -= f[q];
    }
    m.rho = rho;
    m.inv_rho = 1.f / (rho + 1e-12f);
    m.ux = jx * m.inv_rho;
    m.uy = jy * m.inv_rho;
    m.uz = jz * m.inv_rho;
    return m;
}

// f_eq for all 19 directions: w_q rho (1 + cu + cu^2/2 - 3/2 u.u), cu = 3 c.u
__device__ __forceinline__ void equilibrium(float rho, float ux, float uy, float uz, float feq[19]) {
    const float usq = 1.5f * (ux * ux + uy * uy + uz * uz);
    const float tx = 3.f * ux, ty = 3.f * uy, tz = 3.f * uz;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        float cu = 0.f;
        if (cx(q) == 1) cu += tx;
        if (cx(q) == -1) cu -= tx;
        if (cy(q) == 1) cu += ty;
        if (cy(q) == -1) cu -= ty;
        if (cz(q) == 1) cu += tz;
        if (cz(q) == -1) cu -= tz;
        feq[q] = wq(q) * rho * (1.f + cu + 0.5f * cu * cu - usq);
    }
}

// Relax the non-equilibrium part n = f - f_eq through the moment basis and
// return df = M^-1 S M n (conserved channels excluded).  g[k] = S_k m_k / |M_k|^2.
__device__ __forceinline__ void mrt_df(const float n[19], const float s[19], float df[19]) {
    const float Fx = n[1] + n[2], Fy = n[3] + n[4], Fz = n[5] + n[6];
    const float sf = Fx + Fy + Fz;
    const float Sxy = n[7] + n[8] + n[9] + n[10];
    const float Sxz = n[11] + n[12] + n[13] + n[14];
    const float Syz = n[15] + n[16] + n[17] + n[18];
    const float se = Sxy + Sxz + Syz;
    const float jxe = (n[7] + n[8] - n[9] - n[10]) + (n[11] + n[12] - n[13] - n[14]);
    const float jye = (n[7] - n[8] + n[9] - n[10]) + (n[15] + n[16] - n[17] - n[18]);
    const float jze = (n[11] - n[12] + n[13] - n[14]) + (n[15] - n[16] + n[17] - n[18]);

    const float m1 = -30.f * n[0] - 11.f * sf + 8.f * se;
    const float m2 = 12.f * n[0] - 4.f * sf + se;
    const float m4 = -4.f * (n[1] - n[2]) + jxe;
    const float m6 = -4.f * (n[3] - n[4]) + jye;
    const float m8 = -4.f * (n[5] - n[6]) + jze;
    const float m9 = 2.f * Fx - Fy - Fz + Sxy + Sxz - 2.f * Syz;
    const float m10 = -4.f * Fx + 2.f * Fy + 2.f * Fz + Sxy + Sxz - 2.f * Syz;
    const float m11 = Fy - Fz + Sxy - Sxz;
    const float m12 = -2.f * Fy + 2.f * Fz + Sxy - Sxz;
    const float m13 = n[7] - n[8] - n[9] + n[10];
    const float m14 = n[15] - n[16] - n[17] + n[18];
    const float m15 = n[11] - n[12] - n[13] + n[14];
    const float m16 = n[7] + n[8] - n[9] - n[10] - n[11] - n[12] + n[13] + n[14];
    const float m17 = -n[7] + n[8] - n[9] + n[10] + n[15] + n[16] - n[17] - n[18];
    const float m18 = n[11] - n[12] + n[13] - n[14] - n[15] + n[16] - n[17] + n[18];

    // divide by squared row norms of M
    const float g1 = s[1] * m1 * (1.f / 2394.f);
    const float g2 = s[2] * m2 * (1.f / 252.f);
    const float g4 = s[4] * m4 * (1.f / 40.f);
    const float g6 = s[6] * m6 * (1.f / 40.f);
    const float g8 = s[8] * m8 * (1.f / 40.f);
    const float g9 = s[9] * m9 * (1.f / 36.f);
    const float g10 = s[10] * m10 * (1.f / 72.f);
    const float g11 = s[11] * m11 * (1.f / 12.f);
    const float g12 = s[12] * m12 * (1.f / 24.f);
    const float g13 = s[13] * m13 * 0.25f;
    const float g14 = s[14] * m14 * 0.25f;
    const float g15 = s[15] * m15 * 0.25f;
    const float g16 = s[16] * m16 * 0.125f;
    const float g17 = s[17] * m17 * 0.125f;
    const float g18 = s[18] * m18 * 0.125f;

    df[0] = -30.f * g1 + 12.f * g2;
    const float face = -11.f * g1 - 4.f * g2;
    const float fx_ = face + 2.f * g9 - 4.f * g10;
    df[1] = fx_ - 4.f * g4;
    df[2] = fx_ + 4.f * g4;
    const float fyz = face - g9 + 2.f * g10;
    const float fy_ = fyz + g11 - 2.f * g12;
    const float fz_ = fyz - g11 + 2.f * g12;
    df[3] = fy_ - 4.f * g6;
    df[4] = fy_ + 4.f * g6;
    df[5] = fz_ - 4.f * g8;
    df[6] = fz_ + 4.f * g8;
    const float edge = 8.f * g1 + g2;
    const float exy = edge + g9 + g10 + g11 + g12;
    df[7] = exy + g4 + g6 + g13 + g16 - g17;
    df[8] = exy + g4 - g6 - g13 + g16 + g17;
    df[9] = exy - g4 + g6 - g13 - g16 - g17;
    df[10] = exy - g4 - g6 + g13 - g16 + g17;
    const float exz = edge + g9 + g10 - g11 - g12;
    df[11] = exz + g4 + g8 + g15 - g16 + g18;
    df[12] = exz + g4 - g8 - g15 - g16 - g18;
    df[13] = exz - g4 + g8 - g15 + g16 + g18;
    df[14] = exz - g4 - g8 + g15 + g16 - g18;
    const float eyz = edge - 2.f * g9 - 2.f * g10;
    df[15] = eyz + g6 + g8 + g14 + g17 - g18;
    df[16] = eyz + g6 - g8 - g14 + g17 + g18;
    df[17] = eyz - g6 + g8 - g14 - g17 - g18;
    df[18] = eyz - g6 - g8 + g14 - g17 + g18;
}

// Collide one fluid cell in place.  Returns the pre-collision macros and
// leaves feq (at those macros) for the sponge stage.
template <int MODE>
__device__ __forceinline__ Macro collide(float f[19], float feq[19], const CollideParams& p) {
    const Macro m = macros_of(f);
    equilibrium(m.rho, m.ux, m.uy, m.uz, feq);
    if (MODE == CM_BGK) {
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = f[q] + p.omega * (feq[q] - f[q]);
    } else if (MODE == CM_TRT) {
        float out[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int o = opp(q);
            const float fp = 0.5f * (f[q] + f[o]);
            const float fm = 0.5f * (f[q] - f[o]);
            const float ep = 0.5f * (feq[q] + feq[o]);
            const float em = 0.5f * (feq[q] - feq[o]);
            out[q] = (fp + p.omega_plus * (ep - fp)) + (fm + p.omega_minus * (em - fm));
        }
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = out[q];
    } else {
        float n[19], df[19], s[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) { n[q] = f[q] - feq[q]; s[q] = p.S[q]; }
        if (MODE == CM_MRT_SMAG) {
            float Pxx = 0.f, Pyy = 0.f, Pzz = 0.f, Pxy = 0.f, Pxz = 0.f, Pyz = 0.f;
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const float a = (float)cx(q), b = (float)cy(q), c = (float)cz(q);
                Pxx += n[q] * a * a; Pyy += n[q] * b * b; Pzz += n[q] * c * c;
                Pxy += n[q] * a * b; Pxz += n[q] * a * c; Pyz += n[q] * b * c;
            }
            const float piF = sqrtf(Pxx * Pxx + Pyy * Pyy + Pzz * Pzz +
                                    2.f * (Pxy * Pxy + Pxz * Pxz + Pyz * Pyz));
            const float nu0 = (1.f / p.omega0 - 0.5f) / 3.f;
            const float disc = nu0 * nu0 + 4.f * p.Cs_dx2 * (piF * m.inv_rho) * 4.5f;
            const float nu_eff = 0.5f * (nu0 + sqrtf(fmaxf(disc, nu0 * nu0)));
            const float om = fminf(1.99f, 1.f / (3.f * nu_eff + 0.5f));
            s[9] = om; s[11] = om; s[13] = om; s[14] = om; s[15] = om;
        }
        mrt_df(n, s, df);
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = f[q] - df[q];
    }
    return m;
}

}  // namespace fc
