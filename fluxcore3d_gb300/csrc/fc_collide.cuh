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
#include "fc_vec.cuh"

namespace fc {

enum CollisionMode : int { CM_BGK = 0, CM_TRT = 1, CM_MRT = 2, CM_MRT_SMAG = 3 };

struct CollideParams {
    float omega;        // BGK rate
    float omega_plus;   // TRT even rate
    float omega_minus;  // TRT odd rate
    float S[19];        // MRT rates (channels 0,3,5,7 ignored: conserved)
    float Cs_dx2;       // (Cs*dx)^2 for Smagorinsky
    float omega0;       // base viscous rate for Smagorinsky
    float SN[19];       // S_k / |M_k|^2 (filled by the host for the shifted-variable collision)
};

// squared row norms of the D3Q19 moment matrix
__host__ __device__ constexpr float mrt_row_norm2(int k) {
    return k == 0 ? 19.f : k == 1 ? 2394.f : k == 2 ? 252.f : (k == 3 || k == 5 || k == 7) ? 10.f
         : (k == 4 || k == 6 || k == 8) ? 40.f : k == 9 ? 36.f : k == 10 ? 72.f : k == 11 ? 12.f
         : k == 12 ? 24.f : k <= 15 ? 4.f : 8.f;
}

// The per-cell operators below are templates on the arithmetic type R: float is
// the reference's FP32 kernel arithmetic, double the FP64 run of the plain
// method that the reduced-precision results are measured against.  Constants
// keep the reference's FP32 values (weights, S rates) in both.
template <class R>
struct MacroT {
    R rho, ux, uy, uz, inv_rho;
};
using Macro = MacroT<float>;

template <class R>
__device__ __forceinline__ MacroT<R> macros_of(const R f[19]) {
    MacroT<R> m;
    R rho = R(0);
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += f[q];
    // momentum sums in direction order (c components are +-1 or 0)
    R jx = R(0), jy = R(0), jz = R(0);
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
    m.inv_rho = R(1) / (rho + R(1e-12));
    m.ux = jx * m.inv_rho;
    m.uy = jy * m.inv_rho;
    m.uz = jz * m.inv_rho;
    return m;
}

// f_eq for all 19 directions: w_q rho (1 + cu + cu^2/2 - 3/2 u.u), cu = 3 c.u
template <class R>
__device__ __forceinline__ void equilibrium(R rho, R ux, R uy, R uz, R feq[19]) {
    const R usq = R(1.5) * (ux * ux + uy * uy + uz * uz);
    const R tx = R(3) * ux, ty = R(3) * uy, tz = R(3) * uz;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        R cu = R(0);
        if (cx(q) == 1) cu += tx;
        if (cx(q) == -1) cu -= tx;
        if (cy(q) == 1) cu += ty;
        if (cy(q) == -1) cu -= ty;
        if (cz(q) == 1) cu += tz;
        if (cz(q) == -1) cu -= tz;
        feq[q] = R(wq(q)) * rho * (R(1) + cu + R(0.5) * cu * cu - usq);
    }
}

// Relax the non-equilibrium part n = f - f_eq through the moment basis and
// return df = M^-1 S M n (conserved channels excluded).  g[k] = S_k m_k / |M_k|^2.
template <class R>
__device__ __forceinline__ void mrt_df(const R n[19], const R s[19], R df[19]) {
    const R Fx = n[1] + n[2], Fy = n[3] + n[4], Fz = n[5] + n[6];
    const R sf = Fx + Fy + Fz;
    const R Sxy = n[7] + n[8] + n[9] + n[10];
    const R Sxz = n[11] + n[12] + n[13] + n[14];
    const R Syz = n[15] + n[16] + n[17] + n[18];
    const R se = Sxy + Sxz + Syz;
    const R jxe = (n[7] + n[8] - n[9] - n[10]) + (n[11] + n[12] - n[13] - n[14]);
    const R jye = (n[7] - n[8] + n[9] - n[10]) + (n[15] + n[16] - n[17] - n[18]);
    const R jze = (n[11] - n[12] + n[13] - n[14]) + (n[15] - n[16] + n[17] - n[18]);

    const R m1 = R(-30) * n[0] - R(11) * sf + R(8) * se;
    const R m2 = R(12) * n[0] - R(4) * sf + se;
    const R m4 = R(-4) * (n[1] - n[2]) + jxe;
    const R m6 = R(-4) * (n[3] - n[4]) + jye;
    const R m8 = R(-4) * (n[5] - n[6]) + jze;
    const R m9 = R(2) * Fx - Fy - Fz + Sxy + Sxz - R(2) * Syz;
    const R m10 = R(-4) * Fx + R(2) * Fy + R(2) * Fz + Sxy + Sxz - R(2) * Syz;
    const R m11 = Fy - Fz + Sxy - Sxz;
    const R m12 = R(-2) * Fy + R(2) * Fz + Sxy - Sxz;
    const R m13 = n[7] - n[8] - n[9] + n[10];
    const R m14 = n[15] - n[16] - n[17] + n[18];
    const R m15 = n[11] - n[12] - n[13] + n[14];
    const R m16 = n[7] + n[8] - n[9] - n[10] - n[11] - n[12] + n[13] + n[14];
    const R m17 = -n[7] + n[8] - n[9] + n[10] + n[15] + n[16] - n[17] - n[18];
    const R m18 = n[11] - n[12] + n[13] - n[14] - n[15] + n[16] - n[17] + n[18];

    // divide by squared row norms of M (the reciprocals are rounded once, to R)
    const R g1 = s[1] * m1 * (R(1) / R(2394));
    const R g2 = s[2] * m2 * (R(1) / R(252));
    const R g4 = s[4] * m4 * (R(1) / R(40));
    const R g6 = s[6] * m6 * (R(1) / R(40));
    const R g8 = s[8] * m8 * (R(1) / R(40));
    const R g9 = s[9] * m9 * (R(1) / R(36));
    const R g10 = s[10] * m10 * (R(1) / R(72));
    const R g11 = s[11] * m11 * (R(1) / R(12));
    const R g12 = s[12] * m12 * (R(1) / R(24));
    const R g13 = s[13] * m13 * R(0.25);
    const R g14 = s[14] * m14 * R(0.25);
    const R g15 = s[15] * m15 * R(0.25);
    const R g16 = s[16] * m16 * R(0.125);
    const R g17 = s[17] * m17 * R(0.125);
    const R g18 = s[18] * m18 * R(0.125);

    df[0] = R(-30) * g1 + R(12) * g2;
    const R face = R(-11) * g1 - R(4) * g2;
    const R fx_ = face + R(2) * g9 - R(4) * g10;
    df[1] = fx_ - R(4) * g4;
    df[2] = fx_ + R(4) * g4;
    const R fyz = face - g9 + R(2) * g10;
    const R fy_ = fyz + g11 - R(2) * g12;
    const R fz_ = fyz - g11 + R(2) * g12;
    df[3] = fy_ - R(4) * g6;
    df[4] = fy_ + R(4) * g6;
    df[5] = fz_ - R(4) * g8;
    df[6] = fz_ + R(4) * g8;
    const R edge = R(8) * g1 + g2;
    const R exy = edge + g9 + g10 + g11 + g12;
    df[7] = exy + g4 + g6 + g13 + g16 - g17;
    df[8] = exy + g4 - g6 - g13 + g16 + g17;
    df[9] = exy - g4 + g6 - g13 - g16 - g17;
    df[10] = exy - g4 - g6 + g13 - g16 + g17;
    const R exz = edge + g9 + g10 - g11 - g12;
    df[11] = exz + g4 + g8 + g15 - g16 + g18;
    df[12] = exz + g4 - g8 - g15 - g16 - g18;
    df[13] = exz - g4 + g8 - g15 + g16 + g18;
    df[14] = exz - g4 - g8 + g15 + g16 - g18;
    const R eyz = edge - R(2) * g9 - R(2) * g10;
    df[15] = eyz + g6 + g8 + g14 + g17 - g18;
    df[16] = eyz + g6 - g8 - g14 + g17 + g18;
    df[17] = eyz - g6 + g8 - g14 - g17 - g18;
    df[18] = eyz - g6 - g8 + g14 - g17 + g18;
}

// Collide one fluid cell in place.  Returns the pre-collision macros and
// leaves feq (at those macros) for the sponge stage.
template <int MODE, class R>
__device__ __forceinline__ MacroT<R> collide(R f[19], R feq[19], const CollideParams& p) {
    const MacroT<R> m = macros_of(f);
    equilibrium(m.rho, m.ux, m.uy, m.uz, feq);
    if (MODE == CM_BGK) {
        const R om = R(p.omega);
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = f[q] + om * (feq[q] - f[q]);
    } else if (MODE == CM_TRT) {
        const R op = R(p.omega_plus), omn = R(p.omega_minus);
        R out[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int o = opp(q);
            const R fp = R(0.5) * (f[q] + f[o]);
            const R fm = R(0.5) * (f[q] - f[o]);
            const R ep = R(0.5) * (feq[q] + feq[o]);
            const R em = R(0.5) * (feq[q] - feq[o]);
            out[q] = (fp + op * (ep - fp)) + (fm + omn * (em - fm));
        }
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = out[q];
    } else {
        R n[19], df[19], s[19];
#pragma unroll
        for (int q = 0; q < 19; ++q) { n[q] = f[q] - feq[q]; s[q] = R(p.S[q]); }
        if (MODE == CM_MRT_SMAG) {
            R Pxx = R(0), Pyy = R(0), Pzz = R(0), Pxy = R(0), Pxz = R(0), Pyz = R(0);
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const R a = R(cx(q)), b = R(cy(q)), c = R(cz(q));
                Pxx += n[q] * a * a; Pyy += n[q] * b * b; Pzz += n[q] * c * c;
                Pxy += n[q] * a * b; Pxz += n[q] * a * c; Pyz += n[q] * b * c;
            }
            const R piF = sqrt(Pxx * Pxx + Pyy * Pyy + Pzz * Pzz + R(2) * (Pxy * Pxy + Pxz * Pxz + Pyz * Pyz));
            const R nu0 = (R(1) / R(p.omega0) - R(0.5)) / R(3);
            const R disc = nu0 * nu0 + R(4) * R(p.Cs_dx2) * (piF * m.inv_rho) * R(4.5);
            const R nu_eff = R(0.5) * (nu0 + sqrt(fmax(disc, nu0 * nu0)));
            const R om = fmin(R(1.99), R(1) / (R(3) * nu_eff + R(0.5)));
            s[9] = om; s[11] = om; s[13] = om; s[14] = om; s[15] = om;
        }
        mrt_df(n, s, df);
#pragma unroll
        for (int q = 0; q < 19; ++q) f[q] = f[q] - df[q];
    }
    return m;
}


// ---------------------------------------------------------------------------
// Collision in shifted variables h_q = f_q - w_q (the fused step's working set).
// With sum_q w_q = 1, sum_q w_q c_q = 0 and sum_q w_q c_q c_q = I/3:
//   rho = 1 + sum h,  j = sum c h,  M f = M h + (1, -11, 3, 0, ...),
// and the MRT equilibrium moments are the closed-form polynomials of rho, j
// for this equilibrium (m_eq = M f_eq evaluated symbolically), so neither f_eq
// nor M f_eq is formed for MRT.  Returns the macros of the input state.
// ---------------------------------------------------------------------------
template <class V>
struct MacroV {
    V drho, rho, inv_rho, jx, jy, jz, ux, uy, uz;
};

// Shared partial sums of the 19 shifted populations: every conserved and
// non-conserved moment below is one or two adds away from these.
template <class V>
struct PairSums {
    V Fx, Fy, Fz, dx1, dy1, dz1;        // face pairs: h1+h2, ... and h1-h2, ...
    V Sxy, Sxz, Syz;                    // edge-plane sums
    V jxe_xy, jxe_xz, jye_xy, jye_yz, jze_xz, jze_yz;
    V p13, p14, p15;                    // raw xy, yz, xz second moments
};

template <class V>
__device__ __forceinline__ PairSums<V> pair_sums(const V h[19]) {
    PairSums<V> p;
    p.Fx = h[1] + h[2]; p.Fy = h[3] + h[4]; p.Fz = h[5] + h[6];
    p.dx1 = h[1] - h[2]; p.dy1 = h[3] - h[4]; p.dz1 = h[5] - h[6];
    const V a78 = h[7] + h[8], a910 = h[9] + h[10], d78 = h[7] - h[8], d910 = h[9] - h[10];
    const V a1112 = h[11] + h[12], a1314 = h[13] + h[14], d1112 = h[11] - h[12], d1314 = h[13] - h[14];
    const V a1516 = h[15] + h[16], a1718 = h[17] + h[18], d1516 = h[15] - h[16], d1718 = h[17] - h[18];
    p.Sxy = a78 + a910; p.jxe_xy = a78 - a910; p.jye_xy = d78 + d910; p.p13 = d78 - d910;
    p.Sxz = a1112 + a1314; p.jxe_xz = a1112 - a1314; p.jze_xz = d1112 + d1314; p.p15 = d1112 - d1314;
    p.Syz = a1516 + a1718; p.jye_yz = a1516 - a1718; p.jze_yz = d1516 + d1718; p.p14 = d1516 - d1718;
    return p;
}

template <class V>
__device__ __forceinline__ MacroV<V> macros_from(const V h0, const PairSums<V>& p) {
    MacroV<V> m;
    m.drho = h0 + (((p.Fx + p.Fy) + p.Fz) + ((p.Sxy + p.Sxz) + p.Syz));
    m.rho = m.drho + 1.f;
    m.jx = p.dx1 + (p.jxe_xy + p.jxe_xz);
    m.jy = p.dy1 + (p.jye_xy + p.jye_yz);
    m.jz = p.dz1 + (p.jze_xz + p.jze_yz);
    m.inv_rho = rcp(m.rho + 1e-12f);
    m.ux = m.jx * m.inv_rho;
    m.uy = m.jy * m.inv_rho;
    m.uz = m.jz * m.inv_rho;
    return m;
}

template <class V>
__device__ __forceinline__ MacroV<V> macros_h(const V h[19]) { return macros_from(h[0], pair_sums(h)); }

// The nine opposite pairs (q, opp(q)) with q the member whose first non-zero
// velocity component is +1: 1|2 3|4 5|6 7|10 8|9 11|14 12|13 15|18 16|17.
__host__ __device__ constexpr int pair_first(int p) {
    return p == 0 ? 1 : p == 1 ? 3 : p == 2 ? 5 : p == 3 ? 7 : p == 4 ? 8 : p == 5 ? 11 : p == 6 ? 12 : p == 7 ? 15 : 16;
}

// c_q . t for the first member q of a pair (t = 3u)
template <int Q, class V>
__device__ __forceinline__ V cu_first(V tx, V ty, V tz) {
    if (Q == 1) return tx;
    if (Q == 3) return ty;
    if (Q == 5) return tz;
    if (Q == 7) return tx + ty;
    if (Q == 8) return tx - ty;
    if (Q == 11) return tx + tz;
    if (Q == 12) return tx - tz;
    if (Q == 15) return ty + tz;
    return ty - tz;   // Q == 16
}

template <int P, class V>
struct EqPair {
    static __device__ __forceinline__ void run(const MacroV<V>& m, V nusq, V tx, V ty, V tz, V heq[19]) {
        constexpr int q = pair_first(P), o = opp(q);
        const V cu = cu_first<q>(tx, ty, tz);
        const V e = fma(0.5f * cu, cu, nusq);
        heq[q] = wq(q) * fma(m.rho, e + cu, m.drho);
        heq[o] = wq(q) * fma(m.rho, e - cu, m.drho);
        EqPair<P + 1, V>::run(m, nusq, tx, ty, tz, heq);
    }
};
template <class V>
struct EqPair<9, V> {
    static __device__ __forceinline__ void run(const MacroV<V>&, V, V, V, V, V*) {}
};

// h_eq,q = f_eq,q - w_q = w_q (drho + rho (cu + cu^2/2 - 3/2 u.u)), evaluated per
// opposite pair from e = cu^2/2 - 3/2 u.u:  h_eq,q = w (drho + rho (e + cu)),
// h_eq,opp(q) = w (drho + rho (e - cu)).
template <class V>
__device__ __forceinline__ void equilibrium_h(const MacroV<V>& m, V heq[19]) {
    const V nusq = -1.5f * fma(m.ux, m.ux, fma(m.uy, m.uy, m.uz * m.uz));
    const V tx = 3.f * m.ux, ty = 3.f * m.uy, tz = 3.f * m.uz;
    heq[0] = wq(0) * fma(m.rho, nusq, m.drho);
    EqPair<0, V>::run(m, nusq, tx, ty, tz, heq);
}

// Subtract d_q = sum_k M[k][q] g_k (g_k = S_k n_k / |M_k|^2) from h, with the
// +-pattern of each edge quartet factored into two pairs of pairs.
template <class V>
__device__ __forceinline__ void apply_minv(V h[19], V g1, V g2, V g4, V g6, V g8, V g9, V g10, V g11, V g12,
                                           V g13, V g14, V g15, V g16, V g17, V g18) {
    h[0] = h[0] - fma(-30.f, g1, 12.f * g2);
    const V face = fma(-11.f, g1, -4.f * g2);
    const V fx_ = fma(2.f, g9, fma(-4.f, g10, face));
    h[1] = fma(4.f, g4, h[1] - fx_);
    h[2] = fma(-4.f, g4, h[2] - fx_);
    const V fyz = fma(2.f, g10, face - g9);
    const V fy_ = fma(-2.f, g12, fyz + g11);
    const V fz_ = fma(2.f, g12, fyz - g11);
    h[3] = fma(4.f, g6, h[3] - fy_);
    h[4] = fma(-4.f, g6, h[4] - fy_);
    h[5] = fma(4.f, g8, h[5] - fz_);
    h[6] = fma(-4.f, g8, h[6] - fz_);
    const V edge = fma(8.f, g1, g2);
    const V g910 = g9 + g10, g1112 = g11 + g12;
    {   // xy edges 7..10: exy +- (g4 + g16) +- ((g6 - g17) +- g13)
        const V exy = edge + (g910 + g1112);
        const V a = g4 + g16, b = g6 - g17;
        const V s1 = exy + a, s2 = exy - a, t1 = b + g13, t2 = b - g13;
        h[7] = h[7] - (s1 + t1); h[8] = h[8] - (s1 - t1); h[9] = h[9] - (s2 + t2); h[10] = h[10] - (s2 - t2);
    }
    {   // xz edges 11..14: exz +- (g4 - g16) +- ((g8 + g18) +- g15)
        const V exz = edge + (g910 - g1112);
        const V a = g4 - g16, b = g8 + g18;
        const V s1 = exz + a, s2 = exz - a, t1 = b + g15, t2 = b - g15;
        h[11] = h[11] - (s1 + t1); h[12] = h[12] - (s1 - t1); h[13] = h[13] - (s2 + t2); h[14] = h[14] - (s2 - t2);
    }
    {   // yz edges 15..18: eyz +- (g6 + g17) +- ((g8 - g18) +- g14)
        const V eyz = fma(-2.f, g910, edge);
        const V a = g6 + g17, b = g8 - g18;
        const V s1 = eyz + a, s2 = eyz - a, t1 = b + g14, t2 = b - g14;
        h[15] = h[15] - (s1 + t1); h[16] = h[16] - (s1 - t1); h[17] = h[17] - (s2 + t2); h[18] = h[18] - (s2 - t2);
    }
}

template <int MODE, class V>
__device__ __forceinline__ MacroV<V> collide_h(V h[19], const CollideParams& p) {
    const PairSums<V> ps = pair_sums(h);
    const MacroV<V> m = macros_from(h[0], ps);
    if (MODE == CM_BGK || MODE == CM_TRT) {
        V heq[19];
        equilibrium_h(m, heq);
        if (MODE == CM_BGK) {
#pragma unroll
            for (int q = 0; q < 19; ++q) h[q] = fma(p.omega, heq[q] - h[q], h[q]);
        } else {
            // even/odd split per opposite pair: h_q -= w+ (d_q + d_o)/2 + w- (d_q - d_o)/2
            const float ap = -0.5f * p.omega_plus, am = 0.5f * p.omega_minus;
            h[0] = fma(-p.omega_plus, h[0] - heq[0], h[0]);
#pragma unroll
            for (int pp = 0; pp < 9; ++pp) {
                const int q = pair_first(pp), o = opp(q);
                const V dq = h[q] - heq[q], dp = h[o] - heq[o];
                const V sp = dq + dp, sm = dq - dp;
                h[q] = fma(ap, sp, fma(-am, sm, h[q]));
                h[o] = fma(ap, sp, fma(am, sm, h[o]));
            }
        }
        return m;
    }
    const V sf = (ps.Fx + ps.Fy) + ps.Fz;
    const V se = (ps.Sxy + ps.Sxz) + ps.Syz;
    const V jxe = ps.jxe_xy + ps.jxe_xz, jye = ps.jye_xy + ps.jye_yz, jze = ps.jze_xz + ps.jze_yz;
    // equilibrium parts (rho u u = j u)
    const V uxx = m.jx * m.ux, uyy = m.jy * m.uy, uzz = m.jz * m.uz;
    const V ryz = uyy + uzz;
    const V rus = uxx + ryz;
    const V pxx = fma(2.f, uxx, -1.f * ryz);
    const V pww = uyy - uzz;
    const V sxyxz = ps.Sxy + ps.Sxz;
    const V dxyxz = ps.Sxy - ps.Sxz;
    // non-equilibrium moments n_k = (M h)_k - (m_eq,k - (M w)_k)
    const V n1 = fma(-30.f, h[0], fma(-11.f, sf, fma(8.f, se, fma(11.f, m.drho, -19.f * rus))));
    const V n2 = fma(12.f, h[0], fma(-4.f, sf, fma(-3.f, m.drho, fma(5.5f, rus, se))));
    const V n4 = fma(-4.f, ps.dx1, fma(2.f / 3.f, m.jx, jxe));
    const V n6 = fma(-4.f, ps.dy1, fma(2.f / 3.f, m.jy, jye));
    const V n8 = fma(-4.f, ps.dz1, fma(2.f / 3.f, m.jz, jze));
    const V fyz2 = ps.Fy + ps.Fz;
    const V e9 = fma(-2.f, ps.Syz, sxyxz);
    const V n9 = fma(2.f, ps.Fx, e9 - fyz2) - pxx;
    const V n10 = fma(-4.f, ps.Fx, fma(2.f, fyz2, fma(0.5f, pxx, e9)));
    const V fymz = ps.Fy - ps.Fz;
    const V n11 = (fymz + dxyxz) - pww;
    const V n12 = fma(-2.f, fymz, fma(0.5f, pww, dxyxz));
    const V n13 = fma(-1.f * m.jx, m.uy, ps.p13);
    const V n14 = fma(-1.f * m.jy, m.uz, ps.p14);
    const V n15 = fma(-1.f * m.jx, m.uz, ps.p15);
    const V n16 = ps.jxe_xy - ps.jxe_xz;
    const V n17 = ps.jye_yz - ps.jye_xy;
    const V n18 = ps.jze_xz - ps.jze_yz;
    V s9 = splat<V>(p.SN[9]), s11 = splat<V>(p.SN[11]), s13 = splat<V>(p.SN[13]);
    V s14 = splat<V>(p.SN[14]), s15 = splat<V>(p.SN[15]);
    if (MODE == CM_MRT_SMAG) {
        // Pi_neq = Pi(h) - rho u u - (drho / 3) I
        const V third = (1.f / 3.f) * m.drho;
        const V Pxx = ((ps.Fx + sxyxz) - uxx) - third;
        const V Pyy = ((ps.Fy + (ps.Sxy + ps.Syz)) - uyy) - third;
        const V Pzz = ((ps.Fz + (ps.Sxz + ps.Syz)) - uzz) - third;
        const V off = fma(n13, n13, fma(n15, n15, n14 * n14));
        const V piF = vsqrt(fma(Pxx, Pxx, fma(Pyy, Pyy, fma(Pzz, Pzz, 2.f * off))));
        const float nu0 = (1.f / p.omega0 - 0.5f) * (1.f / 3.f);
        const V disc = fma(18.f * p.Cs_dx2, piF * m.inv_rho, splat<V>(nu0 * nu0));
        const V nu_eff = 0.5f * (vsqrt(vmax(disc, splat<V>(nu0 * nu0))) + nu0);
        const V om = vmin(rcp(fma(3.f, nu_eff, splat<V>(0.5f))), 1.99f);
        s9 = (1.f / 36.f) * om; s11 = (1.f / 12.f) * om;
        s13 = 0.25f * om; s14 = s13; s15 = s13;
    }
    apply_minv(h, p.SN[1] * n1, p.SN[2] * n2, p.SN[4] * n4, p.SN[6] * n6, p.SN[8] * n8, s9 * n9,
               p.SN[10] * n10, s11 * n11, p.SN[12] * n12, s13 * n13, s14 * n14, s15 * n15,
               p.SN[16] * n16, p.SN[17] * n17, p.SN[18] * n18);
    return m;
}
}  // namespace fc
