/*
 * lbm_oracle.c -- TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the
 * reference's CUDA-path lattice kernels (fluxcore3D solver/lbm_kernels.cu),
 * used by the tests as the parity oracle and by bench.py as the timed CPU
 * baseline.  The product library never links or calls this code.
 *
 * Compiled twice by oracle/build_oracle.py: REAL=float (FP32 parity oracle)
 * and REAL=double (FP64 plain-method oracle), with -ffp-contract=off so the
 * arithmetic is the same on x86-64 and aarch64, and -fopenmp for the cell
 * loops.  Parity status: pinned against fixtures generated from the reference's
 * own Python/torch implementation (tests/golden/make_golden.py) for collide,
 * stream, interpolated bounce-back + reset and the MRT matrix; the Zou/He and
 * convective plane kernels follow lbm_kernels.cu:791-969 / 1170-1344, for which
 * the reference has no CPU twin with the same semantics (their parity is
 * checked by invariants instead).
 *
 * Layout: f[q*N + flat], flat = i*ny*nz + j*nz + k (lbm_kernels.cu:6-9).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef REAL
#define REAL double
#endif

typedef long long i64;

static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

/* weights and 2nd-order Hermite diagonal literals are supplied by the caller
 * (lbm_kernels.cu:65-71 and :836-838 use 8-digit decimals) */
static REAL Wq[19];
static REAL QD_ON = (REAL)0.66666667, QD_OFF = (REAL)-0.33333333;

void or_set_constants(const double* w19, double qd_on, double qd_off) {
    for (int q = 0; q < 19; ++q) Wq[q] = (REAL)w19[q];
    QD_ON = (REAL)qd_on;
    QD_OFF = (REAL)qd_off;
}

int or_sizeof_real(void) { return (int)sizeof(REAL); }

/* lbm_kernels.cu:77-113 */
static void feq_of(REAL rho, REAL ux, REAL uy, REAL uz, REAL feq[19]) {
    const REAL t = (REAL)1.5 * (ux * ux + uy * uy + uz * uz);
    for (int q = 0; q < 19; ++q) {
        const REAL cu = (REAL)3 * (CX[q] * ux + CY[q] * uy + CZ[q] * uz);
        feq[q] = Wq[q] * rho * ((REAL)1 + cu + (REAL)0.5 * cu * cu - t);
    }
}

/* lbm_kernels.cu:286-297 */
static void macros_of(const REAL f[19], REAL* rho, REAL* ux, REAL* uy, REAL* uz, REAL* inv_rho) {
    REAL r = 0, jx = 0, jy = 0, jz = 0;
    for (int q = 0; q < 19; ++q) {
        r += f[q];
        jx += CX[q] * f[q];
        jy += CY[q] * f[q];
        jz += CZ[q] * f[q];
    }
    const REAL ir = (REAL)1 / (r + (REAL)1e-12);
    *rho = r; *inv_rho = ir;
    *ux = jx * ir; *uy = jy * ir; *uz = jz * ir;
}

/* params: [omega, omega_plus, omega_minus, Cs_dx2, omega0]; S, M, Minv only for MRT modes.
 * mode 0 BGK (:258-308), 1 TRT (:315-365), 2 MRT (:374-436), 3 MRT+Smagorinsky (:1018-1117). */
void or_macro_collide(int mode, const REAL* f, REAL* fp, REAL* rho, REAL* u, REAL* v, REAL* w,
                      const uint8_t* solid, const double* params, const double* S, const double* M,
                      const double* Minv, i64 N) {
    const REAL omega = (REAL)params[0], op = (REAL)params[1], om = (REAL)params[2];
    const REAL Cs_dx2 = (REAL)params[3], omega0 = (REAL)params[4];
#pragma omp parallel for schedule(static)
    for (i64 x = 0; x < N; ++x) {
        if (solid[x]) {
            for (int q = 0; q < 19; ++q) fp[q * N + x] = Wq[q];
            rho[x] = 1; u[x] = 0; v[x] = 0; w[x] = 0;
            continue;
        }
        REAL fi[19], feq[19], out[19];
        for (int q = 0; q < 19; ++q) fi[q] = f[q * N + x];
        REAL r, ux, uy, uz, ir;
        macros_of(fi, &r, &ux, &uy, &uz, &ir);
        rho[x] = r; u[x] = ux; v[x] = uy; w[x] = uz;
        feq_of(r, ux, uy, uz, feq);
        if (mode == 0) {
            for (int q = 0; q < 19; ++q) out[q] = fi[q] + omega * (feq[q] - fi[q]);
        } else if (mode == 1) {
            for (int q = 0; q < 19; ++q) {
                const int o = OPP[q];
                const REAL fpl = (REAL)0.5 * (fi[q] + fi[o]), fmi = (REAL)0.5 * (fi[q] - fi[o]);
                const REAL epl = (REAL)0.5 * (feq[q] + feq[o]), emi = (REAL)0.5 * (feq[q] - feq[o]);
                out[q] = (fpl + op * (epl - fpl)) + (fmi + om * (emi - fmi));
            }
        } else {
            REAL s[19], m[19], meq[19], dm[19];
            for (int k = 0; k < 19; ++k) {
                s[k] = (REAL)S[k];
                REAL a = 0, b = 0;
                for (int q = 0; q < 19; ++q) {
                    a += (REAL)M[k * 19 + q] * fi[q];
                    b += (REAL)M[k * 19 + q] * feq[q];
                }
                m[k] = a; meq[k] = b;
            }
            if (mode == 3) {
                REAL P[6] = {0, 0, 0, 0, 0, 0};
                for (int q = 0; q < 19; ++q) {
                    const REAL n = fi[q] - feq[q];
                    const REAL a = CX[q], b = CY[q], c = CZ[q];
                    P[0] += n * a * a; P[1] += n * b * b; P[2] += n * c * c;
                    P[3] += n * a * b; P[4] += n * a * c; P[5] += n * b * c;
                }
                const REAL piF = (REAL)sqrt((double)(P[0] * P[0] + P[1] * P[1] + P[2] * P[2] +
                                                     (REAL)2 * (P[3] * P[3] + P[4] * P[4] + P[5] * P[5])));
                const REAL nu0 = ((REAL)1 / omega0 - (REAL)0.5) / (REAL)3;
                const REAL disc = nu0 * nu0 + (REAL)4 * Cs_dx2 * (piF * ir) * (REAL)4.5;
                const REAL dd = disc > nu0 * nu0 ? disc : nu0 * nu0;
                const REAL nu_eff = (REAL)0.5 * (nu0 + (REAL)sqrt((double)dd));
                REAL oe = (REAL)1 / ((REAL)3 * nu_eff + (REAL)0.5);
                if (oe > (REAL)1.99) oe = (REAL)1.99;
                s[9] = oe; s[11] = oe; s[13] = oe; s[14] = oe; s[15] = oe;
            }
            for (int k = 0; k < 19; ++k) dm[k] = s[k] * (m[k] - meq[k]);
            dm[0] = 0; dm[3] = 0; dm[5] = 0; dm[7] = 0;
            for (int q = 0; q < 19; ++q) {
                REAL d = 0;
                for (int k = 0; k < 19; ++k) d += (REAL)Minv[q * 19 + k] * dm[k];
                out[q] = fi[q] - d;
            }
        }
        for (int q = 0; q < 19; ++q) fp[q * N + x] = out[q];
    }
}

/* lbm_kernels.cu:447-496: pull; periodic axes wrap, a non-periodic source outside keeps own value */
void or_stream_pull(const REAL* fin, REAL* fout, int nx, int ny, int nz, int px, int py, int pz) {
    const i64 N = (i64)nx * ny * nz;
    const i64 nynz = (i64)ny * nz;
#pragma omp parallel for schedule(static)
    for (i64 x = 0; x < N; ++x) {
        const int i = (int)(x / nynz), j = (int)((x % nynz) / nz), k = (int)(x % nz);
        for (int q = 0; q < 19; ++q) {
            int si = i - CX[q], sj = j - CY[q], sk = k - CZ[q];
            int self = 0;
            if (si < 0 || si >= nx) { if (px) si = (si + nx) % nx; else self = 1; }
            if (!self && (sj < 0 || sj >= ny)) { if (py) sj = (sj + ny) % ny; else self = 1; }
            if (!self && (sk < 0 || sk >= nz)) { if (pz) sk = (sk + nz) % nz; else self = 1; }
            const i64 src = self ? x : (si * nynz + (i64)sj * nz + sk);
            fout[q * N + x] = fin[q * N + src];
        }
    }
}

/* lbm_kernels.cu:505-528 */
void or_sponge(REAL* f, const REAL* rho, const REAL* u, const REAL* v, const REAL* w, const REAL* sigma, i64 N) {
#pragma omp parallel for schedule(static)
    for (i64 x = 0; x < N; ++x) {
        const REAL sg = sigma[x];
        if (sg <= 0) continue;
        REAL feq[19];
        feq_of(rho[x], u[x], v[x], w[x], feq);
        for (int q = 0; q < 19; ++q) f[q * N + x] = f[q * N + x] - sg * (f[q * N + x] - feq[q]);
    }
}

/* lbm_kernels.cu:542-588 (links are independent: each (dir, x_f) occurs once) */
void or_ibb(const REAL* fpost, REAL* fs, const int64_t* fluid_flat, const int64_t* dir_i, const int64_t* dir_opp,
            const REAL* w1, const REAL* w2, const uint8_t* ge, const int64_t* ff_flat, const uint8_t* ff_valid,
            i64 n_links, i64 N) {
#pragma omp parallel for schedule(static)
    for (i64 l = 0; l < n_links; ++l) {
        const i64 xf = fluid_flat[l];
        const int qi = (int)dir_i[l], qo = (int)dir_opp[l];
        const REAL a = fpost[qo * N + xf];
        REAL bb;
        if (ge[l]) bb = w1[l] * a + w2[l] * fpost[qi * N + xf];
        else if (ff_valid[l]) bb = w1[l] * a + w2[l] * fpost[qo * N + ff_flat[l]];
        else bb = a;
        fs[qi * N + xf] = bb;
    }
}

/* lbm_kernels.cu:597-609 */
void or_reset_solid(REAL* f, const uint8_t* solid, i64 N) {
#pragma omp parallel for schedule(static)
    for (i64 x = 0; x < N; ++x)
        if (solid[x])
            for (int q = 0; q < 19; ++q) f[q * N + x] = Wq[q];
}

/* LBM_CHT.py:1322-1328: in-cell direction swap at flow-solid cells (no-link path) */
void or_swap_solid(REAL* f, const uint8_t* solid, i64 N) {
#pragma omp parallel for schedule(static)
    for (i64 x = 0; x < N; ++x) {
        if (!solid[x]) continue;
        REAL t[19];
        for (int q = 0; q < 19; ++q) t[q] = f[q * N + x];
        for (int q = 0; q < 19; ++q) f[q * N + x] = t[OPP[q]];
    }
}

static i64 pflat(int axis, int p, int a, int b, int ny, int nz) {
    if (axis == 0) return ((i64)p * ny + a) * nz + b;
    if (axis == 1) return ((i64)a * ny + p) * nz + b;
    return ((i64)a * ny + b) * nz + p;
}
static int cax(int q, int axis) { return axis == 0 ? CX[q] : (axis == 1 ? CY[q] : CZ[q]); }
static REAL qdiag(int c) { return c != 0 ? QD_ON : QD_OFF; }

/* lbm_kernels.cu:791-969: regularized Zou/He, velocity inlet (0) or pressure outlet (1) */
void or_zou_he(REAL* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int plane_idx, int interior_idx,
               int bc_type, double u_in_d, double rho_out_d, int sign) {
    const i64 N = (i64)nx * ny * nz;
    const int n1 = axis == 0 ? ny : nx, n2 = axis == 2 ? ny : nz;
    const REAL u_in = (REAL)u_in_d, rho_out = (REAL)rho_out_d;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < n1 * n2; ++t) {
        const int a = t / n2, b = t % n2;
        const i64 fb = pflat(axis, plane_idx, a, b, ny, nz), fin = pflat(axis, interior_idx, a, b, ny, nz);
        if (solid[fb]) continue;
        REAL fi[19];
        for (int q = 0; q < 19; ++q) fi[q] = f[q * N + fb];
        const int unknown = plane_idx == 0 ? 1 : -1, known = -unknown;
        REAL s0 = 0, sk = 0;
        for (int q = 0; q < 19; ++q) {
            if (cax(q, axis) == 0) s0 += fi[q];
            if (cax(q, axis) == known) sk += fi[q];
        }
        REAL rho_bc, uax, ub = 0, vb = 0, wb = 0;
        if (bc_type == 0) {
            uax = u_in;
            rho_bc = (s0 + (REAL)2 * sk) / ((REAL)1 - (REAL)fabs((double)u_in) + (REAL)1e-12);
            if (rho_bc < (REAL)0.2) rho_bc = (REAL)0.2;
            if (rho_bc > (REAL)5.0) rho_bc = (REAL)5.0;
            if (axis == 0) ub = uax; else if (axis == 1) vb = uax; else wb = uax;
        } else {
            rho_bc = rho_out;
            uax = (REAL)known * ((s0 + (REAL)2 * sk) / (rho_bc + (REAL)1e-12) - (REAL)1);
            if (uax * (REAL)sign < 0) {
                for (int q = 0; q < 19; ++q) f[q * N + fb] = f[q * N + fin];
                continue;
            }
            REAL g[19], r, ux, uy, uz, ir;
            for (int q = 0; q < 19; ++q) g[q] = f[q * N + fin];
            macros_of(g, &r, &ux, &uy, &uz, &ir);
            if (axis == 0) { ub = uax; vb = uy; wb = uz; }
            else if (axis == 1) { ub = ux; vb = uax; wb = uz; }
            else { ub = ux; vb = uy; wb = uax; }
        }
        REAL feq[19], g[19];
        feq_of(rho_bc, ub, vb, wb, feq);
        for (int q = 0; q < 19; ++q)
            g[q] = cax(q, axis) == unknown ? fi[OPP[q]] + feq[q] - feq[OPP[q]] : fi[q];
        REAL Pxx = 0, Pyy = 0, Pzz = 0, Pxy = 0, Pxz = 0, Pyz = 0;
        for (int q = 0; q < 19; ++q) {
            const REAL n = g[q] - feq[q];
            Pxx += n * qdiag(CX[q]); Pyy += n * qdiag(CY[q]); Pzz += n * qdiag(CZ[q]);
            Pxy += n * (REAL)(CX[q] * CY[q]); Pxz += n * (REAL)(CX[q] * CZ[q]); Pyz += n * (REAL)(CY[q] * CZ[q]);
        }
        for (int q = 0; q < 19; ++q) {
            const REAL s = qdiag(CX[q]) * Pxx + qdiag(CY[q]) * Pyy + qdiag(CZ[q]) * Pzz +
                           (REAL)2 * ((REAL)(CX[q] * CY[q]) * Pxy + (REAL)(CX[q] * CZ[q]) * Pxz +
                                      (REAL)(CY[q] * CZ[q]) * Pyz);
            f[q * N + fb] = feq[q] + Wq[q] * s * (REAL)4.5;
        }
    }
}

/* lbm_kernels.cu:1170-1344: zero-gradient copy of incoming populations, then
 * scale the fluid outlet nodes by rho_out * count / sum(rho) */
void or_convective(REAL* f, const uint8_t* solid, int nx, int ny, int nz, int axis, int outlet_idx, int interior_idx,
                   int unknown_cax, double rho_out) {
    const i64 N = (i64)nx * ny * nz;
    const int n1 = axis == 0 ? ny : nx, n2 = axis == 2 ? ny : nz;
    double sum = 0.0;
    long cnt = 0;
    for (int t = 0; t < n1 * n2; ++t) {
        const int a = t / n2, b = t % n2;
        const i64 fo = pflat(axis, outlet_idx, a, b, ny, nz), fi = pflat(axis, interior_idx, a, b, ny, nz);
        if (solid[fo]) continue;
        REAL r = 0;
        for (int q = 0; q < 19; ++q) {
            if (cax(q, axis) == unknown_cax) f[q * N + fo] = f[q * N + fi];
            r += f[q * N + fo];
        }
        sum += (double)r;
        cnt += 1;
    }
    if (cnt < 1 || sum < 1e-10) return;
    const REAL corr = (REAL)(rho_out * (double)cnt / sum);
    for (int t = 0; t < n1 * n2; ++t) {
        const int a = t / n2, b = t % n2;
        const i64 fo = pflat(axis, outlet_idx, a, b, ny, nz);
        if (solid[fo]) continue;
        for (int q = 0; q < 19; ++q) f[q * N + fo] *= corr;
    }
}
