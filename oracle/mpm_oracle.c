/*
 * CPU oracle for the MPM substep of MPM_Simulator_WARP.p2g2p.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it.
 * The product (reduced_mpm_stress_training_gb300) never links or calls it.
 *
 * It restates, operation for operation, the Warp kernels of the reference in
 * plain C on the reference's own data layout (AoS vec3 / row-major mat33 per
 * particle, dense (n,n,n) C-order grid):
 *   engine_stress/mpm_utils.py:4-19     update_x_from_u / update_u_from_x /
 *                                       update_F_disp_from_F
 *   engine_stress/mpm_utils.py:29-52    Kirchhoff stresses (FCR, StVK, DP)
 *   engine_stress/mpm_utils.py:54-57    compute_dweight
 *   engine_stress/mpm_utils.py:59-84    von_mises_return_mapping
 *   engine_stress/mpm_utils.py:87-112   sand_return_mapping
 *   engine_stress/mpm_utils.py:115-123  zero_grid
 *   engine_stress/mpm_utils.py:190-227  p2g_apic_stress_given
 *   engine_stress/mpm_utils.py:229-237  grid_normalization_and_gravity
 *   engine_stress/mpm_utils.py:241-306  g2p_apic_and_stress
 *   engine_stress/mpm_solver_warp.py:429-449  surface collider kernel
 *   engine_stress/mpm_solver_warp.py:505-523  bounding-box kernel
 *   engine_stress/mpm_solver_warp.py:156-199  p2g2p launch order
 *   engine_stress/mpm_utils.py:318-471  reduced sampled-quadrature kernels
 *                                       (update_neighboring_cells[_for_grid_v],
 *                                       p2g_sample_all,
 *                                       grid_normalization_and_gravity_sample_all,
 *                                       g2p_sample)
 *   engine_stress/mpm_solver_warp.py:214-227  p2g2p_reduced launch order
 *
 * The 3x3 SVD (Warp's wp.svd3, third-party, unpinned version, source not in
 * the reference tree) is restated from the published method it follows:
 * McAdams, Selle, Tamstorf, Teran, Sifakis, "Computing the Singular Value
 * Decomposition of 3x3 matrices with minimal branching and elementary floating
 * point operations", UW-Madison CS TR1690 (2011): Jacobi eigen-analysis of
 * A^T A with quaternion-accumulated approximate Givens rotations,
 * column sort by norm with sign-corrected swaps, Givens QR.  The paper uses 4
 * Jacobi sweeps; near F = I (nearly equal singular values, the common case
 * here) 4 sweeps leave a 1e-6 relative off-diagonal in A^T A and a 1e-5
 * reconstruction error, while 5 sweeps converge to float32 rounding, so the
 * float build uses ORC_SWEEPS = 5 (the GPU kernel uses the same count).  Convention:
 * U, V proper rotations, singular values sorted by magnitude, the sign of
 * det(A) carried by s[2].  In the f64 build the Jacobi rotations are exact
 * and iterated to convergence, so the f64 oracle is an accurate rerun.
 *
 * Pinning: the reference ships no tests, golden vectors or fixtures for this
 * path, and warp-lang is not installed.  Its unmodified solver
 * (engine_stress/mpm_solver_warp.py, mpm_utils.py) was therefore run on the
 * CPU through a test-only stand-in of the Warp API (tests/refshim); the
 * fixtures it wrote (tests/golden/ref_*.npz, by
 * tests/golden/make_ref_fixtures.py) pin this oracle substep by substep
 * (tests/test_ref_fixtures_cpu.py), next to closed-form known-answer cases
 * and an independent NumPy/LAPACK restatement.
 *
 * Deliberate deviation from the reference (which has undefined behaviour
 * there): a particle whose stencil would leave the grid (base index outside
 * [0, n-3] or a non-finite position) is skipped by P2G and G2P and flagged in
 * the status word (bit 1) instead of indexing out of bounds.
 *
 * Built twice from this one source: -DORC_F64 gives the orc64_* symbols
 * (double), otherwise orc32_* (float).  Compile with -ffp-contract=off so the
 * float build rounds like the reference's scalar arithmetic on every host.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORC_F64
typedef double real;
#define PFX(name) orc64_##name
#define RLOG log
#define REXP exp
#define RSQRT sqrt
#define RABS fabs
#else
typedef float real;
#define PFX(name) orc32_##name
#define RLOG logf
#define REXP expf
#define RSQRT sqrtf
#define RABS fabsf
#endif

#ifndef ORC_SWEEPS
#define ORC_SWEEPS 5
#endif

#define ST_OUT_OF_DOMAIN 1
#define ST_CFL 2
#define ST_NONFINITE 4
#define ST_BAD_INPUT 16

/* Model parameters in double; every use rounds to `real` first, as Warp
 * stores them as float32 struct members (engine_stress/warp_utils.py:61-81). */
typedef struct {
    int32_t n_grid;
    int32_t material; /* 0 jelly, 1 metal, 2 sand */
    int32_t hardening;
    int32_t pad0;
    double dx, inv_dx;
    double mu, lam, alpha, xi;
    double gravity[3]; /* reference: (0, -g, 0), mpm_utils.py:236 */
} OrcModel;

/* Dirichlet_collider (warp_utils.py:126-151).  kind 0 = surface collider,
 * 1 = bounding box, 2 = velocity on an infinite plane, 3 = column moving as
 * a circle, 4 = rotation on a disk, 5 = velocity on a cube, 6 = sphere
 * leader (mpm_solver_warp.py:407-720).  The moving kinds' points are
 * advanced by the caller between substeps (the reference's modify_bc). */
typedef struct {
    int32_t kind;
    int32_t surface_type;
    double point[3];
    double normal[3];
    double friction;
    double start_time, end_time;
    int32_t reset;
    int32_t pad;
    double velocity[3];
    double threshold, radius, width, height, v_scale;
    double x_unit[3], y_unit[3];
    double R;
} OrcCollider;

/* ------------------------------------------------------------------ */
/* small matrix helpers (row-major 3x3)                                */
/* ------------------------------------------------------------------ */
static void mm3(const real *a, const real *b, real *c) {
    real t[9];
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
            /* Warp's mat33 product accumulates left to right */
            real s = a[r * 3 + 0] * b[0 * 3 + k];
            s = s + a[r * 3 + 1] * b[1 * 3 + k];
            s = s + a[r * 3 + 2] * b[2 * 3 + k];
            t[r * 3 + k] = s;
        }
    memcpy(c, t, sizeof(t));
}
static void transpose3(const real *a, real *t) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t[c * 3 + r] = a[r * 3 + c];
}
static real det3(const real *a) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

/* ------------------------------------------------------------------ */
/* 3x3 SVD (published method named in the header)                      */
/* ------------------------------------------------------------------ */
static void quat_mul_axis(real q[4], int k, real ch, real sh) {
    /* q <- q (x) (ch, sh e_k); q = (w, x, y, z) */
    real w = q[0], v[3] = {q[1], q[2], q[3]};
    real r[3] = {0, 0, 0};
    r[k] = sh;
    real nw = w * ch - (v[0] * r[0] + v[1] * r[1] + v[2] * r[2]);
    real cx = v[1] * r[2] - v[2] * r[1];
    real cy = v[2] * r[0] - v[0] * r[2];
    real cz = v[0] * r[1] - v[1] * r[0];
    q[0] = nw;
    q[1] = w * r[0] + ch * v[0] + cx;
    q[2] = w * r[1] + ch * v[1] + cy;
    q[3] = w * r[2] + ch * v[2] + cz;
}

/* One Jacobi conjugation S <- G^T S G in the (p,q) plane, G a right-handed
 * rotation about axis k; returns nothing, updates S (full symmetric) and q. */
static void jacobi_rotate(real S[3][3], real q[4], int p, int qq, int k) {
    real a = S[p][p], b = S[p][qq], d = S[qq][qq];
    real ch, sh;
#ifdef ORC_F64
    if (b == 0.0) return;
    {
        double tau = (a - d) / (2.0 * b);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t);
        double s = t * c;
        ch = sqrt(0.5 * (1.0 + c));
        sh = s / (2.0 * ch);
    }
#else
    {
        /* approximate Givens half-angle, McAdams et al. 2011, sec. 2.2 */
        const real gamma = 5.828427124746190f; /* 3 + 2 sqrt(2) */
        const real cstar = 0.923879532511287f; /* cos(pi/8) */
        const real sstar = 0.382683432365090f; /* sin(pi/8) */
        ch = 2.0f * (a - d);
        sh = b;
        if (gamma * sh * sh < ch * ch) {
            real w = 1.0f / sqrtf(ch * ch + sh * sh);
            ch = w * ch;
            sh = w * sh;
        } else {
            ch = cstar;
            sh = sstar;
        }
    }
#endif
    real c = ch * ch - sh * sh;
    real s = 2 * ch * sh;
    real app = c * c * a + 2 * c * s * b + s * s * d;
    real aqq = s * s * a - 2 * c * s * b + c * c * d;
    real apq = b * (c * c - s * s) + (d - a) * c * s;
    real apk = c * S[p][k] + s * S[qq][k];
    real aqk = -s * S[p][k] + c * S[qq][k];
    S[p][p] = app;
    S[qq][qq] = aqq;
    S[p][qq] = S[qq][p] = apq;
    S[p][k] = S[k][p] = apk;
    S[qq][k] = S[k][qq] = aqk;
    quat_mul_axis(q, k, ch, sh);
}

static void swap_cols_neg(real B[3][3], real V[3][3], int i, int j) {
    for (int r = 0; r < 3; ++r) {
        real tb = B[r][i];
        B[r][i] = B[r][j];
        B[r][j] = -tb;
        real tv = V[r][i];
        V[r][i] = V[r][j];
        V[r][j] = -tv;
    }
}

static void givens_qr_step(real B[3][3], real U[3][3], int p, int q, int col) {
    real a1 = B[p][col], a2 = B[q][col];
    real rho = RSQRT(a1 * a1 + a2 * a2);
    real c = 1, s = 0;
    if (rho > 0) {
        c = a1 / rho;
        s = a2 / rho;
    }
    for (int j = 0; j < 3; ++j) {
        real bp = B[p][j], bq = B[q][j];
        B[p][j] = c * bp + s * bq;
        B[q][j] = -s * bp + c * bq;
    }
    for (int r = 0; r < 3; ++r) {
        real up = U[r][p], uq = U[r][q];
        U[r][p] = c * up + s * uq;
        U[r][q] = -s * up + c * uq;
    }
}

void PFX(svd3)(const real *A, real *Uo, real *so, real *Vo) {
    real S[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            real acc = A[0 * 3 + i] * A[0 * 3 + j];
            acc = acc + A[1 * 3 + i] * A[1 * 3 + j];
            acc = acc + A[2 * 3 + i] * A[2 * 3 + j];
            S[i][j] = acc;
        }
    real q[4] = {1, 0, 0, 0};
#ifdef ORC_F64
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = S[0][1] * S[0][1] + S[1][2] * S[1][2] + S[0][2] * S[0][2];
        double dia = S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2];
        if (off <= 1e-34 * dia || off == 0.0) break;
        jacobi_rotate(S, q, 0, 1, 2);
        jacobi_rotate(S, q, 1, 2, 0);
        jacobi_rotate(S, q, 2, 0, 1);
    }
#else
    for (int sweep = 0; sweep < ORC_SWEEPS; ++sweep) {
        jacobi_rotate(S, q, 0, 1, 2);
        jacobi_rotate(S, q, 1, 2, 0);
        jacobi_rotate(S, q, 2, 0, 1);
    }
#endif
    real qn = RSQRT(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    real w = q[0] / qn, x = q[1] / qn, y = q[2] / qn, z = q[3] / qn;
    real V[3][3] = {
        {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
        {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
        {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    real B[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            real acc = A[r * 3 + 0] * V[0][c];
            acc = acc + A[r * 3 + 1] * V[1][c];
            acc = acc + A[r * 3 + 2] * V[2][c];
            B[r][c] = acc;
        }
    real rho[3];
    for (int c = 0; c < 3; ++c) rho[c] = B[0][c] * B[0][c] + B[1][c] * B[1][c] + B[2][c] * B[2][c];
    if (rho[0] < rho[1]) {
        swap_cols_neg(B, V, 0, 1);
        real t = rho[0]; rho[0] = rho[1]; rho[1] = t;
    }
    if (rho[0] < rho[2]) {
        swap_cols_neg(B, V, 0, 2);
        real t = rho[0]; rho[0] = rho[2]; rho[2] = t;
    }
    if (rho[1] < rho[2]) {
        swap_cols_neg(B, V, 1, 2);
        real t = rho[1]; rho[1] = rho[2]; rho[2] = t;
    }
    real U[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    givens_qr_step(B, U, 0, 1, 0);
    givens_qr_step(B, U, 0, 2, 0);
    givens_qr_step(B, U, 1, 2, 1);
    so[0] = B[0][0];
    so[1] = B[1][1];
    so[2] = B[2][2];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            Uo[r * 3 + c] = U[r][c];
            Vo[r * 3 + c] = V[r][c];
        }
}

void PFX(svd3_batch)(int64_t n, const real *A, real *U, real *s, real *V) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) PFX(svd3)(A + 9 * p, U + 9 * p, s + 3 * p, V + 9 * p);
}

/* U diag(d) V^T */
static void udvt(const real *U, const real *d, const real *V, real *out) {
    real D[9] = {d[0], 0, 0, 0, d[1], 0, 0, 0, d[2]};
    real Vt[9], t[9];
    transpose3(V, Vt);
    mm3(U, D, t);
    mm3(t, Vt, out);
}

/* ------------------------------------------------------------------ */
/* stresses, mpm_utils.py:29-52                                        */
/* ------------------------------------------------------------------ */
static void kirchoff_stress_FCR(const real *F, const real *U, const real *V, real J, real mu,
                                real lam, real *tau) {
    real Vt[9], R[9], FmR[9], Ft[9], t[9];
    transpose3(V, Vt);
    mm3(U, Vt, R);
    for (int i = 0; i < 9; ++i) FmR[i] = F[i] - R[i];
    for (int i = 0; i < 9; ++i) FmR[i] = (2 * mu) * FmR[i];
    transpose3(F, Ft);
    mm3(FmR, Ft, t);
    real diag = lam * J * (J - 1);
    for (int i = 0; i < 9; ++i) tau[i] = t[i] + ((i % 4 == 0) ? diag : 0);
}

static void kirchoff_stress_StVK(const real *U, const real *V, const real *sig_in, real mu,
                                 real lam, real *tau) {
    real sig[3];
    for (int i = 0; i < 3; ++i) sig[i] = sig_in[i] > (real)0.01 ? sig_in[i] : (real)0.01;
    real eps[3] = {RLOG(sig[0]), RLOG(sig[1]), RLOG(sig[2])};
    real lss = RLOG(sig[0]) + RLOG(sig[1]) + RLOG(sig[2]);
    real t[3];
    for (int i = 0; i < 3; ++i) t[i] = 2 * mu * eps[i] + lam * lss * 1;
    udvt(U, t, V, tau);
}

static void kirchoff_stress_drucker_prager(const real *F, const real *U, const real *V,
                                           const real *sig, real mu, real lam, real *tau) {
    real lss = RLOG(sig[0]) + RLOG(sig[1]) + RLOG(sig[2]);
    real c[3];
    for (int i = 0; i < 3; ++i)
        c[i] = 2 * mu * RLOG(sig[i]) * (1 / sig[i]) + lam * lss * (1 / sig[i]);
    real t[9], Ft[9];
    udvt(U, c, V, t);
    transpose3(F, Ft);
    mm3(t, Ft, tau);
}

/* ------------------------------------------------------------------ */
/* return mappings, mpm_utils.py:59-112                                */
/* ------------------------------------------------------------------ */
static void von_mises_return_mapping(const real *F_trial, real mu, real lam, int hardening,
                                     real xi, real *yield_p, real *F_out) {
    real U[9], V[9], sig_old[3];
    PFX(svd3)(F_trial, U, sig_old, V);
    real sig[3];
    for (int i = 0; i < 3; ++i) sig[i] = sig_old[i] > (real)0.01 ? sig_old[i] : (real)0.01;
    real eps[3] = {RLOG(sig[0]), RLOG(sig[1]), RLOG(sig[2])};
    real temp = (eps[0] + eps[1] + eps[2]) / 3;
    real tau[3];
    real se = eps[0] + eps[1] + eps[2];
    for (int i = 0; i < 3; ++i) tau[i] = 2 * mu * eps[i] + lam * se * 1;
    real sum_tau = tau[0] + tau[1] + tau[2];
    real cond[3] = {tau[0] - sum_tau / 3, tau[1] - sum_tau / 3, tau[2] - sum_tau / 3};
    real cl = RSQRT(cond[0] * cond[0] + cond[1] * cond[1] + cond[2] * cond[2]);
    if (cl > *yield_p) {
        real eh[3] = {eps[0] - temp, eps[1] - temp, eps[2] - temp};
        real ehn = RSQRT(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]) + (real)1e-6;
        real dg = ehn - *yield_p / (2 * mu);
        for (int i = 0; i < 3; ++i) eps[i] = eps[i] - (dg / ehn) * eh[i];
        real se2[3] = {REXP(eps[0]), REXP(eps[1]), REXP(eps[2])};
        udvt(U, se2, V, F_out);
        if (hardening == 1) *yield_p = *yield_p + 2 * mu * xi * dg;
    } else {
        memcpy(F_out, F_trial, 9 * sizeof(real));
    }
}

static void sand_return_mapping(const real *F_trial, real mu, real lam, real alpha,
                                real *F_out) {
    real U[9], V[9], sig[3];
    PFX(svd3)(F_trial, U, sig, V);
    real eps[3];
    for (int i = 0; i < 3; ++i) {
        real a = RABS(sig[i]);
        eps[i] = RLOG(a > (real)1e-14 ? a : (real)1e-14);
    }
    real tr = eps[0] + eps[1] + eps[2];
    real eh[3] = {eps[0] - tr / 3, eps[1] - tr / 3, eps[2] - tr / 3};
    real ehn = RSQRT(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
    real dg = ehn + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha;
    if (dg <= 0) {
        memcpy(F_out, F_trial, 9 * sizeof(real));
    } else if (tr > 0) {
        real Vt[9];
        transpose3(V, Vt);
        mm3(U, Vt, F_out);
    } else {
        real H[3], sn[3];
        for (int i = 0; i < 3; ++i) H[i] = eps[i] - eh[i] * (dg / ehn);
        for (int i = 0; i < 3; ++i) sn[i] = REXP(H[i]);
        udvt(U, sn, V, F_out);
    }
}

/* Return map + stress for one particle exactly as g2p_apic_and_stress does
 * after F_trial is formed (mpm_utils.py:284-306): first SVD inside the return
 * map, second SVD of the new F for the stress. */
static void return_map_and_stress(const OrcModel *m, const real *F_trial, real *yield_p,
                                  real *F_out, real *tau) {
    real mu = (real)m->mu, lam = (real)m->lam;
    if (m->material == 1) {
        von_mises_return_mapping(F_trial, mu, lam, m->hardening, (real)m->xi, yield_p, F_out);
    } else if (m->material == 2) {
        sand_return_mapping(F_trial, mu, lam, (real)m->alpha, F_out);
    } else {
        memcpy(F_out, F_trial, 9 * sizeof(real));
    }
    real J = det3(F_out);
    real U[9], V[9], sig[3];
    PFX(svd3)(F_out, U, sig, V);
    memset(tau, 0, 9 * sizeof(real));
    if (m->material == 0) kirchoff_stress_FCR(F_out, U, V, J, mu, lam, tau);
    if (m->material == 1) kirchoff_stress_StVK(U, V, sig, mu, lam, tau);
    if (m->material == 2) kirchoff_stress_drucker_prager(F_out, U, V, sig, mu, lam, tau);
}

void PFX(return_map_batch)(const OrcModel *m, int64_t n, const real *F_trial, real *yield,
                           real *F_out, real *tau) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        real y = yield ? yield[p] : 0;
        return_map_and_stress(m, F_trial + 9 * p, &y, F_out + 9 * p, tau + 9 * p);
        if (yield) yield[p] = y;
    }
}

/* ------------------------------------------------------------------ */
/* per-particle conversions, mpm_utils.py:4-19                         */
/* ------------------------------------------------------------------ */
void PFX(update_x_from_u)(int64_t n, const real *x0, const real *u, real *x) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < 3 * n; ++i) x[i] = x0[i] + u[i];
}
void PFX(update_u_from_x)(int64_t n, const real *x, const real *x0, real *u) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < 3 * n; ++i) u[i] = x[i] - x0[i];
}
void PFX(update_F_disp_from_F)(int64_t n, const real *F, real *Fd) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p)
        for (int k = 0; k < 9; ++k) Fd[9 * p + k] = F[9 * p + k] - ((k % 4 == 0) ? 1 : 0);
}

/* ------------------------------------------------------------------ */
/* grid kernels                                                        */
/* ------------------------------------------------------------------ */
void PFX(zero_grid)(int64_t n_nodes, real *gm, real *gvin, real *gvout) {
    memset(gm, 0, (size_t)n_nodes * sizeof(real));
    memset(gvin, 0, (size_t)n_nodes * 3 * sizeof(real));
    memset(gvout, 0, (size_t)n_nodes * 3 * sizeof(real));
}

/* Stencil set-up shared by P2G and G2P (mpm_utils.py:196-209, 244-257).
 * Returns 0 if the particle's 3x3x3 stencil lies inside the grid. */
static int stencil(const real *xp, real inv_dx, int n, int base[3], real fx[3], real w[3][3],
                   real dw[3][3]) {
    for (int d = 0; d < 3; ++d) {
        real gp = xp[d] * inv_dx;
        real t = gp - (real)0.5;
        if (!(t > (real)-1 && t < (real)(n - 2))) return 1; /* also catches NaN */
        base[d] = (int)t; /* wp.int truncates toward zero */
        fx[d] = gp - (real)base[d];
    }
    for (int d = 0; d < 3; ++d) {
        real wa = (real)1.5 - fx[d];
        real wb = fx[d] - (real)1.0;
        real wc = fx[d] - (real)0.5;
        /* w[d][i]: dimension d, node offset i (wp.mat33 built from columns) */
        w[d][0] = wa * wa * (real)0.5;
        w[d][1] = ((real)0.0 - wb * wb) + (real)0.75;
        w[d][2] = wc * wc * (real)0.5;
        dw[d][0] = fx[d] - (real)1.5;
        dw[d][1] = (real)-2.0 * (fx[d] - (real)1.0);
        dw[d][2] = fx[d] - (real)0.5;
    }
    return 0;
}

static inline int64_t gidx(int n, int ix, int iy, int iz) {
    return ((int64_t)ix * n + iy) * n + iz;
}

static inline void add_real(real *dst, real v, int par) {
    if (par) {
#pragma omp atomic
        *dst += v;
    } else {
        *dst += v;
    }
}

/* mpm_utils.py:190-227.  nthreads == 1 gives a deterministic sequential
 * scatter (particle order); nthreads > 1 scatters with atomics. */
void PFX(p2g_apic_stress_given)(const OrcModel *m, int64_t np, const real *x, const real *v,
                                const real *C, const real *stress, const real *mass,
                                const real *vol, real dt, real *gm, real *gvin, int32_t *status,
                                int nthreads) {
    const int n = m->n_grid;
    const real inv_dx = (real)m->inv_dx, dx = (real)m->dx;
    int par = nthreads > 1;
    int st = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) \
    reduction(| : st) if (par)
    for (int64_t p = 0; p < np; ++p) {
        int base[3];
        real fx[3], w[3][3], dw[3][3];
        if (stencil(x + 3 * p, inv_dx, n, base, fx, w, dw)) {
            st |= ST_OUT_OF_DOMAIN;
            continue;
        }
        const real *Cp = C + 9 * p, *tp = stress + 9 * p, *vp = v + 3 * p;
        real mp = mass[p], volp = vol[p];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    real dpos[3] = {((real)i - fx[0]) * dx, ((real)j - fx[1]) * dx,
                                    ((real)k - fx[2]) * dx};
                    real weight = w[0][i] * w[1][j] * w[2][k];
                    real dweight[3] = {dw[0][i] * w[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * w[1][j] * dw[2][k] * inv_dx};
                    int64_t g = gidx(n, base[0] + i, base[1] + j, base[2] + k);
                    real wm = weight * mp;
                    for (int r = 0; r < 3; ++r) {
                        real cd = Cp[r * 3 + 0] * dpos[0];
                        cd = cd + Cp[r * 3 + 1] * dpos[1];
                        cd = cd + Cp[r * 3 + 2] * dpos[2];
                        add_real(&gvin[3 * g + r], wm * (vp[r] + cd), par);
                    }
                    for (int r = 0; r < 3; ++r) {
                        /* elastic_force = (-vol * stress) * dweight */
                        real f = (-volp * tp[r * 3 + 0]) * dweight[0];
                        f = f + (-volp * tp[r * 3 + 1]) * dweight[1];
                        f = f + (-volp * tp[r * 3 + 2]) * dweight[2];
                        add_real(&gvin[3 * g + r], dt * f, par);
                    }
                    add_real(&gm[g], weight * mp, par);
                }
    }
    if (status) *status |= st;
}

/* mpm_utils.py:229-237, with the gravity vector generalised:
 * reference gravity = (0, -g, 0). */
void PFX(grid_normalization_and_gravity)(const OrcModel *m, real dt, const real *gm,
                                         const real *gvin, real *gvout) {
    const int n = m->n_grid;
    const int64_t nn = (int64_t)n * n * n;
    real gdt[3];
    for (int c = 0; c < 3; ++c) gdt[c] = dt * (real)m->gravity[c];
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < nn; ++g) {
        if (gm[g] > (real)1e-15f) {
            real inv = (real)1.0 / gm[g];
            for (int c = 0; c < 3; ++c) gvout[3 * g + c] = gvin[3 * g + c] * inv + gdt[c];
        }
    }
}

/* mpm_solver_warp.py:429-449 (every surface type writes zero, :449) */
void PFX(collide_surface)(const OrcModel *m, const OrcCollider *col, double time, real *gvout) {
    if (!((float)time >= (float)col->start_time && (float)time < (float)col->end_time)) return;
    const int n = m->n_grid;
    const real dx = (real)m->dx;
    real pt[3] = {(real)col->point[0], (real)col->point[1], (real)col->point[2]};
    real nr[3] = {(real)col->normal[0], (real)col->normal[1], (real)col->normal[2]};
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < n; ++ix)
        for (int iy = 0; iy < n; ++iy)
            for (int iz = 0; iz < n; ++iz) {
                real off[3] = {(real)ix * dx - pt[0], (real)iy * dx - pt[1], (real)iz * dx - pt[2]};
                real dp = off[0] * nr[0] + off[1] * nr[1] + off[2] * nr[2];
                if (dp < 0) {
                    int64_t g = gidx(n, ix, iy, iz);
                    gvout[3 * g + 0] = 0;
                    gvout[3 * g + 1] = 0;
                    gvout[3 * g + 2] = 0;
                }
            }
}

/* mpm_solver_warp.py:505-523, padding 3 */
void PFX(collide_bounding_box)(const OrcModel *m, const OrcCollider *col, double time,
                               real *gvout) {
    if (!((float)time >= (float)col->start_time && (float)time < (float)col->end_time)) return;
    const int n = m->n_grid, pad = 3;
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < n; ++ix)
        for (int iy = 0; iy < n; ++iy)
            for (int iz = 0; iz < n; ++iz) {
                int64_t g = gidx(n, ix, iy, iz);
                real *vv = gvout + 3 * g;
                int id[3] = {ix, iy, iz};
                for (int c = 0; c < 3; ++c) {
                    if (id[c] < pad && vv[c] < 0) vv[c] = 0;
                    if (id[c] >= n - pad && vv[c] > 0) vv[c] = 0;
                }
            }
}

/* float32 window tests, as the reference's kernels see float time and times */
static int col_active(const OrcCollider *col, double time) {
    return (float)time >= (float)col->start_time && (float)time < (float)col->end_time;
}

/* angle of the circling column's bottom point about (0.5, *, 0.5)
 * (mpm_solver_warp.py:585-592), float32 */
static float circle_theta(const OrcCollider *col) {
    const float z0 = (float)col->point[0] - 0.5f, z1 = (float)col->point[1], z2 = (float)col->point[2] - 0.5f;
    const float len = sqrtf(z0 * z0 + z1 * z1 + z2 * z2);
    float c = z0 / len;
    c = c < -1.0f ? -1.0f : (c > 1.0f ? 1.0f : c);
    const float th = acosf(c);
    return z2 < 0.0f ? -th : th;
}

/* kinds 2-6: mpm_solver_warp.py:545-559, :580-592, :635-659, :680-689,
 * :709-714; every node of the dense grid, as the reference launches them */
void PFX(collide_extended)(const OrcModel *m, const OrcCollider *col, double time, real dt, real *gvout) {
    const int act = col_active(col, time);
    const float tf = (float)time, dtf = (float)dt;
    const int n = m->n_grid;
    const float dx = (float)m->dx;
    const float pt[3] = {(float)col->point[0], (float)col->point[1], (float)col->point[2]};
    const float nr[3] = {(float)col->normal[0], (float)col->normal[1], (float)col->normal[2]};
    const float vel[3] = {(float)col->velocity[0], (float)col->velocity[1], (float)col->velocity[2]};
    const float xu[3] = {(float)col->x_unit[0], (float)col->x_unit[1], (float)col->x_unit[2]};
    const float yu[3] = {(float)col->y_unit[0], (float)col->y_unit[1], (float)col->y_unit[2]};
    const float thr = (float)col->threshold, rad = (float)col->radius, wid = (float)col->width;
    const float hei = (float)col->height, vs = (float)col->v_scale, endf = (float)col->end_time;
    const int reset_plane = !act && col->reset == 1 && tf < endf + 1.5f * dtf * 10.0f;
    const int reset_all = !act && col->reset == 1 && tf < endf + 1.5f * dtf;
    if (!act && !reset_plane && !reset_all) return;
    const float cth = col->kind == 3 ? circle_theta(col) : 0.0f;
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < n; ++ix)
        for (int iy = 0; iy < n; ++iy)
            for (int iz = 0; iz < n; ++iz) {
                real *vv = gvout + 3 * gidx(n, ix, iy, iz);
                const float o0 = (float)ix * dx - pt[0], o1 = (float)iy * dx - pt[1], o2 = (float)iz * dx - pt[2];
                float set[3];
                int write = 0;
                if (col->kind == 2) {
                    const float dp = o0 * nr[0] + o1 * nr[1] + o2 * nr[2];
                    if (fabsf(dp) <= thr) {
                        write = act || reset_plane;
                        for (int c = 0; c < 3; ++c) set[c] = act ? vel[c] : 0.0f;
                    }
                } else if (col->kind == 3) {
                    if (act && o0 * o0 + o2 * o2 < rad * rad && fabsf(o1) < hei) {
                        write = 1;
                        set[0] = -vs * sinf(cth);
                        set[1] = 0.0f;
                        set[2] = vs * cosf(cth);
                    }
                } else if (col->kind == 4) {
                    if (act) {
                        const float dp = o0 * nr[0] + o1 * nr[1] + o2 * nr[2];
                        const float rl = sqrtf(o1 * o1 + o2 * o2);
                        if (fabsf(dp) < wid && rl < rad) {
                            write = 1;
                            if (rl > 0.0f) {  /* the reference divides 0 by 0 on the axis */
                                float c = (o1 * xu[1] + o2 * xu[2]) / rl;
                                c = c < -1.0f ? -1.0f : (c > 1.0f ? 1.0f : c);
                                float th = acosf(c);
                                if (o1 * yu[1] + o2 * yu[2] < 0.0f) th = -th;
                                const float sx = -rl * sinf(th) * vs, sy = rl * cosf(th) * vs;
                                for (int c2 = 0; c2 < 3; ++c2) set[c2] = sx * xu[c2] + sy * yu[c2];
                            } else {
                                set[0] = set[1] = set[2] = 0.0f;
                            }
                        }
                    } else if (reset_all) {
                        write = 1;
                        set[0] = set[1] = set[2] = 0.0f;
                    }
                } else if (col->kind == 5) {
                    if (act) {
                        if (fabsf(o0) < wid && fabsf(o1) < wid && fabsf(o2) < wid) {
                            write = 1;
                            for (int c = 0; c < 3; ++c) set[c] = vel[c];
                        }
                    } else if (reset_all) {
                        write = 1;
                        set[0] = set[1] = set[2] = 0.0f;
                    }
                } else if (col->kind == 6) {
                    if (act && sqrtf(o0 * o0 + o1 * o1 + o2 * o2) < rad) {
                        write = 1;
                        for (int c = 0; c < 3; ++c) set[c] = vel[c];
                    }
                }
                if (write)
                    for (int c = 0; c < 3; ++c) vv[c] = (real)set[c];
            }
}

/* mpm_utils.py:241-306 */
void PFX(g2p_apic_and_stress)(const OrcModel *m, int64_t np, real dt, const real *gvout,
                              real *x, real *v, real *C, real *F_trial, real *F, real *stress,
                              real *yield, int32_t *status) {
    const int n = m->n_grid;
    const real inv_dx = (real)m->inv_dx;
    int st = 0;
#pragma omp parallel for schedule(static) reduction(| : st)
    for (int64_t p = 0; p < np; ++p) {
        int base[3];
        real fx[3], w[3][3], dw[3][3];
        if (stencil(x + 3 * p, inv_dx, n, base, fx, w, dw)) {
            st |= ST_OUT_OF_DOMAIN;
            continue;
        }
        real nv[3] = {0, 0, 0}, nC[9] = {0}, nF[9] = {0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    real dpos[3] = {(real)i - fx[0], (real)j - fx[1], (real)k - fx[2]};
                    real weight = w[0][i] * w[1][j] * w[2][k];
                    const real *gv = gvout + 3 * gidx(n, base[0] + i, base[1] + j, base[2] + k);
                    for (int r = 0; r < 3; ++r) nv[r] = nv[r] + gv[r] * weight;
                    real sc = weight * inv_dx * (real)4.0;
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) nC[r * 3 + c] = nC[r * 3 + c] + gv[r] * dpos[c] * sc;
                    real dweight[3] = {dw[0][i] * w[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * w[1][j] * dw[2][k] * inv_dx};
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) nF[r * 3 + c] = nF[r * 3 + c] + gv[r] * dweight[c];
                }
        for (int r = 0; r < 3; ++r) v[3 * p + r] = nv[r];
        for (int r = 0; r < 3; ++r) x[3 * p + r] = x[3 * p + r] + dt * nv[r];
        memcpy(C + 9 * p, nC, sizeof(nC));
        real A[9];
        for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? (real)1 : (real)0) + nF[k] * dt;
        real Ft[9];
        mm3(A, F + 9 * p, Ft);
        memcpy(F_trial + 9 * p, Ft, sizeof(Ft));
        real y = yield ? yield[p] : 0;
        return_map_and_stress(m, Ft, &y, F + 9 * p, stress + 9 * p);
        if (yield) yield[p] = y;
        for (int k = 0; k < 9; ++k)
            if (!isfinite(F[9 * p + k]) || !isfinite(stress[9 * p + k])) st |= ST_NONFINITE;
    }
    if (status) *status |= st;
}

/* Whole substep in the reference's launch order (mpm_solver_warp.py:156-199).
 * Buffers are the reference's particle and grid arrays. */
typedef struct {
    real *x0, *x, *u, *v, *C, *F, *F_trial, *F_disp, *stress, *mass, *vol, *yield;
    real *grid_m, *grid_v_in, *grid_v_out;
} PFX(State);

void PFX(p2g2p)(const OrcModel *m, PFX(State) * s, int64_t np, const OrcCollider *cols, int ncol,
                double time, real dt, int nthreads_p2g, int32_t *status) {
    const int n = m->n_grid;
    const int64_t nn = (int64_t)n * n * n;
    PFX(update_x_from_u)(np, s->x0, s->u, s->x);
    PFX(zero_grid)(nn, s->grid_m, s->grid_v_in, s->grid_v_out);
    PFX(p2g_apic_stress_given)(m, np, s->x, s->v, s->C, s->stress, s->mass, s->vol, dt, s->grid_m,
                               s->grid_v_in, status, nthreads_p2g);
    PFX(grid_normalization_and_gravity)(m, dt, s->grid_m, s->grid_v_in, s->grid_v_out);
    for (int k = 0; k < ncol; ++k) {
        if (cols[k].kind == 0) PFX(collide_surface)(m, &cols[k], time, s->grid_v_out);
        else if (cols[k].kind == 1) PFX(collide_bounding_box)(m, &cols[k], time, s->grid_v_out);
        else PFX(collide_extended)(m, &cols[k], time, dt, s->grid_v_out);
    }
    PFX(g2p_apic_and_stress)(m, np, dt, s->grid_v_out, s->x, s->v, s->C, s->F_trial, s->F,
                             s->stress, s->yield, status);
    /* CFL check of mpm_solver_warp.py:188-192 as a status bit */
    real vmax = (real)(m->dx / (double)dt);
    int st = 0;
#pragma omp parallel for schedule(static) reduction(| : st)
    for (int64_t i = 0; i < 3 * np; ++i)
        if (RABS(s->v[i]) > vmax) st |= ST_CFL;
    if (status) *status |= st;
    PFX(update_u_from_x)(np, s->x, s->x0, s->u);
    PFX(update_F_disp_from_F)(np, s->F, s->F_disp);
}

/* ------------------------------------------------------------------ */
/* reduced sampled-quadrature substep, mpm_utils.py:318-471            */
/* ------------------------------------------------------------------ */

/* update_neighboring_cells (mpm_utils.py:318-335, hi = 2) and
 * update_neighboring_cells_for_grid_v (:338-351, hi = 4): mark the cells at
 * offsets -2..hi of each sample point's base cell that lie inside the grid.
 * A sample index outside [0, np) is flagged (the reference reads out of
 * bounds); a non-finite position marks nothing and is flagged. */
void PFX(update_neighboring_cells)(const OrcModel *m, int64_t ns, const int32_t *sample, int64_t np,
                                   const real *x, int hi, int32_t *mask, int32_t *status) {
    const int n = m->n_grid;
    const real inv_dx = (real)m->inv_dx;
    int st = 0;
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t p = sample[s];
        if (p < 0 || p >= np) {
            st |= ST_BAD_INPUT;
            continue;
        }
        int base[3], skip = 0;
        for (int d = 0; d < 3; ++d) {
            real t = x[3 * p + d] * inv_dx - (real)0.5;
            if (!(t > (real)-8 && t < (real)(n + 8))) { /* no offset lands inside */
                if (t != t) st |= ST_OUT_OF_DOMAIN;
                skip = 1;
                break;
            }
            base[d] = (int)t; /* wp.int truncates toward zero */
        }
        if (skip) continue;
        for (int i = -2; i <= hi; ++i)
            for (int j = -2; j <= hi; ++j)
                for (int k = -2; k <= hi; ++k) {
                    int ix = base[0] + i, iy = base[1] + j, iz = base[2] + k;
                    if (0 <= ix && ix < n && 0 <= iy && iy < n && 0 <= iz && iz < n) mask[gidx(n, ix, iy, iz)] = 1;
                }
    }
    if (status) *status |= st;
}

/* p2g_sample_all (mpm_utils.py:353-402); nthreads == 1 scatters sequentially
 * in particle order, more threads with atomics.  A particle whose base cell is marked sets F = F_disp + I, takes the
 * FCR (jelly, metal) or Drucker-Prager (sand) stress of that F with
 * J = s0 s1 s2, and scatters momentum w m v, mass w m and the force
 * dt (-(m / density) stress grad w) as three separate adds per node.  A
 * base cell outside the grid (the reference reads the mark array out of
 * bounds) or a marked particle whose stencil leaves the grid is skipped and
 * flagged. */
void PFX(p2g_sample_all)(const OrcModel *m, int64_t np, const real *x, const real *v, real *F,
                         const real *F_disp, const real *mass, const real *density, const int32_t *mask,
                         real dt, real *gm, real *gvin, int32_t *status, int nthreads) {
    const int n = m->n_grid;
    const real inv_dx = (real)m->inv_dx, mu = (real)m->mu, lam = (real)m->lam;
    const int par = nthreads > 1;
    int st = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) \
    reduction(| : st) if (par)
    for (int64_t p = 0; p < np; ++p) {
        int cb[3], cell_in = 1;
        for (int d = 0; d < 3; ++d) {
            real t = x[3 * p + d] * inv_dx - (real)0.5;
            if (!(t > (real)-1 && t < (real)n)) cell_in = 0;
            else cb[d] = (int)t;
        }
        if (!cell_in) {
            st |= ST_OUT_OF_DOMAIN;
            continue;
        }
        if (mask[gidx(n, cb[0], cb[1], cb[2])] <= 0) continue;
        int base[3];
        real fx[3], w[3][3], dw[3][3];
        if (stencil(x + 3 * p, inv_dx, n, base, fx, w, dw)) {
            st |= ST_OUT_OF_DOMAIN;
            continue;
        }
        real *Fp = F + 9 * p;
        for (int k = 0; k < 9; ++k) Fp[k] = F_disp[9 * p + k] + ((k % 4 == 0) ? (real)1 : (real)0);
        real U[9], V[9], sig[3], tau[9];
        PFX(svd3)(Fp, U, sig, V);
        real J = 1;
        for (int d = 0; d < 3; ++d) J = J * sig[d];
        memset(tau, 0, sizeof(tau));
        if (m->material == 0 || m->material == 1) kirchoff_stress_FCR(Fp, U, V, J, mu, lam, tau);
        else if (m->material == 2) kirchoff_stress_drucker_prager(Fp, U, V, sig, mu, lam, tau);
        const real mp = mass[p];
        const real a = -(mp / density[p]);
        real M[9];
        for (int k = 0; k < 9; ++k) M[k] = a * tau[k];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    real weight = w[0][i] * w[1][j] * w[2][k];
                    int64_t g = gidx(n, base[0] + i, base[1] + j, base[2] + k);
                    real wm = weight * mp;
                    for (int r = 0; r < 3; ++r) add_real(&gvin[3 * g + r], wm * v[3 * p + r], par);
                    add_real(&gm[g], weight * mp, par);
                    real dweight[3] = {dw[0][i] * w[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * w[1][j] * dw[2][k] * inv_dx};
                    for (int r = 0; r < 3; ++r) {
                        real f = M[r * 3 + 0] * dweight[0];
                        f = f + M[r * 3 + 1] * dweight[1];
                        f = f + M[r * 3 + 2] * dweight[2];
                        f = f + (real)0; /* + body_force (zero) */
                        add_real(&gvin[3 * g + r], dt * f, par);
                    }
                }
    }
    if (status) *status |= st;
}

/* grid_normalization_and_gravity_sample_all (mpm_utils.py:405-413): marked
 * nodes with m > 1e-10 get v_in / m (a division) + dt g; the rest keep the
 * zero written by zero_grid. */
void PFX(grid_normalization_and_gravity_sample_all)(const OrcModel *m, real dt, const int32_t *mask,
                                                    const real *gm, const real *gvin, real *gvout) {
    const int n = m->n_grid;
    const int64_t nn = (int64_t)n * n * n;
    real gdt[3];
    for (int c = 0; c < 3; ++c) gdt[c] = dt * (real)m->gravity[c];
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < nn; ++g)
        if (mask[g] > 0 && gm[g] > (real)1e-10f)
            for (int c = 0; c < 3; ++c) gvout[3 * g + c] = gvin[3 * g + c] / gm[g] + gdt[c];
}

/* g2p_sample (mpm_utils.py:415-471): for sample s, particle p = sample[s]
 * gathers v and grad v from grid_v_out, x += dt v, F_trial = (I + dt grad v) F,
 * F = return map(F_trial) with yield_stress[s] for von Mises (the reference
 * passes the loop index, :464), u = x - x_initial, F_disp = F - I. */
void PFX(g2p_sample)(const OrcModel *m, int64_t ns, const int32_t *sample, int64_t np, real dt,
                     const real *gvout, real *x, const real *x0, real *v, real *u, real *F, real *F_disp,
                     real *yield, int32_t *status) {
    const int n = m->n_grid;
    const real inv_dx = (real)m->inv_dx, mu = (real)m->mu, lam = (real)m->lam;
    int st = 0;
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t p = sample[s];
        if (p < 0 || p >= np || (m->material == 1 && s >= np)) {
            st |= ST_BAD_INPUT;
            continue;
        }
        int base[3];
        real fx[3], w[3][3], dw[3][3];
        if (stencil(x + 3 * p, inv_dx, n, base, fx, w, dw)) {
            st |= ST_OUT_OF_DOMAIN;
            continue;
        }
        real nv[3] = {0, 0, 0}, nF[9] = {0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    real weight = w[0][i] * w[1][j] * w[2][k];
                    const real *gv = gvout + 3 * gidx(n, base[0] + i, base[1] + j, base[2] + k);
                    for (int r = 0; r < 3; ++r) nv[r] = nv[r] + gv[r] * weight;
                    real dweight[3] = {dw[0][i] * w[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * dw[1][j] * w[2][k] * inv_dx,
                                       w[0][i] * w[1][j] * dw[2][k] * inv_dx};
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) nF[r * 3 + c] = nF[r * 3 + c] + gv[r] * dweight[c];
                }
        for (int r = 0; r < 3; ++r) v[3 * p + r] = nv[r];
        for (int r = 0; r < 3; ++r) x[3 * p + r] = x[3 * p + r] + dt * nv[r];
        real A[9], Ft[9];
        for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? (real)1 : (real)0) + dt * nF[k];
        mm3(A, F + 9 * p, Ft);
        if (m->material == 1)
            von_mises_return_mapping(Ft, mu, lam, m->hardening, (real)m->xi, yield + s, F + 9 * p);
        else if (m->material == 2)
            sand_return_mapping(Ft, mu, lam, (real)m->alpha, F + 9 * p);
        else
            memcpy(F + 9 * p, Ft, sizeof(Ft));
        for (int k = 0; k < 9; ++k)
            if (!isfinite(F[9 * p + k])) st |= ST_NONFINITE;
        for (int r = 0; r < 3; ++r) u[3 * p + r] = x[3 * p + r] - x0[3 * p + r];
        for (int k = 0; k < 9; ++k) F_disp[9 * p + k] = F[9 * p + k] - ((k % 4 == 0) ? (real)1 : (real)0);
    }
    if (status) *status |= st;
}

/* p2g2p_reduced in the reference's launch order (mpm_solver_warp.py:214-227):
 * update_x_from_u, zero_grid (grids and both mark arrays), the P2G marks,
 * p2g_sample_all, the sample-all normalization, every collider.  The caller
 * advances moving colliders and time. */
void PFX(p2g2p_reduced)(const OrcModel *m, PFX(State) * s, int64_t np, const real *density, int64_t ns,
                        const int32_t *sample, int32_t *mask, int32_t *mask_v, const OrcCollider *cols,
                        int ncol, double time, real dt, int nthreads_p2g, int32_t *status) {
    const int n = m->n_grid;
    const int64_t nn = (int64_t)n * n * n;
    PFX(update_x_from_u)(np, s->x0, s->u, s->x);
    PFX(zero_grid)(nn, s->grid_m, s->grid_v_in, s->grid_v_out);
    memset(mask, 0, (size_t)nn * sizeof(int32_t));
    memset(mask_v, 0, (size_t)nn * sizeof(int32_t));
    PFX(update_neighboring_cells)(m, ns, sample, np, s->x, 2, mask, status);
    PFX(p2g_sample_all)(m, np, s->x, s->v, s->F, s->F_disp, s->mass, density, mask, dt, s->grid_m,
                        s->grid_v_in, status, nthreads_p2g);
    PFX(grid_normalization_and_gravity_sample_all)(m, dt, mask, s->grid_m, s->grid_v_in, s->grid_v_out);
    for (int k = 0; k < ncol; ++k) {
        if (cols[k].kind == 0) PFX(collide_surface)(m, &cols[k], time, s->grid_v_out);
        else if (cols[k].kind == 1) PFX(collide_bounding_box)(m, &cols[k], time, s->grid_v_out);
        else PFX(collide_extended)(m, &cols[k], time, dt, s->grid_v_out);
    }
}

int PFX(max_threads)(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
