// Surrogate stress stage: the network (mpm_mlp.cuh) replaces the SVD return
// map + Kirchhoff stress of sand particles, with an exact-invariant
// correction and a per-particle error gate; gated-out particles take the
// SVD path (return_map_stress, the reference's sand_return_mapping +
// kirchoff_stress_drucker_prager, engine_stress/mpm_utils.py:45-52, :87-112).
//
// Why the correction is exact: for Drucker-Prager in Hencky strain the
// return map keeps the trace of the log strain (it only shrinks the
// deviator) and the stress is tau = U diag(2 mu e + lam tr e) U^T.  With
// e_i = log s_i = 0.5 log(1 + beta_i), beta_i the eigenvalues of
// B = F F^T - I (closed form, no iteration), the mean stress
// (2 mu + 3 lam) tr e / 3 and the deviatoric norm (2 mu |e_hat| when
// elastic, 2 mu (|e_hat| - dgamma) on the cone) are known exactly.  Only
// the principal directions are missing: the network supplies them.  The
// plastic F update is F = exp(-dgamma N) F_trial with N the unit
// deviatoric direction (the reference's U diag(exp(e - dgamma h/|h|)) V^T
// rewritten in the spatial frame).
#include "mpm_mlp.cuh"
#include "mpm_mlp_tc.cuh"
#include "mpm_launch.h"

namespace mpm {
namespace sur {

using namespace mpm::mlp;

enum {
    ACC_ELASTIC = MPM_SUR_ELASTIC,
    ACC_PLASTIC = MPM_SUR_PLASTIC,
    FB_DOMAIN = MPM_SUR_FB_DOMAIN,
    FB_APEX = MPM_SUR_FB_APEX,
    FB_STEP = MPM_SUR_FB_STEP,
    FB_GATE = MPM_SUR_FB_GATE,
    FB_MATERIAL = MPM_SUR_FB_MATERIAL,
    kCodes = 7
};

// Poisson's ratio and friction angle (degrees) of a scene from lam, mu and
// alpha = sqrt(2/3) 2 sin(phi) / (3 - sin(phi)) (engine_stress/mpm_solver_warp.py:116)
__device__ __forceinline__ void scene_nu_phi(const MpmScene &S, float &nu, float &phi_deg) {
    nu = S.lam / (2.0f * (S.lam + S.mu));
    const float sphi = 3.0f * S.alpha / (2.0f * sqrtf(2.0f / 3.0f) + S.alpha);
    phi_deg = asinf(fminf(fmaxf(sphi, -1.0f), 1.0f)) * (180.0f / 3.14159265358979f);
}

__device__ __forceinline__ void features(const float B[6], float rho, float nu, float phi, float x[12]) {
    const float ir = 1.0f / fmaxf(rho, 1e-30f);
    x[0] = B[0] * ir; x[1] = B[1] * ir; x[2] = B[2] * ir;
    x[3] = B[1] * ir; x[4] = B[3] * ir; x[5] = B[4] * ir;
    x[6] = B[2] * ir; x[7] = B[4] * ir; x[8] = B[5] * ir;
    x[9] = (log10f(fmaxf(rho, 1e-30f)) + 2.5f) * (1.0f / 1.5f);
    x[10] = (nu - 0.3f) * 10.0f;
    x[11] = (phi - 30.0f) * 0.1f;
}

// exp(X) for symmetric X with |X| <= 0.25: Taylor series to degree 6 in
// Horner form (truncation below 0.25^7 / 7! = 1.2e-8)
__device__ __forceinline__ void exp_small(const float X[9], float E[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k) E[k] = ((k % 4 == 0) ? 1.0f : 0.0f) + X[k] * (1.0f / 6.0f);
#pragma unroll
    for (int d = 5; d >= 1; --d) {
        float T[9];
        mat_mul(X, E, T);
        const float inv = 1.0f / (float)d;
#pragma unroll
        for (int k = 0; k < 9; ++k) E[k] = ((k % 4 == 0) ? 1.0f : 0.0f) + T[k] * inv;
    }
}

// Exact part of one sand particle's stress, before the network runs: the
// domain, the regime (elastic / cone / apex / increment too large), the
// mean stress pm and the deviatoric norm dn (see the file comment).
struct Pre {
    float pm, dn, dg, xe;  // xe: Lode parameter 3 sqrt(6) det(h) / |h|^3 of the strain deviator
    float ev[3];           // eigenvalues of B = F F^T - I, largest first
    int code;              // ACC_ELASTIC / ACC_PLASTIC (tentative) or FB_*
};

__device__ __forceinline__ void pre_particle(const MpmScene &S, const MpmSurrogateConfig &cfg, const float B[6],
                                             float rho, Pre &p) {
    float nu, phi;
    scene_nu_phi(S, nu, phi);
    p.pm = p.dn = p.dg = p.xe = 0.0f;
    p.ev[0] = p.ev[1] = p.ev[2] = 0.0f;
    if (!(rho >= cfg.rho_min && rho <= cfg.rho_max && nu >= cfg.nu_min && nu <= cfg.nu_max &&
          phi >= cfg.phi_min && phi <= cfg.phi_max)) {
        p.code = FB_DOMAIN;
        return;
    }
    sym_eig3(B, p.ev);
    if (!(p.ev[2] > -0.9f)) {
        p.code = FB_DOMAIN;
        return;
    }
    const float e0 = 0.5f * log1pf(p.ev[0]), e1 = 0.5f * log1pf(p.ev[1]), e2 = 0.5f * log1pf(p.ev[2]);
    const float tr = e0 + e1 + e2;
    const float h0 = e0 - tr * (1.0f / 3.0f), h1 = e1 - tr * (1.0f / 3.0f), h2 = e2 - tr * (1.0f / 3.0f);
    const float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
    const float mu = S.mu, lam = S.lam;
    p.dg = hn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * S.alpha;
    if (p.dg <= 0.0f) {
        p.code = ACC_ELASTIC;
        p.dn = 2.0f * mu * hn;
    } else if (tr > 0.0f) {
        p.code = FB_APEX;
        return;
    } else if (!(p.dg <= cfg.dgamma_max)) {
        p.code = FB_STEP;
        return;
    } else {
        p.code = ACC_PLASTIC;
        p.dn = 2.0f * mu * (hn - p.dg);
    }
    p.pm = (2.0f * mu + 3.0f * lam) * tr * (1.0f / 3.0f);
    p.xe = hn > 0.0f ? fminf(fmaxf(7.348469228349534f * h0 * h1 * h2 / (hn * hn * hn), -1.0f), 1.0f) : 0.0f;
}

// Given the network's normalised stress y (6): the corrected stress
// tau = pm I + dn N (N the unit deviator of the network's stress), its error
// estimate, and the F update.  Returns the final outcome code; on ACC_* Fo
// and tau hold the result.
//
// Error estimate (relative to |tau|): the stress error is dn |N - N*| with N*
// the exact direction, which commutes with B and has the strain deviator's
// Lode angle.  So: the commutator |N Bd - Bd N| / |Bd| divided by the
// smaller eigenvalue gap of the unit deviator Bd (at least 0.2, the
// commutator sees rotations weighted by the gaps), and the Lode-angle
// difference / 3, both scaled by the deviatoric share w = dn / |tau|; N
// pointing against the strain deviator (<N, Bd> < 0.5 |Bd|) fails outright.
__device__ __forceinline__ int post_particle(const MpmScene &S, const MpmSurrogateConfig &cfg, const float F[9],
                                             const float B[6], float rho, const Pre &p, const float y[6],
                                             float Fo[9], float tau[9]) {
    const float sc = S.mu * rho;
    float D[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) D[k] = y[k] * sc;
    const float pt = (D[0] + D[3] + D[5]) * (1.0f / 3.0f);
    D[0] -= pt; D[3] -= pt; D[5] -= pt;
    const float dnorm = sym_norm(D);
    const float pm = p.pm, dn = p.dn;
    const float tcn = sqrtf(3.0f * pm * pm + dn * dn);  // |corrected stress|_F
    if (!(tcn > 0.0f)) return FB_GATE;
    const float w = dn / tcn;
    float err = 0.0f;
    if (!(dnorm > 1e-6f * tcn)) {
        if (w > 1e-3f) return FB_GATE;  // deviator needed but no direction given
#pragma unroll
        for (int k = 0; k < 6; ++k) D[k] = 0.0f;
    } else {
        const float inv = 1.0f / dnorm;
#pragma unroll
        for (int k = 0; k < 6; ++k) D[k] *= inv;  // unit deviatoric direction N
    }
    if (w > 1e-4f) {
        float Bd[6] = {B[0], B[1], B[2], B[3], B[4], B[5]};
        const float qb = (B[0] + B[3] + B[5]) * (1.0f / 3.0f);
        Bd[0] -= qb; Bd[3] -= qb; Bd[5] -= qb;
        const float bn = sym_norm(Bd);
        if (bn > 0.0f) {
            const float align = (D[0] * Bd[0] + D[3] * Bd[3] + D[5] * Bd[5] +
                                 2.0f * (D[1] * Bd[1] + D[2] * Bd[2] + D[4] * Bd[4])) / bn;
            if (!(align >= 0.5f)) return FB_GATE;
            float Nf[9], Bf[9], NB[9];
            sym_full(D, Nf);
            sym_full(Bd, Bf);
            mat_mul(Nf, Bf, NB);
            const float c01 = NB[1] - NB[3], c02 = NB[2] - NB[6], c12 = NB[5] - NB[7];
            const float comm = sqrtf(2.0f * (c01 * c01 + c02 * c02 + c12 * c12)) / bn;
            const float gap = fmaxf(fminf(p.ev[0] - p.ev[1], p.ev[1] - p.ev[2]) / bn, 0.2f);
            err = fmaxf(err, w * comm / gap);
        }
        const float detN = D[0] * (D[3] * D[5] - D[4] * D[4]) - D[1] * (D[1] * D[5] - D[4] * D[2]) +
                           D[2] * (D[1] * D[4] - D[3] * D[2]);
        const float xn = fminf(fmaxf(7.348469228349534f * detN, -1.0f), 1.0f);
        err = fmaxf(err, w * fabsf(acosf(xn) - acosf(p.xe)) * (1.0f / 3.0f));
    }
    if (!(err <= cfg.tol)) return FB_GATE;
    const float Tc[6] = {pm + dn * D[0], dn * D[1], dn * D[2], pm + dn * D[3], dn * D[4], pm + dn * D[5]};
    sym_full(Tc, tau);
    if (p.code == ACC_ELASTIC) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = F[k];
    } else {
        float X[9], E[9];
        sym_full(D, X);
#pragma unroll
        for (int k = 0; k < 9; ++k) X[k] *= -p.dg;
        exp_small(X, E);
        mat_mul(E, F, Fo);
    }
    return p.code;
}

// ---------------------------------------------------------------------------
// Training tuples: x (n,12), y (n,6) from F_trial, the scene and the stress
// ---------------------------------------------------------------------------
__global__ void features_kernel(MpmScene S, const float *__restrict__ F, const float *__restrict__ stress,
                                float *__restrict__ x, float *__restrict__ y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[9], B[6], xi[12];
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = F[i * 9 + k];
    left_strain(f, B);
    const float rho = sym_norm(B);
    float nu, phi;
    scene_nu_phi(S, nu, phi);
    features(B, rho, nu, phi, xi);
#pragma unroll
    for (int k = 0; k < 12; ++k) x[i * 12 + k] = xi[k];
    if (stress) {
        const float inv = 1.0f / (S.mu * fmaxf(rho, 1e-30f));
        const float *t = stress + i * 9;
        y[i * 6 + 0] = t[0] * inv;
        y[i * 6 + 1] = t[1] * inv;
        y[i * 6 + 2] = t[2] * inv;
        y[i * 6 + 3] = t[4] * inv;
        y[i * 6 + 4] = t[5] * inv;
        y[i * 6 + 5] = t[8] * inv;
    }
}

// ---------------------------------------------------------------------------
// In-step stage.  Persistent CTAs of 8 warps keep the weights in shared
// memory; a warp takes 32 consecutive sorted particles of one G2P chunk
// (all of one scene): lane = particle for the features and the epilogue,
// two m16 tiles through the tensor cores in between.
// ---------------------------------------------------------------------------
constexpr int kSurWarps = 8;
constexpr int kLDX = 24;  // bf16 row of the per-warp input tile (16 inputs + pad: conflict-free ldmatrix)

constexpr int kPreStride = 9;  // floats per lane of the saved pre-pass (odd stride: conflict-free)
struct SurWarp {
    __nv_bfloat16 x[32 * kLDX];
    float F[32 * 9];
    float y[32 * 7];
    float pre[32 * kPreStride];
};
struct SurSmem {
    WSmem w;
    SurWarp warp[kSurWarps];
};

__device__ __forceinline__ void ld_F(const PState &st, int pos, float F[9]) {
    const float4 a = ldrec(st, pos, 8), b = ldrec(st, pos, 9);
    const float f8 = recword(st, pos, rec::F8);
    F[0] = a.x; F[1] = a.y; F[2] = a.z; F[3] = a.w;
    F[4] = b.x; F[5] = b.y; F[6] = b.z; F[7] = b.w;
    F[8] = f8;
}

__device__ __forceinline__ void st_F_tau(const PState &st, int pos, const float F[9], const float t[9]) {
    recword(st, pos, rec::F8) = F[8];
    recword(st, pos, rec::TAU) = t[0];
    strec(st, pos, 6, make_float4(t[1], t[2], t[3], t[4]));
    strec(st, pos, 7, make_float4(t[5], t[6], t[7], t[8]));
    strec(st, pos, 8, make_float4(F[0], F[1], F[2], F[3]));
    strec(st, pos, 9, make_float4(F[4], F[5], F[6], F[7]));
}

// One warp, 32 particles of one sand scene (lane = particle, F of the lane
// given, `valid` false for padding lanes): exact pre-pass, then -- only if
// some lane needs it -- two m16 tiles through the network, then the per-lane
// correction and gate.  Returns the outcome code of the lane's particle.
__device__ __forceinline__ int surrogate_warp(const WSmem &w, SurWarp &sw, const MpmScene &S,
                                              const MpmSurrogateConfig &cfg, const float F[9], bool valid,
                                              float Fo[9], float tau[9]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    int code;
    {
        float B[6];
        left_strain(F, B);
        const float rho = sym_norm(B);
        Pre p;
        pre_particle(S, cfg, B, rho, p);
        code = valid ? p.code : FB_DOMAIN;
        const bool need = code == ACC_ELASTIC || code == ACC_PLASTIC;
        if (__ballot_sync(0xffffffffu, need) == 0u) return code;  // nothing for the network
        float xi[12], nu, phi;
        scene_nu_phi(S, nu, phi);
        features(B, rho, nu, phi, xi);
        float *pr = sw.pre + lane * kPreStride;
        pr[0] = p.pm; pr[1] = p.dn; pr[2] = p.dg; pr[3] = p.xe;
        pr[4] = p.ev[0]; pr[5] = p.ev[1]; pr[6] = p.ev[2];
        pr[7] = __int_as_float(code);
#pragma unroll
        for (int k = 0; k < 9; ++k) sw.F[lane * 9 + k] = F[k];
        uint32_t *xr = reinterpret_cast<uint32_t *>(sw.x + lane * kLDX);
#pragma unroll
        for (int k = 0; k < 6; ++k) xr[k] = pack_bf16(xi[2 * k], xi[2 * k + 1]);
        xr[6] = 0u;
        xr[7] = 0u;
    }
    __syncwarp();
#pragma unroll 1
    for (int mt = 0; mt < 2; ++mt) {
        uint32_t a1[1][4];
        const int r = (lane & 7) + ((lane >> 3) & 1) * 8, c = (lane >> 4) * 8;
        ldsm_x4(a1[0], sw.x + (mt * 16 + r) * kLDX + c);
        float out[2][4];
        mlp_core(w, a1, out, nullptr, 0, 0);
        // columns 0..5 live in out[0] of lanes t = 0, 1, 2
        if (t < 3) {
            const int row = mt * 16 + g;
            sw.y[row * 7 + 2 * t] = out[0][0];
            sw.y[row * 7 + 2 * t + 1] = out[0][1];
            sw.y[(row + 8) * 7 + 2 * t] = out[0][2];
            sw.y[(row + 8) * 7 + 2 * t + 1] = out[0][3];
        }
    }
    __syncwarp();
    float yv[6], Fl[9];
    Pre p;
#pragma unroll
    for (int k = 0; k < 6; ++k) yv[k] = sw.y[lane * 7 + k];
#pragma unroll
    for (int k = 0; k < 9; ++k) Fl[k] = sw.F[lane * 9 + k];
    {
        const float *pr = sw.pre + lane * kPreStride;
        p.pm = pr[0]; p.dn = pr[1]; p.dg = pr[2]; p.xe = pr[3];
        p.ev[0] = pr[4]; p.ev[1] = pr[5]; p.ev[2] = pr[6];
        p.code = __float_as_int(pr[7]);
    }
    __syncwarp();  // the tiles are refilled by the next call
    if (p.code != ACC_ELASTIC && p.code != ACC_PLASTIC) return p.code;
    float B[6];
    left_strain(Fl, B);
    return post_particle(S, cfg, Fl, B, sym_norm(B), p, yv, Fo, tau);
}

__device__ __forceinline__ void count_codes(int cnt[kCodes], int *stats) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kCodes; ++k) {
        int v = cnt[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v) atomicAdd(stats + k, v);
    }
}

// The surrogate on plain arrays of one scene: F_trial (n,9) -> F (n,9),
// stress (n,9), outcome code (n); gated-out rows take the SVD return map.
__global__ void __launch_bounds__(kSurWarps * 32, 1)
    surrogate_apply_kernel(MpmScene S, const __nv_bfloat16 *__restrict__ wts, const float *__restrict__ bias,
                           MpmSurrogateConfig cfg, const float *__restrict__ Fin, float *__restrict__ Fout,
                           float *__restrict__ tau_out, int *__restrict__ codes, int64_t n) {
    extern __shared__ __align__(16) unsigned char sur_smem_raw[];
    SurSmem &sm = *reinterpret_cast<SurSmem *>(sur_smem_raw);
    load_weights(sm.w, wts, bias);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SurWarp &sw = sm.warp[warp];
    const int64_t n_items = (n + 31) / 32;
    for (int64_t item = (int64_t)blockIdx.x * kSurWarps + warp; item < n_items;
         item += (int64_t)gridDim.x * kSurWarps) {
        const int64_t i = item * 32 + lane;
        const bool valid = i < n;
        float F[9], Fo[9], tau[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = valid ? Fin[i * 9 + k] : ((k % 4 == 0) ? 1.0f : 0.0f);
        int code = FB_MATERIAL;
        if (S.material == MPM_SAND) code = surrogate_warp(sm.w, sw, S, cfg, F, valid, Fo, tau);
        if (!valid) continue;
        if (code != ACC_ELASTIC && code != ACC_PLASTIC) {
            float yld = 0.0f;
            return_map_stress(S, F, yld, Fo, tau);
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            Fout[i * 9 + k] = Fo[k];
            tau_out[i * 9 + k] = tau[k];
        }
        codes[i] = code;
    }
}

// The in-step stage on the tcgen05 tensor cores: one CTA of 128 threads walks
// the G2P chunk list in tiles of up to 128 particles of one scene (thread =
// particle), runs the exact pre-pass, and -- if any particle of the tile
// needs it -- the network on the tile (mpm_mlp_tc.cuh), then the correction
// and gate.  A timed-out tensor-core wait raises MPM_ST_INTERNAL.
constexpr int kTcRows = mlptc::kRows;

__global__ void __launch_bounds__(mlptc::kThreads, 2)
    surrogate_tc_kernel(const MpmScene *__restrict__ scenes, PState st, Ws ws, const __nv_bfloat16 *__restrict__ wts,
                        const float *__restrict__ bias, MpmSurrogateConfig cfg, int2 *__restrict__ fallback,
                        int *__restrict__ stats, int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char tc_raw[];
    mlptc::TcSmem &s = *reinterpret_cast<mlptc::TcSmem *>(tc_raw);
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t tbase = mlptc::tc_setup(s, wts, bias);
    uint32_t phase = 0;
    bool ok = true;
    const int tpc = (ws.chunk_size + kTcRows - 1) / kTcRows;  // tiles per chunk
    const int n_items = *ws.n_chunks * tpc;
    int cnt[kCodes];
#pragma unroll
    for (int k = 0; k < kCodes; ++k) cnt[k] = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
        const int4 ch = ws.chunks[item / tpc];
        const int sub = item % tpc;
        const int count = min(ch.z - sub * kTcRows, kTcRows);
        if (ch.w < 0 || count <= 0) continue;  // CTA-uniform
        const MpmScene &S = scenes[ch.w];
        const int pos = ch.y + sub * kTcRows + tid;
        const bool valid = tid < kTcRows && tid < count && pos < ws.n;  // threads >= 128 help the network only
        float F[9], Fo[9], tau[9];
        if (valid) {
            ld_F(st, pos, F);
        } else {
#pragma unroll
            for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0f : 0.0f;
        }
        int code = FB_MATERIAL;
        if (S.material == MPM_SAND) {  // CTA-uniform: one scene per chunk
            float B[6];
            left_strain(F, B);
            const float rho = sym_norm(B);
            Pre p;
            pre_particle(S, cfg, B, rho, p);
            code = valid ? p.code : FB_DOMAIN;
            const bool need = code == ACC_ELASTIC || code == ACC_PLASTIC;
            if (__syncthreads_or(need ? 1 : 0)) {
                if (tid < kTcRows) {
                    float xi[12], nu, phi;
                    scene_nu_phi(S, nu, phi);
                    features(B, rho, nu, phi, xi);
                    mlptc::tc_store_inputs(s, xi);
                }
                float out[16];
                ok = mlptc::tc_tile_forward(s, tbase, phase, out, nullptr);
                if (!ok) break;
                if (need) {
                    const float y6[6] = {out[0], out[1], out[2], out[3], out[4], out[5]};
                    code = post_particle(S, cfg, F, B, rho, p, y6, Fo, tau);
                }
            }
        }
        const bool accepted = valid && (code == ACC_ELASTIC || code == ACC_PLASTIC);
        if (accepted) {
            float chk = 0.0f;
#pragma unroll
            for (int k = 0; k < 9; ++k) chk += fabsf(Fo[k]) + fabsf(tau[k]);
            if (!isfinite(chk)) atomicOr(status, MPM_ST_NONFINITE);
            st_F_tau(st, pos, Fo, tau);
        }
        const bool fb = valid && !accepted;
        const unsigned m = __ballot_sync(0xffffffffu, fb);
        if (m) {
            int base = 0;
            if (lane == 0) base = atomicAdd(stats + MPM_SUR_LAST_FALLBACKS, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (fb) fallback[base + __popc(m & ((1u << lane) - 1u))] = make_int2(pos, ch.w);
        }
        if (valid) {
#pragma unroll
            for (int k = 0; k < kCodes; ++k) cnt[k] += (code == k);
        }
    }
    if (!ok && tid == 0) atomicOr(status, MPM_ST_INTERNAL);
    count_codes(cnt, stats);
    mlptc::tc_teardown(s, tbase, ok, phase);
}

// SVD return map for the listed particles (the exact path)
__global__ void fallback_kernel(const MpmScene *__restrict__ scenes, PState st, const int2 *__restrict__ list,
                                const int *__restrict__ stats, int *__restrict__ status) {
    const int n = stats[MPM_SUR_LAST_FALLBACKS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int2 e = list[i];
        const MpmScene &S = scenes[e.y];
        float F[9], Fo[9], tau[9];
        ld_F(st, e.x, F);
        float yld = recword(st, e.x, rec::YLD);
        return_map_stress(S, F, yld, Fo, tau);
        float chk = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) chk += fabsf(Fo[k]) + fabsf(tau[k]);
        if (!isfinite(chk)) atomicOr(status, MPM_ST_NONFINITE);
        if (S.material == MPM_METAL && S.hardening == 1) recword(st, e.x, rec::YLD) = yld;
        st_F_tau(st, e.x, Fo, tau);
    }
}

}  // namespace sur

// both surrogate kernels use more than 48 KB of dynamic shared memory: opt in once per device
static cudaError_t surrogate_attrs() {
    static bool attr_set[64] = {false};
    const int bytes = (int)sizeof(sur::SurSmem);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(sur::surrogate_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(mlptc::TcSmem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(sur::surrogate_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    return cudaSuccess;
}

cudaError_t launch_surrogate(const Ctx &cx, const void *mlp_params, const MpmSurrogateConfig &cfg,
                             int2 *fallback, int *stats) {
    using namespace sur;
    const int bytes = (int)sizeof(mlptc::TcSmem);
    cudaError_t e = surrogate_attrs();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(stats + MPM_SUR_LAST_FALLBACKS, 0, sizeof(int), cx.stream);
    if (e != cudaSuccess) return e;
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(mlp_params);
    const float *b = reinterpret_cast<const float *>(static_cast<const char *>(mlp_params) +
                                                     (int64_t)mlp::W_COUNT * 2);
    // records live in st2 (G2P wrote the updated, sorted records there)
    const int64_t items = (int64_t)cx.ws.max_chunks * ((cx.ws.chunk_size + kTcRows - 1) / kTcRows);
    int grid = (int)(items < 2 * (int64_t)cx.num_sms ? items : 2 * (int64_t)cx.num_sms);
    if (grid < 1) grid = 1;
    surrogate_tc_kernel<<<grid, mlptc::kThreads, bytes, cx.stream>>>(cx.scenes, cx.st2, cx.ws, w, b, cfg, fallback, stats,
                                                             cx.status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int fgrid = cx.num_sms * 4;
    const int64_t fwant = ((int64_t)cx.n + 127) / 128;
    if (fwant < fgrid) fgrid = (int)(fwant > 0 ? fwant : 1);
    fallback_kernel<<<fgrid, 128, 0, cx.stream>>>(cx.scenes, cx.st2, fallback, stats, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_surrogate_apply(const MpmScene &scene, const void *mlp_params, const MpmSurrogateConfig &cfg,
                                   const float *F, float *Fo, float *tau, int *codes, int64_t n, int num_sms,
                                   cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = surrogate_attrs();
    if (e != cudaSuccess) return e;
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(mlp_params);
    const float *b = reinterpret_cast<const float *>(static_cast<const char *>(mlp_params) +
                                                     (int64_t)mlp::W_COUNT * 2);
    const int64_t items = (n + 32 * sur::kSurWarps - 1) / (32 * sur::kSurWarps);
    const int grid = (int)(items < num_sms ? items : num_sms);
    sur::surrogate_apply_kernel<<<grid, sur::kSurWarps * 32, sizeof(sur::SurSmem), stream>>>(
        scene, w, b, cfg, F, Fo, tau, codes, n);
    return cudaGetLastError();
}

cudaError_t launch_features(const MpmScene &scene, const float *F, const float *stress, float *x, float *y,
                            int64_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    sur::features_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(scene, F, stress, x, y, n);
    return cudaGetLastError();
}

}  // namespace mpm
