// Reverse mode of one substep (sand): the adjoints of G2P with its fused
// return map + Kirchhoff stress, of the grid update and of P2G.  The
// reference has no counterpart (no wp.Tape / gradient code); the forward it
// inverts is g2p_apic_and_stress + sand_return_mapping +
// kirchoff_stress_drucker_prager (engine_stress/mpm_utils.py:241-306,
// :87-112, :45-52), grid_normalization_and_gravity and the colliders
// (:229-237, engine_stress/mpm_solver_warp.py:429-449, :505-523) and
// p2g_apic_stress_given (mpm_utils.py:190-227).
//
// Preconditions (one call = one substep, newest first): the live state
// buffer holds the state BEFORE the substep, and mpm_sort, mpm_p2g and
// mpm_grid_update have run on it, so the sorted order, the grid momentum and
// mass (grid_acc) and the post-collider grid velocity (grid_v) of the
// substep are in the workspace.  Particle adjoints are indexed by the user
// particle index (uid), 36 floats each:
//   x 0-2, v 3-5, C 6-14, F 15-23, stress 24-32 (row-major), 33-35 unused.
//
// Return map derivative.  F_trial = U diag(s) V^T (the forward's own SVD);
// the returned F is U diag(g(s)) V^T and the stress U diag(t(s)) U^T, with
// g, t the Drucker-Prager map in principal space (elastic: g = s; cone:
// g = exp(e - dgamma h/|h|); apex: g = 1).  With dP = U^T dF_trial V the
// diagonal of dP drives g and t through their 3x3 Jacobians (forward-mode
// duals over s and the three material parameters); the off-diagonal part
// rotates the frames:
//   (U^T dG V)_ij = a_ij dP_ij + b_ij dP_ji,
//   a, b = [Dg_ij +- (g_i + g_j)/(s_i + s_j)] / 2,  Dg_ij = (g_i - g_j)/(s_i - s_j)
//   (U^T dtau U)_ij = Dt_ij (s_j dP_ij + s_i dP_ji) / (s_i + s_j)
// with the divided differences Dg, Dt evaluated in closed form
// (log1p/expm1 of log(s_i/s_j)), so they stay finite as s_i -> s_j.
#include "mpm_launch.h"

namespace mpm {
namespace adj {

constexpr int kAdjWords = 36;
enum { AX = 0, AV = 3, AC = 6, AF = 15, AT = 24 };

// ---------------------------------------------------------------------------
// forward-mode dual numbers over (s0, s1, s2, mu, lam, alpha)
// ---------------------------------------------------------------------------
struct D6 {
    float v;
    float d[6];
};
__device__ __forceinline__ D6 dc(float c) {
    D6 r;
    r.v = c;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = 0.0f;
    return r;
}
__device__ __forceinline__ D6 dvar(float c, int i) {
    D6 r = dc(c);
    r.d[i] = 1.0f;
    return r;
}
__device__ __forceinline__ D6 operator+(const D6 &a, const D6 &b) {
    D6 r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
__device__ __forceinline__ D6 operator-(const D6 &a, const D6 &b) {
    D6 r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
__device__ __forceinline__ D6 operator*(const D6 &a, const D6 &b) {
    D6 r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
__device__ __forceinline__ D6 operator*(float s, const D6 &a) {
    D6 r;
    r.v = s * a.v;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = s * a.d[k];
    return r;
}
__device__ __forceinline__ D6 operator/(const D6 &a, const D6 &b) {
    D6 r;
    const float inv = 1.0f / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
__device__ __forceinline__ D6 dlog(const D6 &a) {
    D6 r;
    r.v = logf(a.v);
    const float inv = 1.0f / a.v;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * inv;
    return r;
}
__device__ __forceinline__ D6 dexp(const D6 &a) {
    D6 r;
    r.v = expf(a.v);
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * r.v;
    return r;
}
__device__ __forceinline__ D6 dsqrt(const D6 &a) {
    D6 r;
    r.v = sqrtf(a.v);
    const float s = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * s;
    return r;
}

enum { REG_ELASTIC = 0, REG_APEX = 1, REG_CONE = 2 };

// sand_return_mapping + the Drucker-Prager stress in principal space
// (mpm_utils.py:87-112, :45-52): returned singular values g and principal
// stresses t, with their derivatives.  k = 1 - dgamma/|h| on the cone.
__device__ __forceinline__ int sand_principal(const float s[3], float mu, float lam, float alpha, D6 g[3],
                                              D6 t[3], float &k) {
    const D6 m = dvar(mu, 3), l = dvar(lam, 4), al = dvar(alpha, 5);
    D6 e[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = fabsf(s[i]);
        e[i] = a > 1e-14f ? dlog(dvar(a, i)) : dc(logf(1e-14f));
    }
    const D6 tr = e[0] + e[1] + e[2];
    D6 h[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) h[i] = e[i] - (1.0f / 3.0f) * tr;
    const D6 hn = dsqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    const D6 c = (3.0f * l + 2.0f * m) / (2.0f * m);
    const D6 dg = hn + c * tr * al;
    k = 1.0f;
    if (dg.v <= 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            g[i] = dvar(s[i], i);
            t[i] = 2.0f * m * e[i] + l * tr;
        }
        return REG_ELASTIC;
    }
    if (tr.v > 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            g[i] = dc(1.0f);
            t[i] = dc(0.0f);
        }
        k = 0.0f;
        return REG_APEX;
    }
    const D6 r = dg / hn;
    k = 1.0f - r.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const D6 ep = e[i] - h[i] * r;
        g[i] = dexp(ep);
        t[i] = 2.0f * m * ep + l * tr;  // sum of the returned log strains = tr
    }
    return REG_CONE;
}

// log(a/b) / (a - b) for a, b > 0, finite as a -> b
__device__ __forceinline__ float log_ratio_over_diff(float a, float b) {
    const float d = a - b;
    const float u = d / b;
    if (fabsf(u) < 1e-3f) return (1.0f - u * (0.5f - u * (1.0f / 3.0f))) / b;
    return log1pf(u) / d;
}
// expm1(x) / x, finite at 0
__device__ __forceinline__ float expm1_over(float x) {
    if (fabsf(x) < 1e-4f) return 1.0f + x * (0.5f + x * (1.0f / 6.0f));
    return expm1f(x) / x;
}

// VJP of (F_new, tau) = return_map_stress(F_trial) for sand: Fb, Tb are the
// adjoints of F_new and tau; adds the adjoint of F_trial to Ftb and of
// (mu, lam, alpha) to thb.
__device__ __forceinline__ void sand_rm_vjp(const MpmScene &S, const float Ft[9], const float Fb[9],
                                            const float Tb[9], float Ftb[9], float thb[3]) {
    Svd sv;
    svd3(Ft, sv);
    const float *U = sv.U, *V = sv.V;
    float s[3] = {fabsf(sv.s[0]), fabsf(sv.s[1]), fabsf(sv.s[2])};
    D6 g[3], t[3];
    float k;
    const int reg = sand_principal(s, S.mu, S.lam, S.alpha, g, t, k);
    // adjoints in the singular frames: Abar = U^T Fb V, Tbar = U^T Tb U
    float UtF[9], Ab[9], UtT[9], Tbr[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            UtF[i * 3 + c] = U[0 * 3 + i] * Fb[0 * 3 + c] + U[1 * 3 + i] * Fb[1 * 3 + c] + U[2 * 3 + i] * Fb[2 * 3 + c];
            UtT[i * 3 + c] = U[0 * 3 + i] * Tb[0 * 3 + c] + U[1 * 3 + i] * Tb[1 * 3 + c] + U[2 * 3 + i] * Tb[2 * 3 + c];
        }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Ab[i * 3 + j] = UtF[i * 3 + 0] * V[0 * 3 + j] + UtF[i * 3 + 1] * V[1 * 3 + j] + UtF[i * 3 + 2] * V[2 * 3 + j];
            Tbr[i * 3 + j] = UtT[i * 3 + 0] * U[0 * 3 + j] + UtT[i * 3 + 1] * U[1 * 3 + j] + UtT[i * 3 + 2] * U[2 * 3 + j];
        }
    float Pb[9];
    // diagonal: through the principal maps; parameters likewise
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        float acc = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) acc += Ab[i * 4] * g[i].d[m] + Tbr[i * 4] * t[i].d[m];
        Pb[m * 4] = acc;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float acc = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) acc += Ab[i * 4] * g[i].d[3 + q] + Tbr[i * 4] * t[i].d[3 + q];
        thb[q] += acc;
    }
    // off-diagonal: frame rotations
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (i == j) continue;
            const float L = log_ratio_over_diff(s[i], s[j]);
            float Dg, Dt;
            if (reg == REG_ELASTIC) {
                Dg = 1.0f;
                Dt = 2.0f * S.mu * L;
            } else if (reg == REG_APEX) {
                Dg = 0.0f;
                Dt = 0.0f;
            } else {
                const float ell = L * (s[i] - s[j]);  // log(s_i / s_j)
                Dg = g[j].v * expm1_over(k * ell) * k * L;
                Dt = 2.0f * S.mu * k * L;
            }
            const float avg = (g[i].v + g[j].v) / (s[i] + s[j]);
            const float a = 0.5f * (Dg + avg), b = 0.5f * (Dg - avg);
            Pb[i * 3 + j] = a * Ab[i * 3 + j] + b * Ab[j * 3 + i] +
                            (Tbr[i * 3 + j] + Tbr[j * 3 + i]) * Dt * s[j] / (s[i] + s[j]);
        }
    // back to the particle frame: Ftb += U Pb V^T
    float UP[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            UP[r * 3 + c] = U[r * 3 + 0] * Pb[0 * 3 + c] + U[r * 3 + 1] * Pb[1 * 3 + c] + U[r * 3 + 2] * Pb[2 * 3 + c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            Ftb[r * 3 + c] += UP[r * 3 + 0] * V[c * 3 + 0] + UP[r * 3 + 1] * V[c * 3 + 1] + UP[r * 3 + 2] * V[c * 3 + 2];
}

// second derivative of the quadratic B-spline weight wrt fx, per node offset
__device__ __forceinline__ float ddw(int node) { return node == 1 ? -2.0f : 1.0f; }

struct NodeW {
    float w;         // weight
    float dw[3];     // gradient wrt x
    float H[3][3];   // Hessian wrt x
};

__device__ __forceinline__ void node_weights(const Weights &W, int i, int j, int k, float inv_dx, NodeW &o) {
    const int nd[3] = {i, j, k};
    float a[3], da[3], dda[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        a[d] = W.w[d][nd[d]];
        da[d] = W.dw[d][nd[d]] * inv_dx;
        dda[d] = ddw(nd[d]) * inv_dx * inv_dx;
    }
    o.w = a[0] * a[1] * a[2];
    o.dw[0] = da[0] * a[1] * a[2];
    o.dw[1] = a[0] * da[1] * a[2];
    o.dw[2] = a[0] * a[1] * da[2];
    o.H[0][0] = dda[0] * a[1] * a[2];
    o.H[1][1] = a[0] * dda[1] * a[2];
    o.H[2][2] = a[0] * a[1] * dda[2];
    o.H[0][1] = o.H[1][0] = da[0] * da[1] * a[2];
    o.H[0][2] = o.H[2][0] = da[0] * a[1] * da[2];
    o.H[1][2] = o.H[2][1] = a[0] * da[1] * da[2];
}

struct PData {
    float x[3], gp[3];
    int base[3];
    bool ok;
    int uid;
};

__device__ __forceinline__ void particle_stencil(const MpmScene &S, const float *w, PData &p) {
    p.uid = __float_as_int(w[rec::UID]);
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        p.x[d] = __fadd_rn(w[rec::X0 + d], w[rec::U + d]);
        p.gp[d] = grid_coord(w[rec::X0 + d], w[rec::U + d], S.inv_dx);
        ok = stencil_base(p.gp[d], S.n_grid, p.base[d]) && ok;
    }
    p.ok = ok;
}

// ---------------------------------------------------------------------------
// G2P adjoint: thread per sorted position.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) g2p_adjoint_kernel(const MpmScene *__restrict__ scenes, int n_scenes,
                                                          PState st, Ws ws, const float *__restrict__ adj_out,
                                                          float *__restrict__ adj_in,
                                                          float4 *__restrict__ grid_adj, double *__restrict__ thb_out,
                                                          float dt) {
    float thb[3] = {0.0f, 0.0f, 0.0f};
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < ws.n; pos += gridDim.x * blockDim.x) {
        const int slot = ws.order[pos];
        // the record quads this kernel reads (x0 | uid, F8 | u | F0-7), as
        // 16-byte loads; w indexes them by record word
        float4 rq[kRecQuads];
#pragma unroll
        for (int q = 0; q < kRecQuads; ++q)
            rq[q] = (q < 3 || q >= 8) ? ldrec(st, slot, q) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float *w = reinterpret_cast<const float *>(rq);
        const int uid = __float_as_int(w[rec::UID]);
        const MpmScene &S = scenes[scene_of_particle(scenes, n_scenes, uid)];
        PData p;
        particle_stencil(S, w, p);
        const float *ao = adj_out + (int64_t)uid * kAdjWords;
        float *ai = adj_in + (int64_t)uid * kAdjWords;
        if (!p.ok) {  // out of the grid: the record is carried over unchanged, so is its adjoint
            for (int k = 0; k < kAdjWords; ++k) ai[k] = ao[k];
            continue;
        }
        if (S.material != MPM_SAND) {  // no adjoint for other materials (the API refuses them)
            for (int k = 0; k < kAdjWords; ++k) ai[k] = 0.0f;
            continue;
        }
        Weights W;
        make_weights(p.gp, p.base, W);
        const float inv_dx = S.inv_dx;
        const int nb = S.n_blocks_axis;
        // forward recompute: nv, nF (velocity gradient), F_trial
        float gv[27][3];
        float nv[3] = {0.f, 0.f, 0.f}, nF[9] = {0.f};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int q = (i * 3 + j) * 3 + k;
                    const float4 g4 = ws.grid_v[node_addr(S.block_begin, nb, p.base[0] + i, p.base[1] + j, p.base[2] + k)];
                    gv[q][0] = g4.x; gv[q][1] = g4.y; gv[q][2] = g4.z;
                    NodeW nw;
                    node_weights(W, i, j, k, inv_dx, nw);
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        nv[r] += gv[q][r] * nw.w;
#pragma unroll
                        for (int c = 0; c < 3; ++c) nF[r * 3 + c] += gv[q][r] * nw.dw[c];
                    }
                }
        float Fo[9];
        Fo[0] = w[rec::F0 + 0]; Fo[1] = w[rec::F0 + 1]; Fo[2] = w[rec::F0 + 2]; Fo[3] = w[rec::F0 + 3];
        Fo[4] = w[rec::F0 + 4]; Fo[5] = w[rec::F0 + 5]; Fo[6] = w[rec::F0 + 6]; Fo[7] = w[rec::F0 + 7];
        Fo[8] = w[rec::F8];
        float A[9], Ft[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) A[q] = ((q % 4 == 0) ? 1.0f : 0.0f) + nF[q] * dt;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                Ft[r * 3 + c] = A[r * 3 + 0] * Fo[0 * 3 + c] + A[r * 3 + 1] * Fo[1 * 3 + c] + A[r * 3 + 2] * Fo[2 * 3 + c];
        // return map adjoint
        float Fb[9], Tb[9], Ftb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            Fb[q] = ao[AF + q];
            Tb[q] = ao[AT + q];
            Ftb[q] = 0.0f;
        }
        sand_rm_vjp(S, Ft, Fb, Tb, Ftb, thb);
        // F_trial = A F: F_old adjoint A^T Ftb; nF adjoint dt Ftb F^T
        float nFb[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ai[AF + r * 3 + c] = A[0 * 3 + r] * Ftb[0 * 3 + c] + A[1 * 3 + r] * Ftb[1 * 3 + c] + A[2 * 3 + r] * Ftb[2 * 3 + c];
                nFb[r * 3 + c] = dt * (Ftb[r * 3 + 0] * Fo[c * 3 + 0] + Ftb[r * 3 + 1] * Fo[c * 3 + 1] + Ftb[r * 3 + 2] * Fo[c * 3 + 2]);
            }
        float nvb[3], nCb[9], xb[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            xb[r] = ao[AX + r];
            nvb[r] = ao[AV + r] + dt * ao[AX + r];  // x' = x + dt v', v' = nv
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) nCb[q] = ao[AC + q];
        const float c4 = 4.0f * inv_dx;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int q = (i * 3 + j) * 3 + k;
                    NodeW nw;
                    node_weights(W, i, j, k, inv_dx, nw);
                    const float dpos[3] = {(float)i - W.fx[0], (float)j - W.fx[1], (float)k - W.fx[2]};
                    const float *g = gv[q];
                    // node adjoint: nv += g w, nC += g dpos^T (4 inv_dx w), nF += g dw^T
                    float gb[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        gb[r] = nvb[r] * nw.w +
                                c4 * nw.w * (nCb[r * 3 + 0] * dpos[0] + nCb[r * 3 + 1] * dpos[1] + nCb[r * 3 + 2] * dpos[2]) +
                                nFb[r * 3 + 0] * nw.dw[0] + nFb[r * 3 + 1] * nw.dw[1] + nFb[r * 3 + 2] * nw.dw[2];
                    }
                    // one vector atomic per node (w, unused until the grid adjoint overwrites it, gets 0)
                    atomicAdd(grid_adj + node_addr(S.block_begin, nb, p.base[0] + i, p.base[1] + j, p.base[2] + k),
                              make_float4(gb[0], gb[1], gb[2], 0.0f));
                    // particle position adjoint through the weights and dpos
                    const float gvb = nvb[0] * g[0] + nvb[1] * g[1] + nvb[2] * g[2];
                    float qv[3], sv[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        qv[c] = nCb[0 * 3 + c] * g[0] + nCb[1 * 3 + c] * g[1] + nCb[2 * 3 + c] * g[2];
                        sv[c] = nFb[0 * 3 + c] * g[0] + nFb[1 * 3 + c] * g[1] + nFb[2 * 3 + c] * g[2];
                    }
                    const float qd = qv[0] * dpos[0] + qv[1] * dpos[1] + qv[2] * dpos[2];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        xb[d] += gvb * nw.dw[d] + c4 * (qd * nw.dw[d] - qv[d] * inv_dx * nw.w) +
                                 sv[0] * nw.H[0][d] + sv[1] * nw.H[1][d] + sv[2] * nw.H[2][d];
                }
#pragma unroll
        for (int d = 0; d < 3; ++d) ai[AX + d] = xb[d];  // v, C and stress adjoints: written by the P2G adjoint
    }
    // parameter adjoints: warp sums, one double atomic per warp and parameter
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float v = thb[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(thb_out + q, (double)v);
    }
}

// ---------------------------------------------------------------------------
// Grid adjoint: v = m v_in / m + dt g, then the colliders (with the same
// masks); turns the velocity adjoint into (momentum adjoint, mass adjoint).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) grid_adjoint_kernel(const MpmScene *__restrict__ scenes, int n_scenes,
                                                           Ws ws, float4 *__restrict__ grid_adj, float time,
                                                           float dt) {
    const int n_active = *ws.n_active;
    const int l = threadIdx.x & 63;
    for (int base = blockIdx.x * 4; base < n_active; base += gridDim.x * 4) {
        const int li = base + (threadIdx.x >> 6);
        if (li >= n_active) continue;
        const int gb = ws.active_list[li];
        const MpmScene &S = scenes[scene_of_block(scenes, n_scenes, gb)];
        int bx, by, bz;
        chunk_block(S, gb, bx, by, bz);
        const int ix = 4 * bx + (l >> 4), iy = 4 * by + ((l >> 2) & 3), iz = 4 * bz + (l & 3);
        const int64_t a = (int64_t)gb * kBlockNodes + l;
        const float4 acc = ws.grid_acc[a];
        const float4 vb4 = grid_adj[a];
        if (!(acc.w > 1e-15f)) {
            grid_adj[a] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        const float inv = 1.0f / acc.w;
        float v[3] = {__fadd_rn(__fmul_rn(acc.x, inv), __fmul_rn(dt, S.gravity[0])),
                      __fadd_rn(__fmul_rn(acc.y, inv), __fmul_rn(dt, S.gravity[1])),
                      __fadd_rn(__fmul_rn(acc.z, inv), __fmul_rn(dt, S.gravity[2]))};
        float keep[3] = {1.f, 1.f, 1.f};
        const int n = S.n_grid;
        for (int k = 0; k < S.n_colliders; ++k) {
            const MpmCollider &cl = S.colliders[k];
            if (!(time >= cl.start_time && time < cl.end_time)) continue;
            if (cl.kind == MPM_COLLIDER_SURFACE) {
                const float o0 = __fsub_rn(__fmul_rn((float)ix, S.dx), cl.point[0]);
                const float o1 = __fsub_rn(__fmul_rn((float)iy, S.dx), cl.point[1]);
                const float o2 = __fsub_rn(__fmul_rn((float)iz, S.dx), cl.point[2]);
                const float dp = __fadd_rn(__fadd_rn(__fmul_rn(o0, cl.normal[0]), __fmul_rn(o1, cl.normal[1])),
                                           __fmul_rn(o2, cl.normal[2]));
                if (dp < 0.0f) {
                    v[0] = v[1] = v[2] = 0.0f;
                    keep[0] = keep[1] = keep[2] = 0.0f;
                }
            } else if (cl.kind == MPM_COLLIDER_BOX) {  // (other kinds are refused by mpm_adjoint_substep)
                const int id[3] = {ix, iy, iz};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if ((id[d] < 3 && v[d] < 0.0f) || (id[d] >= n - 3 && v[d] > 0.0f)) {
                        v[d] = 0.0f;
                        keep[d] = 0.0f;
                    }
                }
            }
        }
        const float b0 = vb4.x * keep[0], b1 = vb4.y * keep[1], b2 = vb4.z * keep[2];
        const float mb = -(b0 * acc.x + b1 * acc.y + b2 * acc.z) * inv * inv;
        grid_adj[a] = make_float4(b0 * inv, b1 * inv, b2 * inv, mb);
    }
}

// ---------------------------------------------------------------------------
// P2G adjoint: thread per sorted position; gathers the node adjoints.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) p2g_adjoint_kernel(const MpmScene *__restrict__ scenes, int n_scenes,
                                                          PState st, Ws ws, const float4 *__restrict__ grid_adj,
                                                          float *__restrict__ adj_in, float dt) {
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < ws.n; pos += gridDim.x * blockDim.x) {
        const int slot = ws.order[pos];
        // record quads 0-7 (x0, m | vol, uid | u, v | C | tau) as 16-byte loads
        float4 rq[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) rq[q] = ldrec(st, slot, q);
        const float *w = reinterpret_cast<const float *>(rq);
        const int uid = __float_as_int(w[rec::UID]);
        const MpmScene &S = scenes[scene_of_particle(scenes, n_scenes, uid)];
        PData p;
        particle_stencil(S, w, p);
        if (!p.ok || S.material != MPM_SAND) continue;
        Weights W;
        make_weights(p.gp, p.base, W);
        const float inv_dx = S.inv_dx, dx = S.dx;
        const int nb = S.n_blocks_axis;
        const float m = w[rec::MASS], vol = w[rec::VOL];
        float v[3], C[9], tau[9];
#pragma unroll
        for (int r = 0; r < 3; ++r) v[r] = w[rec::V + r];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            C[q] = w[rec::C + q];
            tau[q] = w[rec::TAU + q];
        }
        float vb[3] = {0.f, 0.f, 0.f}, Cb[9] = {0.f}, Tb[9] = {0.f}, xb[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    NodeW nw;
                    node_weights(W, i, j, k, inv_dx, nw);
                    const float4 g = grid_adj[node_addr(S.block_begin, nb, p.base[0] + i, p.base[1] + j, p.base[2] + k)];
                    const float mvb[3] = {g.x, g.y, g.z};
                    const float dpos[3] = {((float)i - W.fx[0]) * dx, ((float)j - W.fx[1]) * dx, ((float)k - W.fx[2]) * dx};
                    float mom[3];  // m (v + C dpos)
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        mom[r] = m * (v[r] + C[r * 3 + 0] * dpos[0] + C[r * 3 + 1] * dpos[1] + C[r * 3 + 2] * dpos[2]);
                    const float wm = nw.w * m;
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        vb[r] += wm * mvb[r];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            Cb[r * 3 + c] += wm * mvb[r] * dpos[c];
                            Tb[r * 3 + c] += -dt * vol * mvb[r] * nw.dw[c];
                        }
                    }
                    const float s0 = mvb[0] * mom[0] + mvb[1] * mom[1] + mvb[2] * mom[2] + g.w * m;
                    float ctm[3], ttm[3];  // C^T mvb, tau^T mvb
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        ctm[c] = C[0 * 3 + c] * mvb[0] + C[1 * 3 + c] * mvb[1] + C[2 * 3 + c] * mvb[2];
                        ttm[c] = tau[0 * 3 + c] * mvb[0] + tau[1 * 3 + c] * mvb[1] + tau[2 * 3 + c] * mvb[2];
                    }
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        xb[d] += s0 * nw.dw[d] - wm * ctm[d] -
                                 dt * vol * (ttm[0] * nw.H[0][d] + ttm[1] * nw.H[1][d] + ttm[2] * nw.H[2][d]);
                }
        float *ai = adj_in + (int64_t)uid * kAdjWords;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            ai[AX + d] += xb[d];
            ai[AV + d] = vb[d];
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            ai[AC + q] = Cb[q];
            ai[AT + q] = Tb[q];
        }
    }
}

// zero the adjoint of the substep's active grid blocks
__global__ void zero_active_kernel(Ws ws, float4 *__restrict__ grid_adj) {
    const int n_active = *ws.n_active;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_active * kBlockNodes; i += gridDim.x * blockDim.x)
        grid_adj[(int64_t)ws.active_list[i / kBlockNodes] * kBlockNodes + i % kBlockNodes] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void return_map_vjp_kernel(MpmScene S, const float *__restrict__ Ft, const float *__restrict__ Fb,
                                      const float *__restrict__ Tb, float *__restrict__ Ftb,
                                      double *__restrict__ thb_out, int64_t n) {
    float thb[3] = {0.f, 0.f, 0.f};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float f[9], fb[9], tb[9], out[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            f[q] = Ft[i * 9 + q];
            fb[q] = Fb[i * 9 + q];
            tb[q] = Tb[i * 9 + q];
            out[q] = 0.0f;
        }
        sand_rm_vjp(S, f, fb, tb, out, thb);
#pragma unroll
        for (int q = 0; q < 9; ++q) Ftb[i * 9 + q] = out[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float v = thb[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(thb_out + q, (double)v);
    }
}

}  // namespace adj

cudaError_t launch_return_map_vjp(const MpmScene &scene, const float *Ft, const float *Fb, const float *Tb,
                                  float *Ftb, double *thb, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t want = (n + 127) / 128;
    adj::return_map_vjp_kernel<<<(unsigned)(want < 1216 ? want : 1216), 128, 0, st>>>(scene, Ft, Fb, Tb, Ftb,
                                                                                       thb, n);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const Ctx &cx, const float *adj_out, float *adj_in, float4 *grid_adj, double *thb,
                           float time, float dt) {
    using namespace adj;
    const int pgrid = (int)((cx.n + 127) / 128 < (int64_t)cx.num_sms * 8 ? (cx.n + 127) / 128 : cx.num_sms * 8);
    const int ggrid = (int)((cx.total_blocks + 3) / 4 < (int64_t)cx.num_sms * 8 ? (cx.total_blocks + 3) / 4
                                                                                : cx.num_sms * 8);
    if (cx.n <= 0) return cudaSuccess;
    zero_active_kernel<<<cx.num_sms * 4, 256, 0, cx.stream>>>(cx.ws, grid_adj);
    g2p_adjoint_kernel<<<pgrid, 128, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.st, cx.ws, adj_out, adj_in,
                                                     grid_adj, thb, dt);
    grid_adjoint_kernel<<<ggrid > 0 ? ggrid : 1, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws, grid_adj,
                                                                      time, dt);
    p2g_adjoint_kernel<<<pgrid, 128, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.st, cx.ws, grid_adj, adj_in, dt);
    return cudaGetLastError();
}

}  // namespace mpm
