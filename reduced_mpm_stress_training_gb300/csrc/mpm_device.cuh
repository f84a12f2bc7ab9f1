// Device-side building blocks shared by the substep kernels: buffer views,
// the stencil set-up, the 3x3 SVD, and the fused return map + Kirchhoff
// stress.  Every function here states the reference lines it follows.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mpm_gb300.h"

namespace mpm {

constexpr int kTile = 6;                // padded node tile per 4^3-cell block
constexpr int kTileNodes = kTile * kTile * kTile;  // 216
constexpr int kBlockNodes = 64;         // nodes of one 4x4x4 grid block
// one bucket per thread, 16 warps per scan tile: scan_finish's per-block cell
// scans spread over twice the warps of a 256-thread CTA with two buckets each
// (measured 34.9 -> 30.9 us per sort on the 1M column)
constexpr int kScanThreads = 512;      // threads per scan CTA
constexpr int kScanPerThread = 1;      // buckets per scan thread
constexpr int kScanTile = kScanThreads * kScanPerThread;  // buckets per scan CTA
constexpr int kSvdSweeps = 5;           // Jacobi sweeps (converged in float32)

// ---------------------------------------------------------------------------
// Views of the caller's buffers (layout fixed by mpm_plan).
// ---------------------------------------------------------------------------
// One particle-state buffer: a particle's 160-byte record (10 float4 quads)
// split over three arrays -- quads 0-3 (64 B), 4-7 (64 B) and 8-9 (32 B) per
// slot -- plus a cell-key array.  Record words (float unless noted):
//   q0:  0-2 x_initial, 3 mass                                    array a
//   q1:  4 vol, 5 uid (int bits, the user's particle index), 6 yield_stress, 7 F[8]
//   q2:  8-10 u, 11 v.x
//   q3:  12-13 v.y v.z, 14-15 C[0..1]
//   q4:  16-19 C[2..5]                                            array b
//   q5:  20-22 C[6..8], 23 stress[0]
//   q6:  24-27 stress[1..4]
//   q7:  28-31 stress[5..8]
//   q8:  32-35 F[0..3]                                            array f
//   q9:  36-39 F[4..7]
// P2G reads q0-q7: one aligned 64-byte piece of a and one of b, so DRAM moves
// exactly what it reads.  G2P reads q0, q1, q2 (one 64-byte piece of a) and
// q8, q9 (32 B of f) and writes all three.  In one 160-byte array, each
// kernel's partial reads dragged in nearly the whole record.  Matrices are
// row-major as in the reference.
constexpr int kRecWords = 40;
constexpr int kRecQuads = 10;
namespace rec {
constexpr int X0 = 0, MASS = 3, VOL = 4, UID = 5, YLD = 6, F8 = 7, U = 8, V = 11, C = 14,
              TAU = 23, F0 = 32;
}
struct PState {
    float4 *a;    // quads 0-3 of each slot (padded stride)
    float4 *b;    // quads 4-7
    float4 *f;    // quads 8-9
    int *key;     // cell key (block * 64 + cell in block) of each slot for the coming sort
    int64_t stride;
};

// address of record quad q (0..9) of a slot
__device__ __forceinline__ float4 *recq(const PState &st, int slot, int q) {
    return q < 4 ? st.a + (int64_t)slot * 4 + q
                 : (q < 8 ? st.b + (int64_t)slot * 4 + (q - 4) : st.f + (int64_t)slot * 2 + (q - 8));
}
__device__ __forceinline__ float4 ldrec(const PState &st, int slot, int q) { return *recq(st, slot, q); }
__device__ __forceinline__ void strec(const PState &st, int slot, int q, float4 v) { *recq(st, slot, q) = v; }
// record word w (0..39) of a slot
__device__ __forceinline__ float &recword(const PState &st, int slot, int w) {
    return reinterpret_cast<float *>(recq(st, slot, w >> 2))[w & 3];
}

struct Ws {  // workspace
    int *order;        // sorted position -> slot
    int *counts;       // particles per grid block (bucket), last = out of domain
    int *cell_counts;  // particles per cell (64 per block)
    int *cell_start;   // first sorted position of each cell
    int *cell_cursor;  // scatter cursor of each cell; equals the cell end afterwards
    int4 *tile_sums;  // per scan tile: (particles, chunks, non-empty blocks)
    unsigned *ticket;
    int4 *chunks;     // G2P work: (global block, start, count <= chunk_size, scene)
    int *n_chunks;
    int4 *blocks;     // P2G work: (global block, start, count, scene), one per non-empty block
    int *n_blocks;
    float4 *grid_acc; // (momentum xyz, mass), block-major
    float4 *grid_v;   // (velocity xyz, mass) after the grid update
    int *block_flag;
    int *active_list;
    int *n_active;
    int *n_active_prev;  // active blocks of the previous substep (to clear)
    float *staging;
    int *slot_of_uid;  // user particle -> slot of the live state (host transfers)
    int nbk;          // buckets = total_blocks + 1 (last = out of domain)
    int n_tiles;
    int max_chunks;
    int chunk_size;
    int n;            // particles (bounds every order[] index)
};

// ---------------------------------------------------------------------------
// Stencil set-up, engine_stress/mpm_utils.py:196-209 and :244-257.
// Explicit _rn intrinsics keep these roundings free of FMA contraction so the
// key computed at the end of G2P and the base recomputed by the next P2G are
// bit-identical (and equal to the reference's x*inv_dx, int(gp-0.5), gp-base).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float grid_coord(float x0, float u, float inv_dx) {
    return __fmul_rn(__fadd_rn(x0, u), inv_dx);  // x = x0 + u (:5-7), gp = x * inv_dx
}

// base index of one axis; returns false when the 3-node stencil would leave
// [0, n-1] or gp is NaN (the reference does not check; we flag and skip).
__device__ __forceinline__ bool stencil_base(float gp, int n, int &base) {
    float t = __fsub_rn(gp, 0.5f);
    bool ok = (t > -1.0f) && (t < (float)(n - 2));
    base = ok ? (int)t : 0;  // wp.int truncates toward zero
    return ok;
}

struct Weights {
    float w[3][3];   // w[axis][node offset]
    float dw[3][3];  // derivative wrt fx (times inv_dx gives the gradient)
    float fx[3];
};

__device__ __forceinline__ void make_weights(const float gp[3], const int base[3], Weights &W) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float fx = __fsub_rn(gp[d], (float)base[d]);
        W.fx[d] = fx;
        float wa = 1.5f - fx, wb = fx - 1.0f, wc = fx - 0.5f;
        W.w[d][0] = wa * wa * 0.5f;
        W.w[d][1] = (0.0f - wb * wb) + 0.75f;
        W.w[d][2] = wc * wc * 0.5f;
        W.dw[d][0] = fx - 1.5f;
        W.dw[d][1] = -2.0f * (fx - 1.0f);
        W.dw[d][2] = fx - 0.5f;
    }
}

// global node index in the block-major grid of one scene
__device__ __forceinline__ int64_t node_addr(int64_t block_begin, int nb, int ix, int iy, int iz) {
    int64_t blk = block_begin + ((int64_t)((ix >> 2) * nb + (iy >> 2)) * nb + (iz >> 2));
    return blk * kBlockNodes + (((ix & 3) << 4) | ((iy & 3) << 2) | (iz & 3));
}

// block coordinates (per axis, in blocks) of a global grid block of scene S
__device__ __forceinline__ void chunk_block(const MpmScene &S, int gblock, int &bx, int &by, int &bz) {
    const int nb = S.n_blocks_axis;
    int lb = (int)(gblock - S.block_begin);
    bz = lb % nb;
    by = (lb / nb) % nb;
    bx = lb / (nb * nb);
}

// scene owning a global grid block / a user-order particle (binary search)
__device__ __forceinline__ int scene_of_block(const MpmScene *sc, int n_scenes, int64_t blk) {
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sc[mid].block_begin <= blk) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int scene_of_particle(const MpmScene *sc, int n_scenes, int64_t p) {
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sc[mid].particle_begin <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// cell key of a particle position: global block id * 64 + cell within the
// block (base cell of the stencil), or sentinel_block * 64 when out of domain
__device__ __forceinline__ int particle_key(const MpmScene &S, float x0x, float x0y, float x0z,
                                            float ux, float uy, float uz, int sentinel_block,
                                            bool &ok) {
    int bx, by, bz;
    bool a = stencil_base(grid_coord(x0x, ux, S.inv_dx), S.n_grid, bx);
    bool b = stencil_base(grid_coord(x0y, uy, S.inv_dx), S.n_grid, by);
    bool c = stencil_base(grid_coord(x0z, uz, S.inv_dx), S.n_grid, bz);
    ok = a && b && c;
    const int nb = S.n_blocks_axis;
    const int blk = (int)(S.block_begin + ((int64_t)((bx >> 2) * nb + (by >> 2)) * nb + (bz >> 2)));
    const int cell = ((bx & 3) << 4) | ((by & 3) << 2) | (bz & 3);
    return ok ? blk * 64 + cell : sentinel_block * 64;
}

// warp-aggregated histogram of cell keys at block and cell level (key < 0: skip)
__device__ __forceinline__ void warp_histogram(int *counts, int *cell_counts, int key) {
    const int lane = threadIdx.x & 31;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(cell_counts + key, __popc(peers));
    const int blk = key >= 0 ? (key >> 6) : -1;
    peers = __match_any_sync(0xffffffffu, blk);
    if (blk >= 0 && lane == __ffs(peers) - 1) atomicAdd(counts + blk, __popc(peers));
}

// ---------------------------------------------------------------------------
// 3x3 SVD: Jacobi eigen-analysis of A^T A with approximate Givens rotations
// accumulated as a quaternion, sort by column norm, Givens QR (McAdams,
// Selle, Tamstorf, Teran, Sifakis 2011, UW-Madison CS TR1690), the method
// behind Warp's wp.svd3 (called at engine_stress/mpm_utils.py:64, 92, 297).
// U, V are rotations; |s| descending; sign(det A) on s[2].
// ---------------------------------------------------------------------------
struct Svd {
    float U[9], s[3], V[9];
};

// Conjugate the (p,q) block [[a,b],[b,d]] (with cross terms xp=S[p][k],
// xq=S[q][k]) by the approximate Jacobi rotation; returns its half angle.
__device__ __forceinline__ void jacobi_pair(float &a, float &d, float &b, float &xp, float &xq,
                                            float &ch, float &sh) {
    const float kGamma = 5.828427124746190f;  // 3 + 2 sqrt(2)
    const float kCstar = 0.923879532511287f;  // cos(pi/8)
    const float kSstar = 0.382683432365090f;  // sin(pi/8)
    float c0 = 2.0f * (a - d), s0 = b;
    bool small = kGamma * s0 * s0 < c0 * c0;
    float w = rsqrtf(c0 * c0 + s0 * s0);
    ch = small ? w * c0 : kCstar;
    sh = small ? w * s0 : kSstar;
    float c = ch * ch - sh * sh, s = 2.0f * ch * sh;
    float cc = c * c, ss = s * s, cs = c * s;
    float na = cc * a + 2.0f * cs * b + ss * d;
    float nd = ss * a - 2.0f * cs * b + cc * d;
    float nb = b * (cc - ss) + (d - a) * cs;
    float np = c * xp + s * xq;
    float nq = -s * xp + c * xq;
    a = na; d = nd; b = nb; xp = np; xq = nq;
}

__device__ __forceinline__ void cond_swap_neg(bool sw, float B[9], float V[9], int i, int j) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float bi = B[r * 3 + i], bj = B[r * 3 + j];
        B[r * 3 + i] = sw ? bj : bi;
        B[r * 3 + j] = sw ? -bi : bj;
        float vi = V[r * 3 + i], vj = V[r * 3 + j];
        V[r * 3 + i] = sw ? vj : vi;
        V[r * 3 + j] = sw ? -vi : vj;
    }
}

__device__ __forceinline__ void qr_givens(float B[9], float U[9], int p, int q, int col) {
    float a1 = B[p * 3 + col], a2 = B[q * 3 + col];
    float r2 = a1 * a1 + a2 * a2;
    float ri = rsqrtf(r2);
    bool nz = r2 > 0.0f;
    float c = nz ? a1 * ri : 1.0f;
    float s = nz ? a2 * ri : 0.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        float bp = B[p * 3 + j], bq = B[q * 3 + j];
        B[p * 3 + j] = c * bp + s * bq;
        B[q * 3 + j] = -s * bp + c * bq;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float up = U[r * 3 + p], uq = U[r * 3 + q];
        U[r * 3 + p] = c * up + s * uq;
        U[r * 3 + q] = -s * up + c * uq;
    }
}

__device__ __forceinline__ void svd3(const float A[9], Svd &out) {
    // S = A^T A (symmetric)
    float s00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
    float s01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
    float s02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
    float s11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
    float s12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
    float s22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
    float qw = 1.f, qx = 0.f, qy = 0.f, qz = 0.f;
#pragma unroll
    for (int sweep = 0; sweep < kSvdSweeps; ++sweep) {
        float ch, sh, w, x, y, z;
        // plane (0,1), axis z
        jacobi_pair(s00, s11, s01, s02, s12, ch, sh);
        w = qw * ch - qz * sh; x = ch * qx + qy * sh; y = ch * qy - qx * sh; z = qw * sh + ch * qz;
        qw = w; qx = x; qy = y; qz = z;
        // plane (1,2), axis x
        jacobi_pair(s11, s22, s12, s01, s02, ch, sh);
        w = qw * ch - qx * sh; x = qw * sh + ch * qx; y = ch * qy + qz * sh; z = ch * qz - qy * sh;
        qw = w; qx = x; qy = y; qz = z;
        // plane (2,0), axis y
        jacobi_pair(s22, s00, s02, s12, s01, ch, sh);
        w = qw * ch - qy * sh; x = ch * qx - qz * sh; y = qw * sh + ch * qy; z = ch * qz + qx * sh;
        qw = w; qx = x; qy = y; qz = z;
    }
    float qn = rsqrtf(qw * qw + qx * qx + qy * qy + qz * qz);
    qw *= qn; qx *= qn; qy *= qn; qz *= qn;
    float *V = out.V;
    V[0] = 1.f - 2.f * (qy * qy + qz * qz); V[1] = 2.f * (qx * qy - qw * qz); V[2] = 2.f * (qx * qz + qw * qy);
    V[3] = 2.f * (qx * qy + qw * qz); V[4] = 1.f - 2.f * (qx * qx + qz * qz); V[5] = 2.f * (qy * qz - qw * qx);
    V[6] = 2.f * (qx * qz - qw * qy); V[7] = 2.f * (qy * qz + qw * qx); V[8] = 1.f - 2.f * (qx * qx + qy * qy);
    float B[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            B[r * 3 + c] = A[r * 3 + 0] * V[0 * 3 + c] + A[r * 3 + 1] * V[1 * 3 + c] + A[r * 3 + 2] * V[2 * 3 + c];
    float r0 = B[0] * B[0] + B[3] * B[3] + B[6] * B[6];
    float r1 = B[1] * B[1] + B[4] * B[4] + B[7] * B[7];
    float r2 = B[2] * B[2] + B[5] * B[5] + B[8] * B[8];
    bool sw = r0 < r1;
    cond_swap_neg(sw, B, V, 0, 1);
    { float t = r0; r0 = sw ? r1 : r0; r1 = sw ? t : r1; }
    sw = r0 < r2;
    cond_swap_neg(sw, B, V, 0, 2);
    { float t = r0; r0 = sw ? r2 : r0; r2 = sw ? t : r2; }
    sw = r1 < r2;
    cond_swap_neg(sw, B, V, 1, 2);
    float *U = out.U;
    U[0] = 1.f; U[1] = 0.f; U[2] = 0.f; U[3] = 0.f; U[4] = 1.f; U[5] = 0.f; U[6] = 0.f; U[7] = 0.f; U[8] = 1.f;
    qr_givens(B, U, 0, 1, 0);
    qr_givens(B, U, 0, 2, 0);
    qr_givens(B, U, 1, 2, 1);
    out.s[0] = B[0];
    out.s[1] = B[4];
    out.s[2] = B[8];
}

// U diag(d) W^T
__device__ __forceinline__ void udwt(const float U[9], const float d[3], const float W[9], float out[9]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[r * 3 + c] = U[r * 3 + 0] * d[0] * W[c * 3 + 0] + U[r * 3 + 1] * d[1] * W[c * 3 + 1] +
                             U[r * 3 + 2] * d[2] * W[c * 3 + 2];
}

// symmetric 3x3 stored as (xx, xy, xz, yy, yz, zz)
__device__ __forceinline__ float sym_norm(const float S[6]) {
    return sqrtf(S[0] * S[0] + S[3] * S[3] + S[5] * S[5] + 2.0f * (S[1] * S[1] + S[2] * S[2] + S[4] * S[4]));
}
__device__ __forceinline__ void sym_full(const float S[6], float M[9]) {
    M[0] = S[0]; M[1] = S[1]; M[2] = S[2];
    M[3] = S[1]; M[4] = S[3]; M[5] = S[4];
    M[6] = S[2]; M[7] = S[4]; M[8] = S[5];
}

// B = F F^T - I through G = F - I (B = G + G^T + G G^T), so that small strains keep their digits
__device__ __forceinline__ void left_strain(const float F[9], float B[6]) {
    float G[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) G[k] = F[k] - ((k % 4 == 0) ? 1.0f : 0.0f);
    auto bij = [&](int i, int j) {
        return G[i * 3 + j] + G[j * 3 + i] + G[i * 3] * G[j * 3] + G[i * 3 + 1] * G[j * 3 + 1] +
               G[i * 3 + 2] * G[j * 3 + 2];
    };
    B[0] = bij(0, 0); B[1] = bij(0, 1); B[2] = bij(0, 2);
    B[3] = bij(1, 1); B[4] = bij(1, 2); B[5] = bij(2, 2);
}

// Eigenvalues of a symmetric 3x3 (largest first) by the closed-form
// trigonometric solution of the characteristic cubic (O. K. Smith,
// "Eigenvalues of a symmetric 3x3 matrix", CACM 4(4), 1961).
__device__ __forceinline__ void sym_eig3(const float B[6], float ev[3]) {
    const float q = (B[0] + B[3] + B[5]) * (1.0f / 3.0f);
    const float d0 = B[0] - q, d1 = B[3] - q, d2 = B[5] - q;
    const float p1 = B[1] * B[1] + B[2] * B[2] + B[4] * B[4];
    const float p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0f * p1;
    if (!(p2 > 0.0f)) {
        ev[0] = ev[1] = ev[2] = q;
        return;
    }
    const float p = sqrtf(p2 * (1.0f / 6.0f));
    const float ip = __fdividef(1.0f, p);
    const float c0 = d0 * ip, c1 = B[1] * ip, c2 = B[2] * ip, c3 = d1 * ip, c4 = B[4] * ip, c5 = d2 * ip;
    const float det = c0 * (c3 * c5 - c4 * c4) - c1 * (c1 * c5 - c4 * c2) + c2 * (c1 * c4 - c3 * c2);
    const float r = fminf(fmaxf(0.5f * det, -1.0f), 1.0f);
    const float a = acosf(r) * (1.0f / 3.0f);
    // cos(a + 2 pi / 3) = -cos(a) / 2 - sin(a) sqrt(3) / 2; a in [0, pi/3], so
    // both terms have one sign and nothing cancels
    float sa, ca;
    sincosf(a, &sa, &ca);
    ev[0] = q + 2.0f * p * ca;
    ev[2] = q - p * (ca + 1.7320508075688772f * sa);
    ev[1] = 3.0f * q - ev[0] - ev[2];
}

__device__ __forceinline__ void mat_mul(const float A[9], const float B[9], float C[9]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            C[r * 3 + c] = A[r * 3] * B[c] + A[r * 3 + 1] * B[3 + c] + A[r * 3 + 2] * B[6 + c];
}

// ---------------------------------------------------------------------------
// Sand return map + stress without an SVD.  Everything sand_return_mapping and
// kirchoff_stress_drucker_prager (engine_stress/mpm_utils.py:87-112, :45-52)
// compute is an isotropic function of the left Cauchy-Green tensor
// b = F F^T = I + B: the log strains are e_i = log s_i = log(1 + beta_i) / 2
// with beta_i the eigenvalues of B, and
//   elastic  F = F_trial,             tau = 2 mu E + lam tr(E) I,    E = e(B)
//   cone     F = exp(-r dev E) F_trial, tau = 2 mu E' + lam tr(E) I, E' = E - r dev E
//   apex     F = b^{-1/2} F_trial (the polar rotation U V^T), tau = 0
// (r = dgamma / |dev e|).  Each matrix function f(B) is evaluated in Newton
// form on the eigenvalues a, b, c (closed form, sym_eig3):
//   f(B) = f(a) I + f[a,b] (B - aI) + f[a,b,c] (B - aI)(B - bI),
// with the most isolated eigenvalue first, so that the divided differences
// divide by the large gaps only and the first-order ones of a close pair are
// taken in closed form (log1p / expm1 / square-root identities): the result
// stays accurate as eigenvalues coincide (F ~ I, the common case), where the
// Jacobi SVD path is limited by its rotation angles.  Returns false (caller
// takes the SVD path) for inverted or extremely compressed elements.
// ---------------------------------------------------------------------------
// log(x / y) / (x - y) for x, y > 0, finite as x -> y
// (x, y >= 0.01 here, so the fast divisions stay in their exact range)
__device__ __forceinline__ float log_ratio_div(float x, float y) {
    const float d = x - y;
    const float u = __fdividef(d, y);
    if (fabsf(u) < 1e-3f) return __fdividef(1.0f - u * (0.5f - u * (1.0f / 3.0f)), y);
    return __fdividef(log1pf(u), d);
}
// expm1(z) / z, finite at 0
__device__ __forceinline__ float expm1_div(float z) {
    if (fabsf(z) < 1e-4f) return 1.0f + z * (0.5f + z * (1.0f / 6.0f));
    return __fdividef(expm1f(z), z);
}

struct Newton3 {
    float a, b, c;  // nodes: isolated eigenvalue first
    float M1[6];    // B - aI
    float M2[6];    // (B - aI)(B - bI)
    bool iso0;      // nodes are (ev0, ev1, ev2) (else (ev2, ev1, ev0))
};

__device__ __forceinline__ void newton3_setup(const float B[6], const float ev[3], Newton3 &N) {
    N.iso0 = (ev[0] - ev[1]) >= (ev[1] - ev[2]);
    N.a = N.iso0 ? ev[0] : ev[2];
    N.b = ev[1];
    N.c = N.iso0 ? ev[2] : ev[0];
    // B^2 (symmetric)
    const float B2[6] = {B[0] * B[0] + B[1] * B[1] + B[2] * B[2], B[0] * B[1] + B[1] * B[3] + B[2] * B[4],
                         B[0] * B[2] + B[1] * B[4] + B[2] * B[5], B[1] * B[1] + B[3] * B[3] + B[4] * B[4],
                         B[1] * B[2] + B[3] * B[4] + B[4] * B[5], B[2] * B[2] + B[4] * B[4] + B[5] * B[5]};
    const float s = N.a + N.b, p = N.a * N.b;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float id = (k == 0 || k == 3 || k == 5) ? 1.0f : 0.0f;
        N.M1[k] = B[k] - N.a * id;
        N.M2[k] = B2[k] - s * B[k] + p * id;
    }
}

// f(B) from f at the sorted eigenvalues (f0 >= ...) and the first divided
// differences of the sorted pairs d01 = f[ev0, ev1], d12 = f[ev1, ev2]
__device__ __forceinline__ void newton3_eval(const Newton3 &N, float f0, float f2, float d01, float d12,
                                             float out[6]) {
    const float fa = N.iso0 ? f0 : f2;
    const float dab = N.iso0 ? d01 : d12;
    const float dbc = N.iso0 ? d12 : d01;
    const float den = N.c - N.a;
    const float d2 = fabsf(den) > 1e-30f ? __fdividef(dbc - dab, den) : 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float id = (k == 0 || k == 3 || k == 5) ? 1.0f : 0.0f;
        out[k] = fa * id + dab * N.M1[k] + d2 * N.M2[k];
    }
}

__device__ __forceinline__ void sym_times(const float S[6], const float A[9], float out[9]) {
    float Sf[9];
    sym_full(S, Sf);
    mat_mul(Sf, A, out);
}

__device__ __forceinline__ bool sand_return_map_spectral(const MpmScene &S, const float Ft[9], float Fo[9],
                                                         float tau[9]) {
    const float J = Ft[0] * (Ft[4] * Ft[8] - Ft[5] * Ft[7]) - Ft[1] * (Ft[3] * Ft[8] - Ft[5] * Ft[6]) +
                    Ft[2] * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
    if (!(J > 0.0f)) return false;
    float B[6], ev[3];
    left_strain(Ft, B);
    sym_eig3(B, ev);
    if (!(ev[2] > -0.99f)) return false;  // smallest singular value below 0.1
    const float mu = S.mu, lam = S.lam;
    const float e0 = 0.5f * log1pf(ev[0]), e1 = 0.5f * log1pf(ev[1]), e2 = 0.5f * log1pf(ev[2]);
    const float tr = e0 + e1 + e2;
    const float tr3 = tr * (1.0f / 3.0f);
    const float h0 = e0 - tr3, h1 = e1 - tr3, h2 = e2 - tr3;
    const float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
    const float dg = hn + __fdividef(3.0f * lam + 2.0f * mu, 2.0f * mu) * tr * S.alpha;
    Newton3 N;
    newton3_setup(B, ev, N);
    const float q0 = 1.0f + ev[0], q1 = 1.0f + ev[1], q2 = 1.0f + ev[2];
    if (dg > 0.0f && tr > 0.0f) {
        // apex: F = b^{-1/2} F_trial, s(beta) = (1 + beta)^{-1/2},
        // s[x, y] = -s(x) s(y) / (sqrt(1 + x) + sqrt(1 + y))
        const float s0 = rsqrtf(q0), s1 = rsqrtf(q1), s2 = rsqrtf(q2);
        const float d01 = -s0 * s1 / (q0 * s0 + q1 * s1);
        const float d12 = -s1 * s2 / (q1 * s1 + q2 * s2);
        float Sm[6];
        newton3_eval(N, s0, s2, d01, d12, Sm);
        sym_times(Sm, Ft, Fo);
#pragma unroll
        for (int k = 0; k < 9; ++k) tau[k] = 0.0f;
        return true;
    }
    // E = e(B), e(beta) = log(1 + beta) / 2
    const float l01 = 0.5f * log_ratio_div(q0, q1), l12 = 0.5f * log_ratio_div(q1, q2);
    float E[6];
    newton3_eval(N, e0, e2, l01, l12, E);
    float T[6];
    if (dg <= 0.0f) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = Ft[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) T[k] = 2.0f * mu * E[k] + ((k == 0 || k == 3 || k == 5) ? lam * tr : 0.0f);
    } else {
        // cone: E' = E - r (E - tr/3 I); F = exp(-r (E - tr/3 I)) F_trial,
        // g(beta) = exp(-r (e(beta) - tr/3)), g[x, y] = g(y) expm1(-r (e(x) - e(y))) / (x - y)
        const float r = __fdividef(dg, hn);  // hn >= dg > 0 on the cone (tr <= 0)
        const float g0 = expf(-r * h0), g1 = expf(-r * h1), g2 = expf(-r * h2);
        const float z01 = -r * l01, z12 = -r * l12;  // (e(x) - e(y)) = l (x - y)
        const float dg01 = g1 * z01 * expm1_div(z01 * (ev[0] - ev[1]));
        const float dg12 = g2 * z12 * expm1_div(z12 * (ev[1] - ev[2]));
        float Gm[6];
        newton3_eval(N, g0, g2, dg01, dg12, Gm);
        sym_times(Gm, Ft, Fo);
        const float k1 = 1.0f - r, k0 = r * tr3;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float id = (k == 0 || k == 3 || k == 5) ? 1.0f : 0.0f;
            T[k] = 2.0f * mu * (k1 * E[k] + k0 * id) + lam * tr * id;
        }
    }
    sym_full(T, tau);
    return true;
}

// ---------------------------------------------------------------------------
// von Mises return map + StVK-Hencky stress without an SVD
// (von_mises_return_mapping, engine_stress/mpm_utils.py:59-84, then
// kirchoff_stress_StVK on the returned F, :36-43 via :301-302).  With
// e_i = log s_i and h = e - tr(e)/3 (E = log(b)/2 as a matrix, b = F F^T):
//   plastic iff |2 mu h| > yield;  r = dgamma / (|h| + 1e-6),
//   dgamma = |h| + 1e-6 - yield / (2 mu)   (the reference's 1e-6 included)
//   F = exp(-r dev E) F_trial  (= U exp(e - r h) V^T), else F = F_trial
//   tau = U diag(2 mu e' + lam tr e') V^T = T R,  T = 2 mu E' + lam tr(E) I,
//   R = U V^T = b^{-1/2} F_trial (the polar rotation, unchanged by the return)
// so everything is a function of b evaluated in Newton form (as for sand),
// plus R.  Returns false (SVD path) for inverted or extremely compressed
// elements, where the reference's 0.01 clamp of the singular values matters.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool metal_return_map_spectral(const MpmScene &S, const float Ft[9], float &yld,
                                                          float Fo[9], float tau[9]) {
    const float J = Ft[0] * (Ft[4] * Ft[8] - Ft[5] * Ft[7]) - Ft[1] * (Ft[3] * Ft[8] - Ft[5] * Ft[6]) +
                    Ft[2] * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
    if (!(J > 0.0f)) return false;
    float B[6], ev[3];
    left_strain(Ft, B);
    sym_eig3(B, ev);
    if (!(ev[2] > -0.99f)) return false;  // smallest singular value below 0.1
    const float mu = S.mu, lam = S.lam;
    const float e0 = 0.5f * log1pf(ev[0]), e1 = 0.5f * log1pf(ev[1]), e2 = 0.5f * log1pf(ev[2]);
    const float tr = e0 + e1 + e2;
    const float h0 = e0 - tr / 3.0f, h1 = e1 - tr / 3.0f, h2 = e2 - tr / 3.0f;
    const float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
    Newton3 N;
    newton3_setup(B, ev, N);
    const float q0 = 1.0f + ev[0], q1 = 1.0f + ev[1], q2 = 1.0f + ev[2];
    // R = b^{-1/2} F_trial: s(beta) = (1 + beta)^{-1/2}
    const float s0 = rsqrtf(q0), s1 = rsqrtf(q1), s2 = rsqrtf(q2);
    float Sm[6], R[9];
    newton3_eval(N, s0, s2, -s0 * s1 / (q0 * s0 + q1 * s1), -s1 * s2 / (q1 * s1 + q2 * s2), Sm);
    sym_times(Sm, Ft, R);
    const float l01 = 0.5f * log_ratio_div(q0, q1), l12 = 0.5f * log_ratio_div(q1, q2);
    float E[6];
    newton3_eval(N, e0, e2, l01, l12, E);
    float T[6];
    if (2.0f * mu * hn > yld) {
        const float hn_eps = hn + 1e-6f;
        const float dg = hn_eps - yld / (2.0f * mu);
        const float r = dg / hn_eps;
        const float g0 = expf(-r * h0), g1 = expf(-r * h1), g2 = expf(-r * h2);
        const float z01 = -r * l01, z12 = -r * l12;
        const float dg01 = g1 * z01 * expm1_div(z01 * (ev[0] - ev[1]));
        const float dg12 = g2 * z12 * expm1_div(z12 * (ev[1] - ev[2]));
        float Gm[6];
        newton3_eval(N, g0, g2, dg01, dg12, Gm);
        sym_times(Gm, Ft, Fo);
        const float k1 = 1.0f - r, k0 = r * tr / 3.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float id = (k == 0 || k == 3 || k == 5) ? 1.0f : 0.0f;
            T[k] = 2.0f * mu * (k1 * E[k] + k0 * id) + lam * tr * id;
        }
        if (S.hardening == 1) yld = yld + 2.0f * mu * S.xi * dg;
    } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = Ft[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) T[k] = 2.0f * mu * E[k] + ((k == 0 || k == 3 || k == 5) ? lam * tr : 0.0f);
    }
    sym_times(T, R, tau);
    return true;
}

// ---------------------------------------------------------------------------
// Fixed-corotated stress without an SVD (kirchoff_stress_FCR,
// engine_stress/mpm_utils.py:29-34, jelly, F = F_trial):
//   tau = 2 mu (F - R) F^T + lam J (J - 1) I,   R = U V^T,
// and (F - R) F^T = b - b^{1/2} = f(B), f(beta) = (1 + beta) - sqrt(1 + beta)
// = sqrt(1 + beta) beta / (1 + sqrt(1 + beta)),  f[x, y] = 1 - 1 / (sqrt(1 + x)
// + sqrt(1 + y)): accurate as B -> 0.  J = det F as in the reference.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool jelly_stress_spectral(const MpmScene &S, const float Ft[9], float Fo[9],
                                                      float tau[9]) {
    const float J = Ft[0] * (Ft[4] * Ft[8] - Ft[5] * Ft[7]) - Ft[1] * (Ft[3] * Ft[8] - Ft[5] * Ft[6]) +
                    Ft[2] * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
    if (!(J > 0.0f)) return false;
    float B[6], ev[3];
    left_strain(Ft, B);
    sym_eig3(B, ev);
    if (!(ev[2] > -0.99f)) return false;
    Newton3 N;
    newton3_setup(B, ev, N);
    const float r0 = sqrtf(1.0f + ev[0]), r1 = sqrtf(1.0f + ev[1]), r2 = sqrtf(1.0f + ev[2]);
    const float f0 = r0 * ev[0] / (1.0f + r0), f2 = r2 * ev[2] / (1.0f + r2);
    const float d01 = 1.0f - 1.0f / (r0 + r1), d12 = 1.0f - 1.0f / (r1 + r2);
    float Fm[6];
    newton3_eval(N, f0, f2, d01, d12, Fm);
    const float dia = S.lam * J * (J - 1.0f);
#pragma unroll
    for (int k = 0; k < 9; ++k) Fo[k] = Ft[k];
    float T[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) T[k] = 2.0f * S.mu * Fm[k] + ((k == 0 || k == 3 || k == 5) ? dia : 0.0f);
    sym_full(T, tau);
    return true;
}

// ---------------------------------------------------------------------------
// Return mapping + Kirchhoff stress for one particle, fused on ONE SVD.
// The reference (g2p_apic_and_stress, engine_stress/mpm_utils.py:284-306)
// takes a second SVD of the returned F for the stress.  The returned F is
// either F_trial itself (whose SVD is the first one, exactly) or
// U diag(s_new) V^T, whose SVD is (U, s_new, V); so the first factors are
// reused, and  U diag(c) V^T F^T = U diag(c * s_new) U^T  for the
// Drucker-Prager stress (:45-52).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void return_map_stress(const MpmScene &S, const float Ft[9], float &yld,
                                                  float Fo[9], float tau[9]) {
    if (S.material == MPM_SAND && sand_return_map_spectral(S, Ft, Fo, tau)) return;
    if (S.material == MPM_METAL && metal_return_map_spectral(S, Ft, yld, Fo, tau)) return;
    if (S.material == MPM_JELLY && jelly_stress_spectral(S, Ft, Fo, tau)) return;
    Svd d;
    svd3(Ft, d);
    const float mu = S.mu, lam = S.lam;
    if (S.material == MPM_SAND) {
        // sand_return_mapping, mpm_utils.py:87-112
        float e0 = logf(fmaxf(fabsf(d.s[0]), 1e-14f));
        float e1 = logf(fmaxf(fabsf(d.s[1]), 1e-14f));
        float e2 = logf(fmaxf(fabsf(d.s[2]), 1e-14f));
        float tr = e0 + e1 + e2;
        float h0 = e0 - tr / 3.0f, h1 = e1 - tr / 3.0f, h2 = e2 - tr / 3.0f;
        float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
        float dg = hn + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * S.alpha;
        float sn[3];
        if (dg <= 0.0f) {
#pragma unroll
            for (int i = 0; i < 9; ++i) Fo[i] = Ft[i];
            sn[0] = d.s[0]; sn[1] = d.s[1]; sn[2] = d.s[2];
        } else if (tr > 0.0f) {
            sn[0] = sn[1] = sn[2] = 1.0f;
            udwt(d.U, sn, d.V, Fo);
        } else {
            float r = dg / hn;
            sn[0] = expf(e0 - h0 * r);
            sn[1] = expf(e1 - h1 * r);
            sn[2] = expf(e2 - h2 * r);
            udwt(d.U, sn, d.V, Fo);
        }
        // kirchoff_stress_drucker_prager, mpm_utils.py:45-52 (unclamped log)
        float l0 = logf(sn[0]), l1 = logf(sn[1]), l2 = logf(sn[2]);
        float ls = l0 + l1 + l2;
        float t[3] = {2.0f * mu * l0 + lam * ls, 2.0f * mu * l1 + lam * ls, 2.0f * mu * l2 + lam * ls};
        udwt(d.U, t, d.U, tau);
    } else if (S.material == MPM_METAL) {
        // von_mises_return_mapping, mpm_utils.py:59-84
        float c0 = fmaxf(d.s[0], 0.01f), c1 = fmaxf(d.s[1], 0.01f), c2 = fmaxf(d.s[2], 0.01f);
        float e0 = logf(c0), e1 = logf(c1), e2 = logf(c2);
        float es = e0 + e1 + e2;
        float temp = es / 3.0f;
        float t0 = 2.0f * mu * e0 + lam * es, t1 = 2.0f * mu * e1 + lam * es, t2 = 2.0f * mu * e2 + lam * es;
        float st = t0 + t1 + t2;
        float k0 = t0 - st / 3.0f, k1 = t1 - st / 3.0f, k2 = t2 - st / 3.0f;
        float sn[3];
        if (sqrtf(k0 * k0 + k1 * k1 + k2 * k2) > yld) {
            float h0 = e0 - temp, h1 = e1 - temp, h2 = e2 - temp;
            float hn = sqrtf(h0 * h0 + h1 * h1 + h2 * h2) + 1e-6f;
            float dg = hn - yld / (2.0f * mu);
            float r = dg / hn;
            sn[0] = expf(e0 - r * h0);
            sn[1] = expf(e1 - r * h1);
            sn[2] = expf(e2 - r * h2);
            udwt(d.U, sn, d.V, Fo);
            if (S.hardening == 1) yld = yld + 2.0f * mu * S.xi * dg;
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) Fo[i] = Ft[i];
            sn[0] = d.s[0]; sn[1] = d.s[1]; sn[2] = d.s[2];
        }
        // kirchoff_stress_StVK, mpm_utils.py:36-43: U diag(2 mu eps + lam tr eps) V^T
        float l0 = logf(fmaxf(sn[0], 0.01f)), l1 = logf(fmaxf(sn[1], 0.01f)), l2 = logf(fmaxf(sn[2], 0.01f));
        float ls = l0 + l1 + l2;
        float t[3] = {2.0f * mu * l0 + lam * ls, 2.0f * mu * l1 + lam * ls, 2.0f * mu * l2 + lam * ls};
        udwt(d.U, t, d.V, tau);
    } else {
        // jelly: F = F_trial, kirchoff_stress_FCR (mpm_utils.py:29-34)
#pragma unroll
        for (int i = 0; i < 9; ++i) Fo[i] = Ft[i];
        float J = Ft[0] * (Ft[4] * Ft[8] - Ft[5] * Ft[7]) - Ft[1] * (Ft[3] * Ft[8] - Ft[5] * Ft[6]) +
                  Ft[2] * (Ft[3] * Ft[7] - Ft[4] * Ft[6]);
        float one[3] = {1.f, 1.f, 1.f};
        float R[9];
        udwt(d.U, one, d.V, R);
        float D[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = 2.0f * mu * (Ft[i] - R[i]);
        float dia = lam * J * (J - 1.0f);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                tau[r * 3 + c] = D[r * 3 + 0] * Ft[c * 3 + 0] + D[r * 3 + 1] * Ft[c * 3 + 1] +
                                 D[r * 3 + 2] * Ft[c * 3 + 2] + (r == c ? dia : 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Colliders: the reference's grid_postprocess kernels
// (engine_stress/mpm_solver_warp.py:407-720), one per collider kind, applied
// in registration order to the node velocity after normalization + gravity.
// The reference sweeps the dense grid; in the substep, nodes outside the
// active blocks carry no mass and are never gathered, so the active blocks are
// enough (the reduced substep sweeps its dense grid as the reference does).  Node
// offsets and dot products use explicitly rounded float32 operations (no FMA
// contraction) so inside/outside decisions match a float32 restatement.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float dot3_rn(float a0, float a1, float a2, const float b[3]) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b[0]), __fmul_rn(a1, b[1])), __fmul_rn(a2, b[2]));
}

// rotation angle of the circling column's centre about (0.5, *, 0.5), from
// its bottom point (set_column_moving_as_circle, :585-592 and :597-603)
__device__ __forceinline__ float circle_theta(const float p[3]) {
    const float z0 = __fsub_rn(p[0], 0.5f), z1 = p[1], z2 = __fsub_rn(p[2], 0.5f);
    const float len = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(z0, z0), __fmul_rn(z1, z1)), __fmul_rn(z2, z2)));
    const float c = __fdiv_rn(z0, len);
    const float th = acosf(fminf(fmaxf(c, -1.0f), 1.0f));
    return z2 < 0.0f ? -th : th;
}

__device__ __forceinline__ void apply_collider(const MpmCollider &cl, const MpmScene &S, int ix, int iy, int iz,
                                               float time, float dt, float v[3]) {
    const bool active = time >= cl.start_time && time < cl.end_time;
    const float o0 = __fsub_rn(__fmul_rn((float)ix, S.dx), cl.point[0]);
    const float o1 = __fsub_rn(__fmul_rn((float)iy, S.dx), cl.point[1]);
    const float o2 = __fsub_rn(__fmul_rn((float)iz, S.dx), cl.point[2]);
    switch (cl.kind) {
        case MPM_COLLIDER_SURFACE:  // :429-449: every surface type writes zero
            if (active && dot3_rn(o0, o1, o2, cl.normal) < 0.0f) v[0] = v[1] = v[2] = 0.0f;
            break;
        case MPM_COLLIDER_BOX: {  // :505-523, padding 3
            if (!active) break;
            const int id[3] = {ix, iy, iz};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (id[d] < 3 && v[d] < 0.0f) v[d] = 0.0f;
                if (id[d] >= S.n_grid - 3 && v[d] > 0.0f) v[d] = 0.0f;
            }
            break;
        }
        case MPM_COLLIDER_VPLANE: {  // :545-559: the slab |(x - p).n| <= threshold moves with velocity
            const bool in = fabsf(dot3_rn(o0, o1, o2, cl.normal)) <= cl.threshold;
            if (active) {
                if (in) v[0] = cl.velocity[0], v[1] = cl.velocity[1], v[2] = cl.velocity[2];
            } else if (cl.reset == 1 && time < __fadd_rn(cl.end_time, __fmul_rn(__fmul_rn(1.5f, dt), 10.0f))) {
                if (in) v[0] = v[1] = v[2] = 0.0f;
            }
            break;
        }
        case MPM_COLLIDER_CIRCLE: {  // :580-592: a vertical column circling about (0.5, *, 0.5)
            if (!active) break;
            if (__fadd_rn(__fmul_rn(o0, o0), __fmul_rn(o2, o2)) < __fmul_rn(cl.radius, cl.radius) &&
                fabsf(o1) < cl.height) {
                const float th = circle_theta(cl.point);
                v[0] = -cl.v_scale * sinf(th);
                v[1] = 0.0f;
                v[2] = cl.v_scale * cosf(th);
            }
            break;
        }
        case MPM_COLLIDER_DISK: {  // :635-659: rigid rotation of a disk about its normal
            if (active) {
                if (fabsf(dot3_rn(o0, o1, o2, cl.normal)) < cl.width) {
                    // the reference takes r = (0, o_y, o_z), not the in-plane projection
                    const float rl = sqrtf(__fadd_rn(__fmul_rn(o1, o1), __fmul_rn(o2, o2)));
                    if (rl < cl.radius) {
                        if (rl > 0.0f) {  // on the axis the reference divides 0 by 0 (NaN); here v = 0
                            const float c = __fdiv_rn(dot3_rn(0.0f, o1, o2, cl.x_unit), rl);
                            float th = acosf(fminf(fmaxf(c, -1.0f), 1.0f));
                            if (dot3_rn(0.0f, o1, o2, cl.y_unit) < 0.0f) th = -th;
                            const float sx = -rl * sinf(th) * cl.v_scale, sy = rl * cosf(th) * cl.v_scale;
#pragma unroll
                            for (int d = 0; d < 3; ++d) v[d] = sx * cl.x_unit[d] + sy * cl.y_unit[d];
                        } else {
                            v[0] = v[1] = v[2] = 0.0f;
                        }
                    }
                }
            } else if (cl.reset == 1 && time < __fadd_rn(cl.end_time, __fmul_rn(1.5f, dt))) {
                v[0] = v[1] = v[2] = 0.0f;  // every node, as the reference does
            }
            break;
        }
        case MPM_COLLIDER_CUBE: {  // :680-689
            if (active) {
                if (fabsf(o0) < cl.width && fabsf(o1) < cl.width && fabsf(o2) < cl.width)
                    v[0] = cl.velocity[0], v[1] = cl.velocity[1], v[2] = cl.velocity[2];
            } else if (cl.reset == 1 && time < __fadd_rn(cl.end_time, __fmul_rn(1.5f, dt))) {
                v[0] = v[1] = v[2] = 0.0f;  // every node, as the reference does
            }
            break;
        }
        case MPM_COLLIDER_SPHERE: {  // :709-714
            if (!active) break;
            const float len = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(o0, o0), __fmul_rn(o1, o1)), __fmul_rn(o2, o2)));
            if (len < cl.radius) v[0] = cl.velocity[0], v[1] = cl.velocity[1], v[2] = cl.velocity[2];
            break;
        }
        default:
            break;
    }
}

}  // namespace mpm
