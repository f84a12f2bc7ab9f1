// Reduced sampled-quadrature substep: MPM_Simulator_WARP.p2g2p_reduced
// (engine_stress/mpm_solver_warp.py:214-227), experiment_for_C (:207-209)
// and the sample-point gather g2p_sample (engine_stress/mpm_utils.py:415-471).
//
// The product of this path is the reference's dense (n, n, n) grid itself,
// so it keeps that layout (C-order, vec3 AoS) for grid_m / grid_v_in /
// grid_v_out and the two int32 mark arrays.  Momentum and mass are
// accumulated with one 16-byte vector atomic per node into a float4 scratch
// grid (the reference issues seven scalar atomics per node), and a single
// sweep then normalizes, applies gravity and every collider, and writes the
// three reference-layout grids.  Particles are read from the cell-sorted
// state records; the user-order side arrays (F_disp, density) and the
// sample list are indexed through the particle's uid.
#include "mpm_launch.h"

namespace mpm {

namespace {

__device__ __forceinline__ int64_t dense_index(int n, int ix, int iy, int iz) {
    return ((int64_t)ix * n + iy) * n + iz;
}

// grid position of a particle record: x = x_initial + u, gp = x * inv_dx
__device__ __forceinline__ void record_gp(const PState &st, int slot, float inv_dx, float gp[3]) {
    const float4 q0 = ldrec(st, slot, 0), q2 = ldrec(st, slot, 2);
    gp[0] = grid_coord(q0.x, q2.x, inv_dx);
    gp[1] = grid_coord(q0.y, q2.y, inv_dx);
    gp[2] = grid_coord(q0.z, q2.z, inv_dx);
}

// kirchoff_stress_FCR (mpm_utils.py:29-34): 2 mu (F - R) F^T + lam J (J - 1) I, R = U V^T
__device__ __forceinline__ void stress_fcr(const float F[9], const Svd &d, float J, float mu, float lam,
                                           float tau[9]) {
    const float one[3] = {1.f, 1.f, 1.f};
    float R[9], D[9];
    udwt(d.U, one, d.V, R);
    const float tm = 2.0f * mu;
#pragma unroll
    for (int i = 0; i < 9; ++i) D[i] = tm * (F[i] - R[i]);
    const float dia = lam * J * (J - 1.0f);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            tau[r * 3 + c] = D[r * 3 + 0] * F[c * 3 + 0] + D[r * 3 + 1] * F[c * 3 + 1] + D[r * 3 + 2] * F[c * 3 + 2] +
                             (r == c ? dia : 0.0f);
}

// kirchoff_stress_drucker_prager (mpm_utils.py:45-52): U diag(c) V^T F^T with
// c_i = (2 mu ln s_i + lam sum ln s) / s_i, logarithms unclamped
__device__ __forceinline__ void stress_dp(const float F[9], const Svd &d, float mu, float lam, float tau[9]) {
    const float l0 = logf(d.s[0]), l1 = logf(d.s[1]), l2 = logf(d.s[2]);
    const float ls = l0 + l1 + l2;
    const float tm = 2.0f * mu;
    const float c[3] = {tm * l0 * (1.0f / d.s[0]) + lam * ls * (1.0f / d.s[0]),
                        tm * l1 * (1.0f / d.s[1]) + lam * ls * (1.0f / d.s[1]),
                        tm * l2 * (1.0f / d.s[2]) + lam * ls * (1.0f / d.s[2])};
    float T[9];
    udwt(d.U, c, d.V, T);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int k = 0; k < 3; ++k)
            tau[r * 3 + k] = T[r * 3 + 0] * F[k * 3 + 0] + T[r * 3 + 1] * F[k * 3 + 1] + T[r * 3 + 2] * F[k * 3 + 2];
}

// the reduced kernels serve single-scene plans whose dense grid matches the scene
__device__ __forceinline__ bool grid_matches(const MpmScene &S, const MpmReducedGrid &g, int *status) {
    if (S.n_grid == g.n_grid) return true;
    if (threadIdx.x == 0) atomicOr(status, MPM_ST_BAD_INPUT);
    return false;
}

}  // namespace

// update_neighboring_cells (mpm_utils.py:318-335, offsets -2..2, HI = 2) and
// update_neighboring_cells_for_grid_v (:338-351, offsets -2..4, HI = 4): one
// warp per sample point, its lanes over the (HI + 3)^3 offsets; cells
// outside the grid are not marked, as there.
template <int HI>
__global__ void __launch_bounds__(256) mark_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                   const int *__restrict__ slot_of_uid, MpmReducedGrid g,
                                                   int32_t *__restrict__ mask, int n, int *status) {
    const MpmScene &S = scenes[0];
    if (!grid_matches(S, g, status)) return;
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= g.n_samples) return;
    const int p = g.sample_index[s];
    if (p < 0 || p >= n) {
        if (lane == 0) atomicOr(status, MPM_ST_BAD_INPUT);
        return;
    }
    const int N = g.n_grid;
    float gp[3];
    record_gp(st, slot_of_uid[p], S.inv_dx, gp);
    int b[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float t = __fsub_rn(gp[d], 0.5f);
        // beyond 8 cells outside the grid no offset lands inside; NaN marks nothing
        if (!(t > -8.0f && t < (float)(N + 8))) {
            if (lane == 0 && !(t == t)) atomicOr(status, MPM_ST_OUT_OF_DOMAIN);
            return;
        }
        b[d] = (int)t;  // wp.int truncates toward zero
    }
    constexpr int W = HI + 3;
    for (int o = lane; o < W * W * W; o += 32) {
        const int ix = b[0] + o / (W * W) - 2, iy = b[1] + (o / W) % W - 2, iz = b[2] + o % W - 2;
        if (ix >= 0 && ix < N && iy >= 0 && iy < N && iz >= 0 && iz < N) mask[dense_index(N, ix, iy, iz)] = 1;
    }
}

// p2g_sample_all (mpm_utils.py:353-402): one thread per particle record.  A
// particle whose base cell is marked sets F = F_disp + I, takes the stress of
// that F (FCR for jelly and metal, Drucker-Prager for sand; :368-378) and
// scatters, per node, w m v + dt (-(m / density) stress grad w) and w m.
// The records are sorted by cell, so neighbouring lanes mostly share a base
// cell and hit the same 27 nodes: each node's contributions are summed over
// every run of lanes with one base cell (a segmented shuffle reduction) and
// the run's first lane issues one 16-byte atomic for it.
__global__ void __launch_bounds__(256) reduced_p2g_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                          MpmReducedGrid g, int n, float dt, int *status) {
    const MpmScene &S = scenes[0];
    if (!grid_matches(S, g, status)) return;  // the same for every thread
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int N = g.n_grid;
    float gp[3] = {0.5f, 0.5f, 0.5f};
    int base[3] = {0, 0, 0};
    bool act = false;
    if (i < n) {
        record_gp(st, i, S.inv_dx, gp);
        bool cell_in = true, stencil_in = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float t = __fsub_rn(gp[d], 0.5f);
            cell_in = cell_in && t > -1.0f && t < (float)N;
            stencil_in = stencil_in && t > -1.0f && t < (float)(N - 2);
            base[d] = (t > -1.0f && t < (float)N) ? (int)t : 0;
        }
        if (!cell_in) {  // the reference reads the mark array out of bounds here
            atomicOr(status, MPM_ST_OUT_OF_DOMAIN);
        } else if (g.neighboring_cells[dense_index(N, base[0], base[1], base[2])] > 0) {
            if (stencil_in) act = true;
            else atomicOr(status, MPM_ST_OUT_OF_DOMAIN);  // marked, but the stencil would leave the grid
        }
    }
    if (__ballot_sync(0xffffffffu, act) == 0u) return;  // the whole warp leaves together
    float tau[9], v[3] = {0.f, 0.f, 0.f}, m = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) tau[k] = 0.0f;
    if (act) {
        float4 q1 = ldrec(st, i, 1);
        const float4 q0 = ldrec(st, i, 0), q2 = ldrec(st, i, 2), q3 = ldrec(st, i, 3);
        const int uid = __float_as_int(q1.y);
        const float *fd = g.f_disp + (int64_t)uid * 9;
        float F[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = __fadd_rn(fd[k], (k % 4 == 0) ? 1.0f : 0.0f);  // F_disp + I (:364)
        q1.w = F[8];
        strec(st, i, 1, q1);
        strec(st, i, 8, make_float4(F[0], F[1], F[2], F[3]));
        strec(st, i, 9, make_float4(F[4], F[5], F[6], F[7]));
        Svd d;
        svd3(F, d);
        if (S.material == MPM_SAND) {
            stress_dp(F, d, S.mu, S.lam, tau);
        } else {
            const float J = d.s[0] * d.s[1] * d.s[2];
            stress_fcr(F, d, J, S.mu, S.lam, tau);
        }
        m = q0.w;
        const float nvol = -__fdiv_rn(m, g.density[uid]);  // -(m / density), :395
#pragma unroll
        for (int k = 0; k < 9; ++k) tau[k] *= nvol;
        v[0] = q2.w;
        v[1] = q3.x;
        v[2] = q3.y;
    } else {  // contributes zeros from a finite stencil
        gp[0] = gp[1] = gp[2] = 0.5f;
        base[0] = base[1] = base[2] = 0;
    }
    // runs of lanes with one base cell (n_grid <= 1024: 10 bits per axis); idle lanes stand alone
    const int key = act ? ((base[0] << 20) | (base[1] << 10) | base[2]) : (0x40000000 | lane);
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const bool solo = heads == 0xffffffffu;  // no two lanes share a cell: plain atomics
    // lane + 2^j belongs to this lane's run when no run starts in (lane, lane + 2^j]
    bool in_run[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const int d = 1 << j;
        in_run[j] = lane + d < 32 && ((((unsigned long long)heads) >> (lane + 1)) & ((1ull << d) - 1ull)) == 0ull;
    }
    Weights W;
    make_weights(gp, base, W);
    const float inv_dx = S.inv_dx;
    float4 *acc = static_cast<float4 *>(g.grid_acc);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float wab = W.w[0][a] * W.w[1][b];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float weight = wab * W.w[2][c];
                const float dg[3] = {W.dw[0][a] * W.w[1][b] * W.w[2][c] * inv_dx,
                                     W.w[0][a] * W.dw[1][b] * W.w[2][c] * inv_dx,
                                     W.w[0][a] * W.w[1][b] * W.dw[2][c] * inv_dx};
                const float wm = weight * m;
                float4 add;
                add.x = wm * v[0] + dt * (tau[0] * dg[0] + tau[1] * dg[1] + tau[2] * dg[2]);
                add.y = wm * v[1] + dt * (tau[3] * dg[0] + tau[4] * dg[1] + tau[5] * dg[2]);
                add.z = wm * v[2] + dt * (tau[6] * dg[0] + tau[7] * dg[1] + tau[8] * dg[2]);
                add.w = wm;
                if (!solo) {
#pragma unroll
                    for (int j = 0; j < 5; ++j) {
                        const int d = 1 << j;
                        const float ox = __shfl_down_sync(0xffffffffu, add.x, d);
                        const float oy = __shfl_down_sync(0xffffffffu, add.y, d);
                        const float oz = __shfl_down_sync(0xffffffffu, add.z, d);
                        const float ow = __shfl_down_sync(0xffffffffu, add.w, d);
                        if (in_run[j]) {
                            add.x += ox;
                            add.y += oy;
                            add.z += oz;
                            add.w += ow;
                        }
                    }
                }
                if (act && head) atomicAdd(acc + dense_index(N, base[0] + a, base[1] + b, base[2] + c), add);
            }
        }
}

// grid_normalization_and_gravity_sample_all (mpm_utils.py:405-413) fused with
// the collider sweeps (mpm_solver_warp.py:220-224): every node of the dense
// grid writes grid_m, grid_v_in and grid_v_out.  v_out = v_in / m + dt g on
// marked nodes with m > 1e-10 (a true division, as there), else 0; then each
// collider in registration order, over every node.
__global__ void __launch_bounds__(256) reduced_grid_kernel(const MpmScene *__restrict__ scenes, MpmReducedGrid g,
                                                           float time, float dt, int *status) {
    const MpmScene &S = scenes[0];
    if (!grid_matches(S, g, status)) return;
    const int N = g.n_grid;
    const int64_t nn = (int64_t)N * N * N;
    const float4 *acc = static_cast<const float4 *>(g.grid_acc);
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = acc[q];
        g.grid_m[q] = a.w;
        g.grid_v_in[3 * q + 0] = a.x;
        g.grid_v_in[3 * q + 1] = a.y;
        g.grid_v_in[3 * q + 2] = a.z;
        float v[3] = {0.0f, 0.0f, 0.0f};
        if (g.neighboring_cells[q] > 0 && a.w > 1e-10f) {
            v[0] = __fadd_rn(__fdiv_rn(a.x, a.w), __fmul_rn(dt, S.gravity[0]));
            v[1] = __fadd_rn(__fdiv_rn(a.y, a.w), __fmul_rn(dt, S.gravity[1]));
            v[2] = __fadd_rn(__fdiv_rn(a.z, a.w), __fmul_rn(dt, S.gravity[2]));
        }
        const int ix = (int)(q / ((int64_t)N * N)), iy = (int)((q / N) % N), iz = (int)(q % N);
        for (int k = 0; k < S.n_colliders; ++k) apply_collider(S.colliders[k], S, ix, iy, iz, time, dt, v);
        g.grid_v_out[3 * q + 0] = v[0];
        g.grid_v_out[3 * q + 1] = v[1];
        g.grid_v_out[3 * q + 2] = v[2];
    }
}

// g2p_sample (mpm_utils.py:415-471): one thread per sample point.  Reads the
// dense grid_v_out; writes the particle's u, v, F and F_disp (C and stress
// are left as they are).  The von Mises return map takes yield_stress of the
// sample's list position s (the reference passes its loop index, :464).
// Words are stored one by one: another sample's thread may update the yield
// word of this record.
__global__ void __launch_bounds__(128) g2p_sample_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                         const int *__restrict__ slot_of_uid, MpmReducedGrid g,
                                                         int n, float dt, int *status) {
    const MpmScene &S = scenes[0];
    if (!grid_matches(S, g, status)) return;
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.n_samples) return;
    const int p = g.sample_index[s];
    const bool metal = S.material == MPM_METAL;
    if (p < 0 || p >= n || (metal && s >= n)) {
        atomicOr(status, MPM_ST_BAD_INPUT);
        return;
    }
    const int N = g.n_grid;
    const int slot = slot_of_uid[p];
    const float4 q0 = ldrec(st, slot, 0), q2 = ldrec(st, slot, 2);
    float gp[3];
    gp[0] = grid_coord(q0.x, q2.x, S.inv_dx);
    gp[1] = grid_coord(q0.y, q2.y, S.inv_dx);
    gp[2] = grid_coord(q0.z, q2.z, S.inv_dx);
    int base[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) ok = stencil_base(gp[d], N, base[d]) && ok;
    if (!ok) {
        atomicOr(status, MPM_ST_OUT_OF_DOMAIN);
        return;
    }
    Weights W;
    make_weights(gp, base, W);
    const float inv_dx = S.inv_dx;
    float nv[3] = {0.f, 0.f, 0.f}, nF[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) nF[k] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float weight = W.w[0][a] * W.w[1][b] * W.w[2][c];
                const float dg[3] = {W.dw[0][a] * W.w[1][b] * W.w[2][c] * inv_dx,
                                     W.w[0][a] * W.dw[1][b] * W.w[2][c] * inv_dx,
                                     W.w[0][a] * W.w[1][b] * W.dw[2][c] * inv_dx};
                const float *gv = g.grid_v_out + 3 * dense_index(N, base[0] + a, base[1] + b, base[2] + c);
                const float v0 = gv[0], v1 = gv[1], v2 = gv[2];
                nv[0] += v0 * weight;
                nv[1] += v1 * weight;
                nv[2] += v2 * weight;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    nF[0 + k] += v0 * dg[k];
                    nF[3 + k] += v1 * dg[k];
                    nF[6 + k] += v2 * dg[k];
                }
            }
    // x = x_initial + u (update_x_from_u at the start of p2g2p_reduced), x += dt v (:458)
    float u[3];
    const float x0[3] = {q0.x, q0.y, q0.z}, uo[3] = {q2.x, q2.y, q2.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float x = __fadd_rn(__fadd_rn(x0[d], uo[d]), __fmul_rn(dt, nv[d]));
        u[d] = __fsub_rn(x, x0[d]);  // :469
    }
    const float4 q8 = ldrec(st, slot, 8), q9 = ldrec(st, slot, 9);
    const float Fo_[9] = {q8.x, q8.y, q8.z, q8.w, q9.x, q9.y, q9.z, q9.w, recword(st, slot, rec::F8)};
    float A[9], Ft[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.0f : 0.0f) + dt * nF[k];
    mat_mul(A, Fo_, Ft);
    float yld = 0.0f;
    const int yslot = metal ? slot_of_uid[s] : 0;
    if (metal) yld = recword(st, yslot, rec::YLD);
    float Fn[9], tau[9];
    if (S.material == MPM_JELLY) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Fn[k] = Ft[k];
    } else {
        return_map_stress(S, Ft, yld, Fn, tau);
    }
    if (metal && S.hardening == 1) recword(st, yslot, rec::YLD) = yld;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) finite = finite && isfinite(Fn[k]);
    if (!finite) atomicOr(status, MPM_ST_NONFINITE);
    recword(st, slot, rec::U + 0) = u[0];
    recword(st, slot, rec::U + 1) = u[1];
    recword(st, slot, rec::U + 2) = u[2];
    recword(st, slot, rec::V + 0) = nv[0];
    recword(st, slot, rec::V + 1) = nv[1];
    recword(st, slot, rec::V + 2) = nv[2];
#pragma unroll
    for (int k = 0; k < 8; ++k) recword(st, slot, rec::F0 + k) = Fn[k];
    recword(st, slot, rec::F8) = Fn[8];
    float *fd = g.f_disp + (int64_t)p * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) fd[k] = Fn[k] - ((k % 4 == 0) ? 1.0f : 0.0f);  // :471
}

cudaError_t launch_p2g2p_reduced(const Ctx &cx, const MpmReducedGrid &g, float time, float dt) {
    const int64_t nn = (int64_t)g.n_grid * g.n_grid * g.n_grid;
    cudaError_t e;
    if ((e = cudaMemsetAsync(g.grid_acc, 0, nn * 16, cx.stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(g.neighboring_cells, 0, nn * 4, cx.stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(g.neighboring_cells_grid_v, 0, nn * 4, cx.stream)) != cudaSuccess) return e;
    if (cx.n > 0) {
        if ((e = launch_slot_of_uid(cx)) != cudaSuccess) return e;
        if (g.n_samples > 0)
            mark_kernel<2><<<(unsigned)((g.n_samples + 7) / 8), 256, 0, cx.stream>>>(
                cx.scenes, cx.st, cx.ws.slot_of_uid, g, g.neighboring_cells, cx.n, cx.status);
        reduced_p2g_kernel<<<(cx.n + 255) / 256, 256, 0, cx.stream>>>(cx.scenes, cx.st, g, cx.n, dt, cx.status);
    }
    const int64_t want = (nn + 255) / 256;
    const int blocks = (int)(want < (int64_t)cx.num_sms * 16 ? want : (int64_t)cx.num_sms * 16);
    reduced_grid_kernel<<<blocks > 0 ? blocks : 1, 256, 0, cx.stream>>>(cx.scenes, g, time, dt, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_mark_grid_v(const Ctx &cx, const MpmReducedGrid &g) {
    if (cx.n == 0 || g.n_samples == 0) return cudaSuccess;
    cudaError_t e = launch_slot_of_uid(cx);
    if (e != cudaSuccess) return e;
    mark_kernel<4><<<(unsigned)((g.n_samples + 7) / 8), 256, 0, cx.stream>>>(
        cx.scenes, cx.st, cx.ws.slot_of_uid, g, g.neighboring_cells_grid_v, cx.n, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_g2p_sample(const Ctx &cx, const MpmReducedGrid &g, float dt) {
    if (cx.n == 0 || g.n_samples == 0) return cudaSuccess;
    cudaError_t e = launch_slot_of_uid(cx);
    if (e != cudaSuccess) return e;
    g2p_sample_kernel<<<(unsigned)((g.n_samples + 127) / 128), 128, 0, cx.stream>>>(
        cx.scenes, cx.st, cx.ws.slot_of_uid, g, cx.n, dt, cx.status);
    return cudaGetLastError();
}

}  // namespace mpm
