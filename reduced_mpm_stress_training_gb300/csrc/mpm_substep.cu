// The three transfer stages of the substep.
//
// Grid storage is block-major: the nodes of each 4x4x4 grid block are 64
// consecutive float4 (momentum xyz + mass, or velocity xyz + mass), blocks
// of all scenes concatenated.  Work is a list of "chunks": up to chunk_size
// sorted particles that share one grid block of base cells, so all their
// 3x3x3 stencils fall in the 6x6x6 node tile anchored at that block.
//
//   p2g  -- one CTA per chunk: accumulate the tile in shared memory with
//           shared atomics, flush each non-zero node with ONE float4
//           atomicAdd to global memory, and register the 8 grid blocks the
//           tile covers in the active-block list.
//   grid -- one thread per node of each active block: momentum/mass +
//           gravity, colliders in registration order; clears the block
//           flag.  (The accumulator is zeroed by the next substep's
//           scatter, so grid mass and momentum stay readable meanwhile.)
//   g2p  -- one CTA per chunk: stage the tile of grid velocities in shared
//           memory, gather 27 nodes per particle, APIC C, velocity
//           gradient, F update, return map + stress on one SVD, the
//           displacement update and the block key + histogram of the next
//           substep.
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

__device__ __forceinline__ void chunk_block(const MpmScene &S, int gblock, int &bx, int &by,
                                            int &bz) {
    const int nb = S.n_blocks_axis;
    int lb = (int)(gblock - S.block_begin);
    bz = lb % nb;
    by = (lb / nb) % nb;
    bx = lb / (nb * nb);
}

// ---------------------------------------------------------------------------
// P2G: p2g_apic_stress_given, engine_stress/mpm_utils.py:190-227
//   grid_v_in += (w m)(v + C dpos) + dt (-vol tau) grad w,  grid_m += w m
// ---------------------------------------------------------------------------
template <int CH>
__global__ void __launch_bounds__(CH) p2g_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                 Ws ws, float dt, int *status) {
    __shared__ float tile[kTileNodes * 4];
    const int n_chunks = *ws.n_chunks;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const int4 ch = ws.chunks[c];
        for (int i = threadIdx.x; i < kTileNodes * 4; i += CH) tile[i] = 0.0f;
        __syncthreads();
        const MpmScene &S = scenes[ch.w];
        int bx, by, bz;
        chunk_block(S, ch.x, bx, by, bz);
        if (threadIdx.x < ch.z) {
            const int slot = ws.order[ch.y + threadIdx.x];
            const int64_t sd = st.stride;
            float gp[3];
            int base[3];
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gp[d] = grid_coord(st.x0[slot + d * sd], st.u[slot + d * sd], S.inv_dx);
                ok &= stencil_base(gp[d], S.n_grid, base[d]);
            }
            const int lx = base[0] - 4 * bx, ly = base[1] - 4 * by, lz = base[2] - 4 * bz;
            ok &= (unsigned)lx < 4u && (unsigned)ly < 4u && (unsigned)lz < 4u;
            if (!ok) {
                atomicOr(status, MPM_ST_INTERNAL);
            } else {
                Weights W;
                make_weights(gp, base, W);
                const float m = st.mass[slot], vol = st.vol[slot];
                const float dx = S.dx;
                float Cm[9], T[9], a0[3];
#pragma unroll
                for (int k = 0; k < 9; ++k) Cm[k] = st.C[slot + k * sd];
                // force term: dt * (-vol tau) * grad w, grad w = inv_dx * (...)
                const float tscale = -vol * dt * S.inv_dx;
#pragma unroll
                for (int k = 0; k < 9; ++k) T[k] = st.tau[slot + k * sd] * tscale;
                // momentum term: (w m)(v + C (ijk - fx) dx) = (w m)(a0 + C ijk dx)
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    float cf = Cm[r * 3 + 0] * W.fx[0] + Cm[r * 3 + 1] * W.fx[1] + Cm[r * 3 + 2] * W.fx[2];
                    a0[r] = st.v[slot + r * sd] - cf * dx;
                }
#pragma unroll
                for (int k = 0; k < 9; ++k) Cm[k] *= dx;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const float p1 = W.dw[0][i] * W.w[1][j];
                        const float p2 = W.w[0][i] * W.dw[1][j];
                        const float p3 = W.w[0][i] * W.w[1][j];
                        float aij[3];
#pragma unroll
                        for (int r = 0; r < 3; ++r)
                            aij[r] = a0[r] + (float)i * Cm[r * 3 + 0] + (float)j * Cm[r * 3 + 1];
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const float w = p3 * W.w[2][k];
                            const float wm = w * m;
                            const float g0 = p1 * W.w[2][k], g1 = p2 * W.w[2][k], g2 = p3 * W.dw[2][k];
                            float* t = tile + 4 * (((lx + i) * kTile + (ly + j)) * kTile + (lz + k));
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
                                float mom = wm * (aij[r] + (float)k * Cm[r * 3 + 2]);
                                float f = T[r * 3 + 0] * g0 + T[r * 3 + 1] * g1 + T[r * 3 + 2] * g2;
                                atomicAdd(t + r, mom + f);
                            }
                            atomicAdd(t + 3, wm);
                        }
                    }
                }
            }
        }
        __syncthreads();
        const int nb = S.n_blocks_axis;
        for (int i = threadIdx.x; i < kTileNodes; i += CH) {
            float4 a = reinterpret_cast<float4 *>(tile)[i];
            if (a.x != 0.0f || a.y != 0.0f || a.z != 0.0f || a.w != 0.0f) {
                const int tx = i / 36, ty = (i / 6) % 6, tz = i % 6;
                const int ix = 4 * bx + tx, iy = 4 * by + ty, iz = 4 * bz + tz;
                if (ix < S.n_grid && iy < S.n_grid && iz < S.n_grid)
                    atomicAdd(ws.grid_acc + node_addr(S.block_begin, nb, ix, iy, iz), a);
            }
        }
        if (threadIdx.x < 8) {
            const int gx = bx + (threadIdx.x >> 2), gy = by + ((threadIdx.x >> 1) & 1),
                      gz = bz + (threadIdx.x & 1);
            if (gx < nb && gy < nb && gz < nb) {
                const int gb = (int)(S.block_begin + ((int64_t)(gx * nb + gy) * nb + gz));
                if (atomicExch(ws.block_flag + gb, 1) == 0)
                    ws.active_list[atomicAdd(ws.n_active, 1)] = gb;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Grid update: grid_normalization_and_gravity (engine_stress/mpm_utils.py:229-237)
// then the colliders of engine_stress/mpm_solver_warp.py:429-449 and :505-523.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) grid_kernel(const MpmScene *__restrict__ scenes,
                                                   int n_scenes, Ws ws, float time, float dt) {
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
        float v[3] = {0.f, 0.f, 0.f};
        if (acc.w > 1e-15f) {
            const float inv = 1.0f / acc.w;
            v[0] = __fadd_rn(__fmul_rn(acc.x, inv), __fmul_rn(dt, S.gravity[0]));
            v[1] = __fadd_rn(__fmul_rn(acc.y, inv), __fmul_rn(dt, S.gravity[1]));
            v[2] = __fadd_rn(__fmul_rn(acc.z, inv), __fmul_rn(dt, S.gravity[2]));
        }
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
                if (dp < 0.0f) v[0] = v[1] = v[2] = 0.0f;  // every surface type (:449)
            } else {
                const int id[3] = {ix, iy, iz};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (id[d] < 3 && v[d] < 0.0f) v[d] = 0.0f;
                    if (id[d] >= n - 3 && v[d] > 0.0f) v[d] = 0.0f;
                }
            }
        }
        ws.grid_v[a] = make_float4(v[0], v[1], v[2], acc.w);
        if (l == 0) ws.block_flag[gb] = 0;
    }
}

// ---------------------------------------------------------------------------
// G2P: g2p_apic_and_stress (engine_stress/mpm_utils.py:241-306) fused with
// update_x_from_u / update_u_from_x (:4-15) and the next substep's key.
// ---------------------------------------------------------------------------
template <int CH>
__global__ void __launch_bounds__(CH) g2p_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                 Ws ws, float dt, int *status) {
    __shared__ float4 tile[kTileNodes];
    const int n_chunks = *ws.n_chunks;
    const int sentinel = ws.nbk - 1;
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const int4 ch = ws.chunks[c];
        const MpmScene &S = scenes[ch.w];
        int bx, by, bz;
        chunk_block(S, ch.x, bx, by, bz);
        const int nb = S.n_blocks_axis;
        for (int i = threadIdx.x; i < kTileNodes; i += CH) {
            const int tx = i / 36, ty = (i / 6) % 6, tz = i % 6;
            const int ix = 4 * bx + tx, iy = 4 * by + ty, iz = 4 * bz + tz;
            float4 gv = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ix < S.n_grid && iy < S.n_grid && iz < S.n_grid)
                gv = ws.grid_v[node_addr(S.block_begin, nb, ix, iy, iz)];
            tile[i] = gv;
        }
        __syncthreads();
        int key = -1;
        if (threadIdx.x < ch.z) {
            const int slot = ws.order[ch.y + threadIdx.x];
            const int64_t sd = st.stride;
            float x0[3], gp[3], xo[3];
            int base[3];
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                x0[d] = st.x0[slot + d * sd];
                xo[d] = __fadd_rn(x0[d], st.u[slot + d * sd]);
                gp[d] = __fmul_rn(xo[d], S.inv_dx);
                ok &= stencil_base(gp[d], S.n_grid, base[d]);
            }
            const int lx = base[0] - 4 * bx, ly = base[1] - 4 * by, lz = base[2] - 4 * bz;
            ok &= (unsigned)lx < 4u && (unsigned)ly < 4u && (unsigned)lz < 4u;
            if (!ok) {
                atomicOr(status, MPM_ST_INTERNAL);
                key = sentinel;
                st.key[slot] = key;
            } else {
                Weights W;
                make_weights(gp, base, W);
                const float inv_dx = S.inv_dx;
                float nv[3] = {0.f, 0.f, 0.f}, nC[9], nF[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) { nC[k] = 0.f; nF[k] = 0.f; }
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const float p1 = W.dw[0][i] * W.w[1][j];
                        const float p2 = W.w[0][i] * W.dw[1][j];
                        const float p3 = W.w[0][i] * W.w[1][j];
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const float4 g = tile[((lx + i) * kTile + (ly + j)) * kTile + (lz + k)];
                            const float gv[3] = {g.x, g.y, g.z};
                            const float w = p3 * W.w[2][k];
                            const float dpos[3] = {(float)i - W.fx[0], (float)j - W.fx[1], (float)k - W.fx[2]};
                            const float sc = w * inv_dx * 4.0f;
                            const float dwt[3] = {p1 * W.w[2][k] * inv_dx, p2 * W.w[2][k] * inv_dx,
                                                  p3 * W.dw[2][k] * inv_dx};
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
                                nv[r] += gv[r] * w;
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    nC[r * 3 + q] += gv[r] * dpos[q] * sc;
                                    nF[r * 3 + q] += gv[r] * dwt[q];
                                }
                            }
                        }
                    }
                // x += dt v (:277), u = x - x0 (:12-15)
                float un[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float xn = __fadd_rn(xo[d], __fmul_rn(dt, nv[d]));
                    un[d] = __fsub_rn(xn, x0[d]);
                }
                // F_trial = (I + dt grad v) F (:281)
                float Fp[9], A[9], Ft[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) Fp[k] = st.F[slot + k * sd];
#pragma unroll
                for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.0f : 0.0f) + nF[k] * dt;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        Ft[r * 3 + q] = A[r * 3 + 0] * Fp[0 * 3 + q] + A[r * 3 + 1] * Fp[1 * 3 + q] +
                                        A[r * 3 + 2] * Fp[2 * 3 + q];
                float yld = (S.material == MPM_METAL) ? st.yld[slot] : 0.0f;
                float Fo[9], tau[9];
                return_map_stress(S, Ft, yld, Fo, tau);
                // stores
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    st.v[slot + d * sd] = nv[d];
                    st.u[slot + d * sd] = un[d];
                }
                float chk = 0.0f;
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    st.C[slot + k * sd] = nC[k];
                    st.F[slot + k * sd] = Fo[k];
                    st.tau[slot + k * sd] = tau[k];
                    chk += fabsf(Fo[k]) + fabsf(tau[k]);
                }
                if (S.material == MPM_METAL && S.hardening == 1) st.yld[slot] = yld;
                int flags = 0;
                const float vmax = S.dx / dt;
                if (fabsf(nv[0]) > vmax || fabsf(nv[1]) > vmax || fabsf(nv[2]) > vmax) flags |= MPM_ST_CFL;
                if (!isfinite(chk)) flags |= MPM_ST_NONFINITE;
                bool kok;
                key = particle_key(S, x0[0], x0[1], x0[2], un[0], un[1], un[2], sentinel, kok);
                if (!kok) flags |= MPM_ST_OUT_OF_DOMAIN;
                if (flags) atomicOr(status, flags);
                st.key[slot] = key;
            }
        }
        warp_histogram(ws.counts, key);
        __syncthreads();
    }
}

template <int CH>
static cudaError_t p2g_t(const Ctx &cx, float dt, int grid) {
    p2g_kernel<CH><<<grid, CH, 0, cx.stream>>>(cx.scenes, cx.st, cx.ws, dt, cx.status);
    return cudaGetLastError();
}
template <int CH>
static cudaError_t g2p_t(const Ctx &cx, float dt, int grid) {
    g2p_kernel<CH><<<grid, CH, 0, cx.stream>>>(cx.scenes, cx.st, cx.ws, dt, cx.status);
    return cudaGetLastError();
}

static int persistent_grid(const Ctx &cx, int per_sm) {
    int g = cx.num_sms * per_sm;
    return g < cx.ws.max_chunks ? g : (cx.ws.max_chunks > 0 ? cx.ws.max_chunks : 1);
}

cudaError_t launch_p2g(const Ctx &cx, float dt) {
    const int grid = persistent_grid(cx, 2048 / cx.ws.chunk_size);
    switch (cx.ws.chunk_size) {
        case 32: return p2g_t<32>(cx, dt, grid);
        case 64: return p2g_t<64>(cx, dt, grid);
        case 128: return p2g_t<128>(cx, dt, grid);
        case 256: return p2g_t<256>(cx, dt, grid);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_grid(const Ctx &cx, float time, float dt) {
    int64_t want = (cx.total_blocks + 3) / 4;
    int grid = (int)(want < (int64_t)cx.num_sms * 8 ? want : (int64_t)cx.num_sms * 8);
    if (grid < 1) grid = 1;
    grid_kernel<<<grid, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws, time, dt);
    return cudaGetLastError();
}

cudaError_t launch_g2p(const Ctx &cx, float dt) {
    const int grid = persistent_grid(cx, 1024 / cx.ws.chunk_size);
    switch (cx.ws.chunk_size) {
        case 32: return g2p_t<32>(cx, dt, grid);
        case 64: return g2p_t<64>(cx, dt, grid);
        case 128: return g2p_t<128>(cx, dt, grid);
        case 256: return g2p_t<256>(cx, dt, grid);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mpm
