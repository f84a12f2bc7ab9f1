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
//           displacement update and the cell key + histograms of the next
//           substep.  Each updated record is written to the other state
//           buffer at its sorted position, so every substep leaves the
//           particle state physically sorted by cell.
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

// ---------------------------------------------------------------------------
// P2G: p2g_apic_stress_given, engine_stress/mpm_utils.py:190-227
//   grid_v_in += (w m)(v + C dpos) + dt (-vol tau) grad w,  grid_m += w m
//
// One warp per non-empty grid block, with a warp-private 6x6x6 node tile in
// shared memory and no floating-point atomics in the particle loop.  The
// sort delivers the block's particles ordered by cell with each cell's range
// (cell_start .. cell_cursor).  The warp walks them "layer-major": layer r
// holds the r-th particle of every cell, so a window of 32 consecutive
// entries has (almost always) 32 distinct cells, whose stencils hit distinct
// nodes for every node offset -- plain read-modify-writes of the tile are
// race-free.  The rare lanes that share a cell (windows spanning two short
// layers) are serialised by __match_any_sync rank.  A window reads 32 whole
// particle records (128 B each, float4 loads), so the scattered order costs
// no extra DRAM sectors.  The tile is flushed with one float4 atomicAdd per
// non-zero node into the global grid.
// ---------------------------------------------------------------------------
constexpr int kP2GWarps = 4;
constexpr int kPassCap = 256;  // layer-major entries buffered per batch
constexpr int kP2GQuads = 8;   // record quads P2G reads (q0-q7, 128 B)

struct P2GWarpSmem {
    float4 tile[kTileNodes];
    int perm[kPassCap];                 // record slots of the batch, layer-major
    float4 rec[kP2GQuads][32];          // records of the next 32-particle window
};

struct P2GParticle {
    Weights W;
    int lx, ly, lz;
    float m;
    float a0[3];  // v - C fx dx
    float Cd[9];  // C dx
    float T[9];   // -dt vol inv_dx tau
};

__device__ __forceinline__ bool p2g_load(const MpmScene &S, const float4 (&q)[kP2GQuads], int bx, int by,
                                         int bz, float dt, P2GParticle &P) {
    // record quads 0-7: x0 m | vol .. | u v.x | v.yz C0 C1 | C2-5 | C6-8 tau0 | tau1-4 | tau5-8
    const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4], q5 = q[5], q6 = q[6], q7 = q[7];
    const float x0[3] = {q0.x, q0.y, q0.z}, u[3] = {q2.x, q2.y, q2.z};
    float gp[3];
    int base[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        gp[d] = grid_coord(x0[d], u[d], S.inv_dx);
        ok &= stencil_base(gp[d], S.n_grid, base[d]);
    }
    P.lx = base[0] - 4 * bx;
    P.ly = base[1] - 4 * by;
    P.lz = base[2] - 4 * bz;
    ok &= (unsigned)P.lx < 4u && (unsigned)P.ly < 4u && (unsigned)P.lz < 4u;
    if (!ok) return false;
    make_weights(gp, base, P.W);
    P.m = q0.w;
    const float vol = q1.x;
    const float dx = S.dx;
    const float v[3] = {q2.w, q3.x, q3.y};
    const float Cm[9] = {q3.z, q3.w, q4.x, q4.y, q4.z, q4.w, q5.x, q5.y, q5.z};
    const float tau[9] = {q5.w, q6.x, q6.y, q6.z, q6.w, q7.x, q7.y, q7.z, q7.w};
    const float tscale = -vol * dt * S.inv_dx;
#pragma unroll
    for (int k = 0; k < 9; ++k) P.T[k] = tau[k] * tscale;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float cf = Cm[r * 3 + 0] * P.W.fx[0] + Cm[r * 3 + 1] * P.W.fx[1] + Cm[r * 3 + 2] * P.W.fx[2];
        P.a0[r] = v[r] - cf * dx;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) P.Cd[k] = Cm[k] * dx;
    return true;
}

// add one particle's 27 node contributions into the tile (read-modify-write).
// Per (i,j) the node value factors over k:
//   add_r = wz_k A_r + k wz_k B_r + dwz_k D_r,  mass = pm wz_k
// with pm = wx_i wy_j m, A_r = pm (a0_r + i Cdx_r + j Cdy_r) + T_r0 dwx_i wy_j
// + T_r1 wx_i dwy_j, B_r = pm Cdz_r, D_r = T_r2 wx_i wy_j.
__device__ __forceinline__ void p2g_scatter(const P2GParticle &P, float4 *tile, unsigned mask) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float p1 = P.W.dw[0][i] * P.W.w[1][j];
            const float p2 = P.W.w[0][i] * P.W.dw[1][j];
            const float p3 = P.W.w[0][i] * P.W.w[1][j];
            const float pm = p3 * P.m;
            float A[3], B[3], D[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float aij = P.a0[r] + (float)i * P.Cd[r * 3 + 0] + (float)j * P.Cd[r * 3 + 1];
                A[r] = pm * aij + P.T[r * 3 + 0] * p1 + P.T[r * 3 + 1] * p2;
                B[r] = pm * P.Cd[r * 3 + 2];
                D[r] = P.T[r * 3 + 2] * p3;
            }
            float4 *t = tile + ((P.lx + i) * kTile + (P.ly + j)) * kTile + P.lz;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float wz = P.W.w[2][k], dwz = P.W.dw[2][k], kwz = (float)k * wz;
                float4 o = t[k];
                o.x += wz * A[0] + kwz * B[0] + dwz * D[0];
                o.y += wz * A[1] + kwz * B[1] + dwz * D[1];
                o.z += wz * A[2] + kwz * B[2] + dwz * D[2];
                o.w += pm * wz;
                t[k] = o;
                __syncwarp(mask);
            }
        }
    }
}

__device__ __forceinline__ void p2g_cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// queue the record copies of window w of the batch (lane = entry)
__device__ __forceinline__ void p2g_prefetch(P2GWarpSmem &sm, const PState &st, int w, int nv, int lane) {
    const int k = w * 32 + lane;
    if (k < nv) {
        const float4 *src = st.rec + (int64_t)sm.perm[k] * kRecQuads;
#pragma unroll
        for (int q = 0; q < kP2GQuads; ++q) p2g_cp_async16(&sm.rec[q][lane], src + q);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__global__ void __launch_bounds__(kP2GWarps * 32, 5) p2g_kernel(const MpmScene *__restrict__ scenes,
                                                                PState st, Ws ws, float dt,
                                                                int *status) {
    extern __shared__ __align__(16) unsigned char p2g_smem_raw[];
    P2GWarpSmem *smem = reinterpret_cast<P2GWarpSmem *>(p2g_smem_raw);
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    P2GWarpSmem &sm = smem[threadIdx.x >> 5];
    const int nblk = *ws.n_blocks;
    for (int bi = blockIdx.x * kP2GWarps + (int)(threadIdx.x >> 5); bi < nblk;
         bi += gridDim.x * kP2GWarps) {
        const int4 be = ws.blocks[bi];
        const MpmScene &S = scenes[be.w];
        int bx, by, bz;
        chunk_block(S, be.x, bx, by, bz);
        for (int i = lane; i < kTileNodes; i += 32) sm.tile[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        // cell ranges of this block: lane owns cells lane and lane + 32
        const int64_t cb = (int64_t)be.x * 64;
        const int s0 = ws.cell_start[cb + lane], s1 = ws.cell_start[cb + lane + 32];
        const int c0 = max(0, ws.cell_cursor[cb + lane] - s0);
        const int c1 = max(0, ws.cell_cursor[cb + lane + 32] - s1);
        const int maxcnt = __reduce_max_sync(full, max(c0, c1));
        int r = 0;
        while (r < maxcnt) {
            // layer-major batch: whole layers while they fit in the buffer
            int nv = 0;
            while (r < maxcnt && nv <= kPassCap - 64) {
                const bool a = c0 > r, b = c1 > r;
                const unsigned ma = __ballot_sync(full, a), mb = __ballot_sync(full, b);
                // sorted positions come from the block's cell ranges (< n); store their slots
                if (a) sm.perm[nv + __popc(ma & lt)] = ws.order[s0 + r];
                if (b) sm.perm[nv + __popc(ma) + __popc(mb & lt)] = ws.order[s1 + r];
                nv += __popc(ma) + __popc(mb);
                ++r;
            }
            __syncwarp();
            // windows of 32 entries; once window w is in registers, the records
            // of window w + 1 stream into the shared buffer while w is scattered
            const int nwin = (nv + 31) >> 5;
            if (nwin > 0) p2g_prefetch(sm, st, 0, nv, lane);
            for (int w = 0; w < nwin; ++w) {
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                __syncwarp();
                const int k = w * 32 + lane;
                bool act = k < nv;
                float4 q[kP2GQuads];
                if (act) {
#pragma unroll
                    for (int qq = 0; qq < kP2GQuads; ++qq) q[qq] = sm.rec[qq][lane];
                }
                __syncwarp();
                if (w + 1 < nwin) p2g_prefetch(sm, st, w + 1, nv, lane);
                P2GParticle P;
                if (act) {
                    act = p2g_load(S, q, bx, by, bz, dt, P);
                    if (!act) atomicOr(status, MPM_ST_INTERNAL);
                }
                const int cell = act ? (P.lx * 4 + P.ly) * 4 + P.lz : -1 - lane;
                const unsigned peers = __match_any_sync(full, cell);
                const int rank = act ? __popc(peers & lt) : 0;
                const int npass = __reduce_max_sync(full, rank) + 1;
                for (int q = 0; q < npass; ++q) {
                    const bool go = act && rank == q;
                    const unsigned gm = __ballot_sync(full, go);
                    if (go) p2g_scatter(P, sm.tile, gm);
                    __syncwarp();
                }
            }
            __syncwarp();  // perm and the record buffers are refilled by the next batch
        }
        // flush the tile: one float4 atomic per non-zero node
        const int nb = S.n_blocks_axis;
        for (int i = lane; i < kTileNodes; i += 32) {
            const float4 a = sm.tile[i];
            if (a.x != 0.0f || a.y != 0.0f || a.z != 0.0f || a.w != 0.0f) {
                const int tx = i / 36, ty = (i / 6) % 6, tz = i % 6;
                const int ix = 4 * bx + tx, iy = 4 * by + ty, iz = 4 * bz + tz;
                if (ix < S.n_grid && iy < S.n_grid && iz < S.n_grid)
                    atomicAdd(ws.grid_acc + node_addr(S.block_begin, nb, ix, iy, iz), a);
            }
        }
        if (lane < 8) {
            const int gx = bx + (lane >> 2), gy = by + ((lane >> 1) & 1), gz = bz + (lane & 1);
            if (gx < nb && gy < nb && gz < nb) {
                const int gb = (int)(S.block_begin + ((int64_t)(gx * nb + gy) * nb + gz));
                if (atomicExch(ws.block_flag + gb, 1) == 0)
                    ws.active_list[atomicAdd(ws.n_active, 1)] = gb;
            }
        }
        __syncwarp();
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
// Reads records from `st` through order[], writes them to `out` at the
// sorted position.  Chunks with scene -1 hold out-of-domain particles,
// which are carried over unchanged.
//
// Software-pipelined over the CTA's chunks: while chunk k is computed, the
// particle records (quads 0,1,2,8,9) and the 6x6x6 grid-velocity tile of
// chunk k+1 stream into the other half of a double buffer in shared memory
// with cp.async, and the order[] indices of chunk k+2 are loaded.  The
// updated records are assembled in shared memory and written to their
// (contiguous) sorted range with coalesced float4 stores.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

constexpr int kG2PQuads = 5;  // record quads G2P reads: 0, 1, 2, 8, 9
__device__ __forceinline__ int g2p_quad(int q) { return q < 3 ? q : q + 5; }

constexpr int kOutStride = kRecQuads + 1;  // padded so the per-thread record writes are conflict-free

template <int CH>
struct G2PSmem {
    float4 tile[2][kTileNodes];
    float4 rec[2][kG2PQuads][CH];
    float4 outrec[CH * kOutStride];  // updated records of the chunk, written out coalesced
};

// queue the async copies of one chunk into buffer b
template <int CH>
__device__ __forceinline__ void g2p_prefetch(const MpmScene *__restrict__ scenes, const PState &st,
                                             const Ws &ws, const int4 &ch, int slot,
                                             G2PSmem<CH> &sm, int b) {
    if (ch.w < 0) return;  // copy chunk: no compute, nothing to stage
    if ((int)threadIdx.x < ch.z && ch.y + (int)threadIdx.x < ws.n) {
#pragma unroll
        for (int q = 0; q < kG2PQuads; ++q)
            cp_async16(&sm.rec[b][q][threadIdx.x], st.rec + (int64_t)slot * kRecQuads + g2p_quad(q), 16);
    }
    const MpmScene &S = scenes[ch.w];
    int bx, by, bz;
    chunk_block(S, ch.x, bx, by, bz);
    const int nb = S.n_blocks_axis;
    for (int i = threadIdx.x; i < kTileNodes; i += CH) {
        const int tx = i / 36, ty = (i / 6) % 6, tz = i % 6;
        const int ix = 4 * bx + tx, iy = 4 * by + ty, iz = 4 * bz + tz;
        const bool in = ix < S.n_grid && iy < S.n_grid && iz < S.n_grid;
        const float4 *src = ws.grid_v + (in ? node_addr(S.block_begin, nb, ix, iy, iz) : 0);
        cp_async16(&sm.tile[b][i], src, in ? 16 : 0);  // outside the grid: zero fill
    }
}

__device__ __forceinline__ int g2p_slot(const Ws &ws, const int4 &ch) {
    const int pos = ch.y + (int)threadIdx.x;
    return ((int)threadIdx.x < ch.z && pos < ws.n) ? ws.order[pos] : 0;
}

// DEFER: leave the return map and stress to a later pass (the surrogate stress
// stage): F_trial is stored as F and the stress words are zeroed.
template <int CH, bool DEFER>
__global__ void __launch_bounds__(CH) g2p_kernel(const MpmScene *__restrict__ scenes, PState st,
                                                 PState out, Ws ws, float dt, int *status) {
    extern __shared__ __align__(16) unsigned char g2p_smem_raw[];
    G2PSmem<CH> &sm = *reinterpret_cast<G2PSmem<CH> *>(g2p_smem_raw);
    const int n_chunks = *ws.n_chunks;
    const int sentinel = (ws.nbk - 1) * 64;  // out-of-domain cell key
    int c = blockIdx.x;
    if (c >= n_chunks) return;
    int4 ch = ws.chunks[c];
    int slot = g2p_slot(ws, ch);
    g2p_prefetch<CH>(scenes, st, ws, ch, slot, sm, 0);
    cp_async_commit();
    int cn = c + gridDim.x;
    int4 chn = make_int4(0, 0, 0, -1);
    int slotn = 0;
    if (cn < n_chunks) {
        chn = ws.chunks[cn];
        slotn = g2p_slot(ws, chn);
    }
    int buf = 0;
    while (c < n_chunks) {
        if (cn < n_chunks) g2p_prefetch<CH>(scenes, st, ws, chn, slotn, sm, buf ^ 1);
        cp_async_commit();
        // order[] indices two chunks ahead
        const int cnn = cn + gridDim.x;
        int4 chnn = make_int4(0, 0, 0, -1);
        int slotnn = 0;
        if (cnn < n_chunks) {
            chnn = ws.chunks[cnn];
            slotnn = g2p_slot(ws, chnn);
        }
        cp_async_wait1();
        __syncthreads();

        const int pos = ch.y + (int)threadIdx.x;
        const bool mine = (int)threadIdx.x < ch.z && pos < ws.n;
        int key = -1;
        if (ch.w < 0) {  // out-of-domain particles: carry the records over (uniform per CTA)
            if (mine) {
#pragma unroll
                for (int q = 0; q < kRecQuads; ++q) strec(out, pos, q, ldrec(st, slot, q));
                out.key[pos] = st.key[slot];
            }
        } else if (mine) {
            const MpmScene &S = scenes[ch.w];
            int bx, by, bz;
            chunk_block(S, ch.x, bx, by, bz);
            const float4 *tile = sm.tile[buf];
            const float4 q0 = sm.rec[buf][0][threadIdx.x], q1 = sm.rec[buf][1][threadIdx.x],
                         q2 = sm.rec[buf][2][threadIdx.x], q8 = sm.rec[buf][3][threadIdx.x],
                         q9 = sm.rec[buf][4][threadIdx.x];
            const float x0[3] = {q0.x, q0.y, q0.z};
            const float xo[3] = {__fadd_rn(q0.x, q2.x), __fadd_rn(q0.y, q2.y), __fadd_rn(q0.z, q2.z)};
            const float Fp[9] = {q8.x, q8.y, q8.z, q8.w, q9.x, q9.y, q9.z, q9.w, q1.w};
            float gp[3];
            int base[3];
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                gp[d] = __fmul_rn(xo[d], S.inv_dx);
                ok &= stencil_base(gp[d], S.n_grid, base[d]);
            }
            const int lx = base[0] - 4 * bx, ly = base[1] - 4 * by, lz = base[2] - 4 * bz;
            ok &= (unsigned)lx < 4u && (unsigned)ly < 4u && (unsigned)lz < 4u;
            float4 *orec = sm.outrec + threadIdx.x * kOutStride;
            if (!ok) {
                atomicOr(status, MPM_ST_INTERNAL);
                key = sentinel;
#pragma unroll
                for (int q = 0; q < kRecQuads; ++q) orec[q] = ldrec(st, slot, q);
                out.key[pos] = key;
            } else {
                Weights W;
                make_weights(gp, base, W);
                const float inv_dx = S.inv_dx;
                // Separable gather (same sums as :261-273, regrouped by axis):
                //   nv  = sum_ijk wx_i wy_j wz_k g
                //   nF  = sum g (x) (dwx wy wz, wx dwy wz, wx wy dwz)   (times inv_dx)
                //   M_c = sum (w g) * (ijk)_c,  C = 4 inv_dx (M - nv (x) fx)
                // z first (S, D, K per (i,j)), then y, then x.
                float nv[3] = {0.f, 0.f, 0.f}, nF[9], M[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) { nF[k] = 0.f; M[k] = 0.f; }
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    float Ti[3] = {0.f, 0.f, 0.f}, Ui[3] = {0.f, 0.f, 0.f}, Ri[3] = {0.f, 0.f, 0.f};
                    float Ji[3] = {0.f, 0.f, 0.f}, Ki[3] = {0.f, 0.f, 0.f};
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const float4 *row = tile + ((lx + i) * kTile + (ly + j)) * kTile + lz;
                        const float4 g0 = row[0], g1 = row[1], g2 = row[2];
                        const float gz[3][3] = {{g0.x, g0.y, g0.z}, {g1.x, g1.y, g1.z}, {g2.x, g2.y, g2.z}};
                        float Sz[3], Dz[3], Kz[3];
#pragma unroll
                        for (int r = 0; r < 3; ++r) {
                            Sz[r] = W.w[2][0] * gz[0][r] + W.w[2][1] * gz[1][r] + W.w[2][2] * gz[2][r];
                            Dz[r] = W.dw[2][0] * gz[0][r] + W.dw[2][1] * gz[1][r] + W.dw[2][2] * gz[2][r];
                            Kz[r] = W.w[2][1] * gz[1][r] + 2.0f * (W.w[2][2] * gz[2][r]);
                        }
                        const float wy = W.w[1][j], dwy = W.dw[1][j];
#pragma unroll
                        for (int r = 0; r < 3; ++r) {
                            Ti[r] += wy * Sz[r];
                            Ui[r] += dwy * Sz[r];
                            Ri[r] += wy * Dz[r];
                            Ki[r] += wy * Kz[r];
                            if (j > 0) Ji[r] += (float)j * (wy * Sz[r]);
                        }
                    }
                    const float wx = W.w[0][i], dwx = W.dw[0][i];
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        nv[r] += wx * Ti[r];
                        nF[r * 3 + 0] += dwx * Ti[r];
                        nF[r * 3 + 1] += wx * Ui[r];
                        nF[r * 3 + 2] += wx * Ri[r];
                        if (i > 0) M[r * 3 + 0] += (float)i * (wx * Ti[r]);
                        M[r * 3 + 1] += wx * Ji[r];
                        M[r * 3 + 2] += wx * Ki[r];
                    }
                }
                float nC[9];
                const float c4 = 4.0f * inv_dx;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q) nC[r * 3 + q] = c4 * (M[r * 3 + q] - nv[r] * W.fx[q]);
#pragma unroll
                for (int k = 0; k < 9; ++k) nF[k] *= inv_dx;
                // x += dt v (:277), u = x - x0 (:12-15)
                float un[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float xn = __fadd_rn(xo[d], __fmul_rn(dt, nv[d]));
                    un[d] = __fsub_rn(xn, x0[d]);
                }
                // F_trial = (I + dt grad v) F (:281)
                float A[9], Ft[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) A[k] = ((k % 4 == 0) ? 1.0f : 0.0f) + nF[k] * dt;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        Ft[r * 3 + q] = A[r * 3 + 0] * Fp[0 * 3 + q] + A[r * 3 + 1] * Fp[1 * 3 + q] +
                                        A[r * 3 + 2] * Fp[2 * 3 + q];
                float yld = (S.material == MPM_METAL) ? q1.z : 0.0f;
                float Fo[9], tau[9];
                if (DEFER) {
#pragma unroll
                    for (int k = 0; k < 9; ++k) {
                        Fo[k] = Ft[k];
                        tau[k] = 0.0f;
                    }
                } else {
                    return_map_stress(S, Ft, yld, Fo, tau);
                }
                // stores: record quads 1-9
                float chk = 0.0f;
#pragma unroll
                for (int k = 0; k < 9; ++k) chk += fabsf(Fo[k]) + fabsf(tau[k]);
                if (!(S.material == MPM_METAL && S.hardening == 1)) yld = q1.z;
                orec[0] = q0;
                orec[1] = make_float4(q1.x, q1.y, yld, Fo[8]);
                orec[2] = make_float4(un[0], un[1], un[2], nv[0]);
                orec[3] = make_float4(nv[1], nv[2], nC[0], nC[1]);
                orec[4] = make_float4(nC[2], nC[3], nC[4], nC[5]);
                orec[5] = make_float4(nC[6], nC[7], nC[8], tau[0]);
                orec[6] = make_float4(tau[1], tau[2], tau[3], tau[4]);
                orec[7] = make_float4(tau[5], tau[6], tau[7], tau[8]);
                orec[8] = make_float4(Fo[0], Fo[1], Fo[2], Fo[3]);
                orec[9] = make_float4(Fo[4], Fo[5], Fo[6], Fo[7]);
                int flags = 0;
                const float vmax = S.dx / dt;
                if (fabsf(nv[0]) > vmax || fabsf(nv[1]) > vmax || fabsf(nv[2]) > vmax) flags |= MPM_ST_CFL;
                if (!isfinite(chk)) flags |= MPM_ST_NONFINITE;
                bool kok;
                key = particle_key(S, x0[0], x0[1], x0[2], un[0], un[1], un[2], ws.nbk - 1, kok);
                if (!kok) flags |= MPM_ST_OUT_OF_DOMAIN;
                if (flags) atomicOr(status, flags);
                out.key[pos] = key;
            }
        }
        warp_histogram(ws.counts, ws.cell_counts, key);
        __syncthreads();
        if (ch.w >= 0) {  // the chunk's records are contiguous in `out`: coalesced write-out
            const int nq = min(ch.z, ws.n - ch.y) * kRecQuads;
            float4 *dst = out.rec + (int64_t)ch.y * kRecQuads;
            for (int l = threadIdx.x; l < nq; l += CH)
                dst[l] = sm.outrec[(l / kRecQuads) * kOutStride + (l % kRecQuads)];
        }
        __syncthreads();  // buffer `buf` and outrec are refilled by the next iteration
        c = cn; ch = chn; slot = slotn;
        cn = cnn; chn = chnn; slotn = slotnn;
        buf ^= 1;
    }
    cp_async_wait0();
}

template <int CH, bool DEFER>
static cudaError_t g2p_t(const Ctx &cx, float dt, int grid) {
    // more than the 48 KB of static shared memory: opt in once per instance and device
    static bool attr_set[64] = {false};
    const int bytes = (int)sizeof(G2PSmem<CH>);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(g2p_kernel<CH, DEFER>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    g2p_kernel<CH, DEFER><<<grid, CH, bytes, cx.stream>>>(cx.scenes, cx.st, cx.st2, cx.ws, dt, cx.status);
    return cudaGetLastError();
}

static int persistent_grid(const Ctx &cx, int per_sm) {
    int g = cx.num_sms * per_sm;
    return g < cx.ws.max_chunks ? g : (cx.ws.max_chunks > 0 ? cx.ws.max_chunks : 1);
}

cudaError_t launch_p2g(const Ctx &cx, float dt) {
    // more than the 48 KB of static shared memory: opt in once per device
    static bool attr_set[64] = {false};
    const int bytes = (int)(sizeof(P2GWarpSmem) * kP2GWarps);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(p2g_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    // persistent: five CTAs (20 warps) per SM, never more warps than blocks
    int64_t want = (cx.total_blocks + kP2GWarps - 1) / kP2GWarps;
    int grid = (int)(want < (int64_t)cx.num_sms * 5 ? want : (int64_t)cx.num_sms * 5);
    if (grid < 1) grid = 1;
    p2g_kernel<<<grid, kP2GWarps * 32, bytes, cx.stream>>>(cx.scenes, cx.st, cx.ws, dt, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_grid(const Ctx &cx, float time, float dt) {
    int64_t want = (cx.total_blocks + 3) / 4;
    int grid = (int)(want < (int64_t)cx.num_sms * 8 ? want : (int64_t)cx.num_sms * 8);
    if (grid < 1) grid = 1;
    grid_kernel<<<grid, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws, time, dt);
    return cudaGetLastError();
}

template <bool DEFER>
static cudaError_t g2p_sized(const Ctx &cx, float dt) {
    const int grid = persistent_grid(cx, 1024 / cx.ws.chunk_size);
    switch (cx.ws.chunk_size) {
        case 32: return g2p_t<32, DEFER>(cx, dt, grid);
        case 64: return g2p_t<64, DEFER>(cx, dt, grid);
        case 128: return g2p_t<128, DEFER>(cx, dt, grid);
        case 256: return g2p_t<256, DEFER>(cx, dt, grid);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_g2p(const Ctx &cx, float dt, bool defer_stress) {
    return defer_stress ? g2p_sized<true>(cx, dt) : g2p_sized<false>(cx, dt);
}

}  // namespace mpm
