// The three transfer stages of the substep.
//
// Grid storage is block-major: the nodes of each 4x4x4 grid block are 64
// consecutive float4 (momentum xyz + mass, or velocity xyz + mass), blocks
// of all scenes concatenated.  The particles whose stencil base cells lie in
// one grid block have all their 3x3x3 stencils in the 6x6x6 node tile
// anchored at that block.
//
//   p2g  -- one warp per non-empty block: per-cell runs of particles summed
//           in registers and added to a warp-private tile in shared memory,
//           each non-zero node flushed with ONE float4 atomicAdd to global
//           memory, and the 8 grid blocks the tile covers registered in the
//           active-block list.
//   grid -- one thread per node of each active block: momentum/mass +
//           gravity, colliders in registration order; clears the block
//           flag.  (The accumulator is zeroed by the next substep's
//           scatter, so grid mass and momentum stay readable meanwhile.)
//   g2p  -- one CTA per chunk (up to chunk_size sorted particles of one
//           block): stage the tile of grid velocities in shared
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
// (cell_start .. cell_cursor).  Particles of one cell share their 27 stencil
// nodes, so a lane takes a run of consecutive particles of one cell, sums
// their contributions in registers (27 nodes x 4 = 108 accumulators) and
// adds them to the tile once: the shared-memory read-modify-writes drop
// from one per particle and node to one per run and node.  A round gives
// each lane a run of the same length L from a DISTINCT cell, whose stencils
// hit distinct nodes for every node offset -- the tile updates are
// race-free.  The cells are chosen longest-remaining first (every cell with
// at least t particles left, t the smallest threshold that leaves at most 32
// such cells, filled up to 32 with cells that have t - 1 left: Hu's list
// schedule for chains), and L is the fewest particles any chosen cell has
// left, at most kRunMax, so no lane idles inside a round.  Each lane streams
// its run's 128-byte records into shared memory with cp.async one particle
// ahead.  The tile is flushed with one
// float4 atomicAdd per non-zero node into the global grid.
//
// Tile layout: rows of 6 nodes along z padded to 8 slots and rotated by
// 4 (y & 1), so a node's 16-byte bank group is (z + 4 (y & 1)) mod 8: the 8
// lanes of a quarter-warp (one 128-bit shared access phase) holding two
// y-adjacent rows of 4 cells hit 8 distinct bank groups for every offset.
// ---------------------------------------------------------------------------
constexpr int kP2GWarps = 1;  // one warp per CTA: the hardware balances unequal blocks
constexpr int kRunMax = 4;     // most particles of one cell a lane takes per round
constexpr int kP2GQuads = 8;   // record quads P2G reads (q0-q7, 128 B)
constexpr int kRowSlots = 8;
constexpr int kP2GSlots = kTile * kTile * kRowSlots;

__device__ __forceinline__ int p2g_slot(int x, int y, int z) {
    return (x * kTile + y) * kRowSlots + ((z + 4 * (y & 1)) & 7);
}

struct P2GWarpSmem {
    float4 tile[kP2GSlots];
    float4 rec[2][kP2GQuads][32];  // each lane's current and next record
    int4 seg[32];                  // the round's runs: first sorted position, cell
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

// add one particle's 27 node contributions to the lane's accumulators
// (x, y packed in axy, z and mass in azw: Blackwell's two-wide FP32 FMA).
// Per (i,j) the node value factors over k:
//   add_r = wz_k A_r + k wz_k B_r + dwz_k D_r,  mass = pm wz_k
// with pm = wx_i wy_j m, A_r = pm (a0_r + i Cdx_r + j Cdy_r) + T_r0 dwx_i wy_j
// + T_r1 wx_i dwy_j, B_r = pm Cdz_r, D_r = T_r2 wx_i wy_j.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

__device__ __forceinline__ void p2g_accumulate(const P2GParticle &P, float2 (&axy)[27], float2 (&azw)[27]) {
    const float2 a0 = f2(P.a0[0], P.a0[1]);
    const float2 cdx = f2(P.Cd[0], P.Cd[3]), cdy = f2(P.Cd[1], P.Cd[4]), cdz = f2(P.Cd[2], P.Cd[5]);
    const float2 t0 = f2(P.T[0], P.T[3]), t1 = f2(P.T[1], P.T[4]), t2 = f2(P.T[2], P.T[5]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float p1 = P.W.dw[0][i] * P.W.w[1][j];
            const float p2 = P.W.w[0][i] * P.W.dw[1][j];
            const float p3 = P.W.w[0][i] * P.W.w[1][j];
            const float pm = p3 * P.m;
            float2 aij = a0;
            if (i > 0) aij = __ffma2_rn(f2((float)i, (float)i), cdx, aij);
            if (j > 0) aij = __ffma2_rn(f2((float)j, (float)j), cdy, aij);
            const float2 A = __ffma2_rn(f2(pm, pm), aij, __ffma2_rn(t0, f2(p1, p1), __fmul2_rn(t1, f2(p2, p2))));
            const float2 B = __fmul2_rn(f2(pm, pm), cdz);
            const float2 D = __fmul2_rn(t2, f2(p3, p3));
            const float az = P.a0[2] + (float)i * P.Cd[6] + (float)j * P.Cd[7];
            const float Az = pm * az + P.T[6] * p1 + P.T[7] * p2;
            const float Bz = pm * P.Cd[8];
            const float Dz = P.T[8] * p3;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float wz = P.W.w[2][k], dwz = P.W.dw[2][k];
                float2 &xy = axy[(i * 3 + j) * 3 + k];
                float2 &zw = azw[(i * 3 + j) * 3 + k];
                xy = __ffma2_rn(f2(wz, wz), A, xy);
                zw = __ffma2_rn(f2(wz, wz), f2(Az, pm), zw);
                xy = __ffma2_rn(f2(dwz, dwz), D, xy);
                zw.x = fmaf(dwz, Dz, zw.x);
                if (k > 0) {
                    const float kwz = k == 1 ? wz : 2.0f * wz;
                    xy = __ffma2_rn(f2(kwz, kwz), B, xy);
                    zw.x = fmaf(kwz, Bz, zw.x);
                }
            }
        }
    }
}

// add a segment's accumulated nodes into the tile (read-modify-write; the
// lanes of `mask` hold distinct cells)
__device__ __forceinline__ void p2g_flush(const float2 (&axy)[27], const float2 (&azw)[27], int lx, int ly,
                                          int lz, float4 *tile, unsigned mask) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float4 *t = tile + p2g_slot(lx + i, ly + j, lz + k);
                const int n = (i * 3 + j) * 3 + k;
                float4 o = *t;
                o.x += axy[n].x;
                o.y += axy[n].y;
                o.z += azw[n].x;
                o.w += azw[n].y;
                *t = o;
                __syncwarp(mask);
            }
}

__device__ __forceinline__ void p2g_cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// queue the copy of one record (slot >= 0) into the lane's buffer b
__device__ __forceinline__ void p2g_prefetch(P2GWarpSmem &sm, const PState &st, int slot, int b, int lane, int n) {
    if (slot >= 0 && slot < n) {
#pragma unroll
        for (int q = 0; q < kP2GQuads; ++q) p2g_cp_async16(&sm.rec[b][q][lane], recq(st, slot, q));
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Choose the next round of a block: up to 32 distinct cells, longest
// remaining first, each giving its next L particles.  Lane `lane` owns cells
// lane and lane + 32 (remaining counts rem0/rem1, next positions pos0/pos1).
// Returns false when the block is done; else the lane's run (first sorted
// position, cell, length len: L or 0) and the round length L.
__device__ __forceinline__ bool p2g_next_round(int &rem0, int &rem1, int &pos0, int &pos1, int lane, unsigned lt,
                                               int4 *seg, int &start, int &cell, int &len, int &L) {
    const unsigned full = 0xffffffffu;
    const int maxrem = __reduce_max_sync(full, max(rem0, rem1));
    if (maxrem == 0) return false;
    // smallest t >= 1 with at most 32 cells holding >= t particles
    int lo = 1, hi = maxrem + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int cnt = __popc(__ballot_sync(full, rem0 >= mid)) + __popc(__ballot_sync(full, rem1 >= mid));
        if (cnt <= 32) hi = mid;
        else lo = mid + 1;
    }
    const unsigned h0 = __ballot_sync(full, rem0 >= lo), h1 = __ballot_sync(full, rem1 >= lo);
    const int need = 32 - __popc(h0) - __popc(h1);
    const unsigned f0 = __ballot_sync(full, lo > 1 && rem0 == lo - 1);
    const unsigned f1 = __ballot_sync(full, lo > 1 && rem1 == lo - 1);
    const bool p0 = rem0 >= lo || (((f0 >> lane) & 1u) && __popc(f0 & lt) < need);
    const bool p1 = rem1 >= lo || (((f1 >> lane) & 1u) && __popc(f0) + __popc(f1 & lt) < need);
    const unsigned b0 = __ballot_sync(full, p0), b1 = __ballot_sync(full, p1);
    // every chosen cell gives its next L particles, L = the fewest any of them has left
    const unsigned least =
        __reduce_min_sync(full, min(p0 ? (unsigned)rem0 : 0xffffffffu, p1 ? (unsigned)rem1 : 0xffffffffu));
    L = min((int)least, kRunMax);
    if (p0) {
        seg[__popc(b0 & lt)] = make_int4(pos0, lane, 0, 0);
        pos0 += L;
        rem0 -= L;
    }
    if (p1) {
        seg[__popc(b0) + __popc(b1 & lt)] = make_int4(pos1, lane + 32, 0, 0);
        pos1 += L;
        rem1 -= L;
    }
    const int tot = __popc(b0) + __popc(b1);
    __syncwarp();
    const int4 mine = lane < tot ? seg[lane] : make_int4(0, 0, 0, 0);
    __syncwarp();  // seg[] is rewritten by the next call
    start = mine.x;
    cell = mine.y;
    len = lane < tot ? L : 0;
    return true;
}

// partials == nullptr: the tile is flushed with float4 atomics into grid_acc.
// Otherwise (the ordered mode of mpm_p2g_ordered) the whole 6x6x6 tile of
// work-list entry bi goes to partials[bi] and blk_index[block] = bi; the
// gather kernel then sums the <= 8 tiles covering each node in a fixed order.
__global__ void __launch_bounds__(kP2GWarps * 32, 2) p2g_kernel(const MpmScene *__restrict__ scenes,
                                                                int n_scenes, PState st, Ws ws, float dt,
                                                                int *status, float4 *partials,
                                                                int *blk_index) {
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
        if ((unsigned)be.x >= (unsigned)(ws.nbk - 1) || (unsigned)be.w >= (unsigned)n_scenes) {
            // a damaged work list: skip, never index with it
            if (lane == 0) atomicOr(status, MPM_ST_INTERNAL);
            continue;
        }
        // by value: the compiler loads the few fields P2G uses once per block into
        // registers (measured 1 us per launch faster than reading them through a reference)
        const MpmScene S = scenes[be.w];
        int bx, by, bz;
        chunk_block(S, be.x, bx, by, bz);
        for (int i = lane; i < kP2GSlots; i += 32) sm.tile[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        // cell ranges of this block: lane owns cells lane and lane + 32
        const int64_t cb = (int64_t)be.x * 64;
        const int s0 = ws.cell_start[cb + lane], s1 = ws.cell_start[cb + lane + 32];
        const int c0 = max(0, ws.cell_cursor[cb + lane] - s0);
        const int c1 = max(0, ws.cell_cursor[cb + lane + 32] - s1);
        // Rounds are software-pipelined: while round A is summed, round B is
        // chosen and its order[] entries load, and A's last iteration already
        // streams B's first records.
        int rem0 = c0, rem1 = c1, pos0 = s0, pos1 = s1;
        int startA, cellA, lenA, LA;
        bool haveA = p2g_next_round(rem0, rem1, pos0, pos1, lane, lt, sm.seg, startA, cellA, lenA, LA);
        int slA[kRunMax];
#pragma unroll
        for (int t = 0; t < kRunMax; ++t) slA[t] = t < lenA && startA + t < ws.n ? ws.order[startA + t] : -1;
        int buf = 0;
        if (haveA) p2g_prefetch(sm, st, slA[0], 0, lane, ws.n);
        bool bad = false;
        while (haveA) {
            int startB, cellB, lenB, LB;
            const bool haveB = p2g_next_round(rem0, rem1, pos0, pos1, lane, lt, sm.seg, startB, cellB, lenB, LB);
            int slB[kRunMax];
#pragma unroll
            for (int t = 0; t < kRunMax; ++t)
                slB[t] = haveB && t < lenB && startB + t < ws.n ? ws.order[startB + t] : -1;
            const int cx = cellA >> 4, cy = (cellA >> 2) & 3, cz = cellA & 3;
            float2 axy[27], azw[27];
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                axy[k] = make_float2(0.f, 0.f);
                azw[k] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int t = 0; t < kRunMax; ++t) {
                if (t < LA) {  // warp-uniform
                    // the next record (this run's, or the next round's first) streams in
                    // while this one is summed
                    int nxt = slB[0];
#pragma unroll
                    for (int u = 0; u + 1 < kRunMax; ++u)
                        if (u == t && t + 1 < LA) nxt = slA[u + 1];
                    p2g_prefetch(sm, st, nxt, buf ^ 1, lane, ws.n);
                    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
                    if (t < lenA && slA[t] < 0) {
                        bad = true;  // position or slot out of range: nothing was staged
                    } else if (t < lenA) {
                        float4 q[kP2GQuads];
#pragma unroll
                        for (int qq = 0; qq < kP2GQuads; ++qq) q[qq] = sm.rec[buf][qq][lane];
                        P2GParticle P;
                        const bool ok =
                            p2g_load(S, q, bx, by, bz, dt, P) && P.lx == cx && P.ly == cy && P.lz == cz;
                        if (ok) p2g_accumulate(P, axy, azw);
                        bad |= !ok;
                    }
                    buf ^= 1;
                }
            }
            const unsigned fm = __ballot_sync(full, lenA > 0);
            if (lenA > 0) p2g_flush(axy, azw, cx, cy, cz, sm.tile, fm);
            __syncwarp();
            haveA = haveB;
            startA = startB;
            cellA = cellB;
            lenA = lenB;
            LA = LB;
#pragma unroll
            for (int t = 0; t < kRunMax; ++t) slA[t] = slB[t];
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        if (bad) atomicOr(status, MPM_ST_INTERNAL);
        const int nb = S.n_blocks_axis;
        if (partials) {
            // ordered mode: the whole tile to this entry's slot, in node order
            float4 *dst = partials + (int64_t)bi * kTileNodes;
            for (int i = lane; i < kTileNodes; i += 32)
                dst[i] = sm.tile[p2g_slot(i / (kTile * kTile), (i / kTile) % kTile, i % kTile)];
            if (lane == 0) blk_index[be.x] = bi;
        }
        // flush the tile: one float4 atomic per non-zero node
        for (int i = lane; i < kP2GSlots && !partials; i += 32) {
            const float4 a = sm.tile[i];
            if (a.x != 0.0f || a.y != 0.0f || a.z != 0.0f || a.w != 0.0f) {
                const int tx = i / (kTile * kRowSlots), ty = (i / kRowSlots) % kTile;
                const int tz = ((i & 7) - 4 * (ty & 1)) & 7;  // unused slots (tz 6, 7) stay zero
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

// The reference's modify_bc callbacks (:561-565, :594-603, :690-693,
// :716-718): after an active substep's grid update, a moving collider's point
// advances by dt times its velocity (the circling column's velocity from its
// current angle), summed in double and stored in float as the host-side
// update does.  One thread per collider slot.
__global__ void advance_colliders_kernel(MpmScene *__restrict__ scenes, int n_scenes, float time, float dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_scenes * MPM_MAX_COLLIDERS) return;
    MpmScene &S = scenes[i / MPM_MAX_COLLIDERS];
    const int k = i % MPM_MAX_COLLIDERS;
    if (k >= S.n_colliders) return;
    MpmCollider &cl = S.colliders[k];
    if (!(time >= cl.start_time && time < cl.end_time)) return;
    float vel[3];
    if (cl.kind == MPM_COLLIDER_VPLANE || cl.kind == MPM_COLLIDER_CUBE || cl.kind == MPM_COLLIDER_SPHERE) {
        vel[0] = cl.velocity[0];
        vel[1] = cl.velocity[1];
        vel[2] = cl.velocity[2];
    } else if (cl.kind == MPM_COLLIDER_CIRCLE) {
        const float th = circle_theta(cl.point);
        vel[0] = -cl.v_scale * sinf(th);
        vel[1] = 0.0f;
        vel[2] = cl.v_scale * cosf(th);
    } else {
        return;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) cl.point[d] = (float)((double)cl.point[d] + (double)dt * (double)vel[d]);
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
        for (int k = 0; k < S.n_colliders; ++k) apply_collider(S.colliders[k], S, ix, iy, iz, time, dt, v);
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
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// three velocity components: x, y as a pair for the two-wide FP32 FMA, z alone
struct V3 {
    float2 xy;
    float z;
};
__device__ __forceinline__ V3 v3zero() { return {make_float2(0.0f, 0.0f), 0.0f}; }
__device__ __forceinline__ V3 v3of(const float4 &g) { return {make_float2(g.x, g.y), g.z}; }
__device__ __forceinline__ V3 v3mul(float a, const V3 &x) { return {__fmul2_rn(make_float2(a, a), x.xy), a * x.z}; }
__device__ __forceinline__ V3 v3fma(float a, const V3 &x, const V3 &acc) {
    return {__ffma2_rn(make_float2(a, a), x.xy, acc.xy), fmaf(a, x.z, acc.z)};
}

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
            cp_async16(&sm.rec[b][q][threadIdx.x], recq(st, slot, g2p_quad(q)), 16);
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
    // The chunk list is walked from its end.  P2G has just streamed the records
    // in ascending block order, so the highest positions are the ones still in
    // L2; and the records written last here (the lowest positions) are the
    // first that the next substep's P2G reads.  Measured 207.2 -> 203.7 us per
    // substep on the 1M column against walking it from the start.
    const int sentinel = (ws.nbk - 1) * 64;  // out-of-domain cell key
    int c = blockIdx.x;
    if (c >= n_chunks) return;
    int4 ch = ws.chunks[n_chunks - 1 - c];
    int slot = g2p_slot(ws, ch);
    g2p_prefetch<CH>(scenes, st, ws, ch, slot, sm, 0);
    cp_async_commit();
    int cn = c + gridDim.x;
    int4 chn = make_int4(0, 0, 0, -1);
    int slotn = 0;
    if (cn < n_chunks) {
        chn = ws.chunks[n_chunks - 1 - cn];
        slotn = g2p_slot(ws, chn);
    }
    int buf = 0;
    while (c < n_chunks) {
        // order[] indices two chunks ahead
        const int cnn = cn + gridDim.x;
        int4 chnn = make_int4(0, 0, 0, -1);
        int slotnn = 0;
        if (cnn < n_chunks) {
            chnn = ws.chunks[n_chunks - 1 - cnn];
            slotnn = g2p_slot(ws, chnn);
        }
        // this chunk's records and tile have landed, for every thread; and every
        // warp is done with the other half of the buffer (the previous chunk),
        // so the next chunk's copies may go there now -- the only CTA-wide
        // barrier of the iteration
        cp_async_wait0();
        __syncthreads();
        if (cn < n_chunks) g2p_prefetch<CH>(scenes, st, ws, chn, slotn, sm, buf ^ 1);
        cp_async_commit();

        const int pos = ch.y + (int)threadIdx.x;
        const bool mine = (int)threadIdx.x < ch.z && pos < ws.n;
        int key = -1;
        if (ch.w < 0) {  // out-of-domain particles: carry the records over (uniform per CTA)
            if (mine) {
#pragma unroll
                for (int q = 0; q < kRecQuads; ++q) strec(out, pos, q, ldrec(st, slot, q));
                key = st.key[slot];  // counted again below: the next sort keeps their copy chunk
                out.key[pos] = key;
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
                // z first (S, D, K per (i,j)), then y, then x.  Velocity
                // components x, y ride together in Blackwell's two-wide FP32
                // FMA (a V3 is (xy pair, z)); nF and M are kept by column.
                V3 nvp = v3zero(), nF0 = v3zero(), nF1 = v3zero(), nF2 = v3zero();
                V3 M0 = v3zero(), M1 = v3zero(), M2 = v3zero();
                const float wz0 = W.w[2][0], wz1 = W.w[2][1], wz2 = W.w[2][2];
                const float dz0 = W.dw[2][0], dz1 = W.dw[2][1], dz2 = W.dw[2][2];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    V3 Ti = v3zero(), Ui = v3zero(), Ri = v3zero(), Ji = v3zero(), Ki = v3zero();
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        const float4 *row = tile + ((lx + i) * kTile + (ly + j)) * kTile + lz;
                        const V3 g0 = v3of(row[0]), g1 = v3of(row[1]), g2 = v3of(row[2]);
                        const V3 Sz = v3fma(wz2, g2, v3fma(wz1, g1, v3mul(wz0, g0)));
                        const V3 Dz = v3fma(dz2, g2, v3fma(dz1, g1, v3mul(dz0, g0)));
                        const V3 Kz = v3fma(2.0f * wz2, g2, v3mul(wz1, g1));
                        const float wy = W.w[1][j], dwy = W.dw[1][j];
                        Ti = v3fma(wy, Sz, Ti);
                        Ui = v3fma(dwy, Sz, Ui);
                        Ri = v3fma(wy, Dz, Ri);
                        Ki = v3fma(wy, Kz, Ki);
                        if (j > 0) Ji = v3fma((float)j * wy, Sz, Ji);
                    }
                    const float wx = W.w[0][i], dwx = W.dw[0][i];
                    nvp = v3fma(wx, Ti, nvp);
                    nF0 = v3fma(dwx, Ti, nF0);
                    nF1 = v3fma(wx, Ui, nF1);
                    nF2 = v3fma(wx, Ri, nF2);
                    if (i > 0) M0 = v3fma((float)i * wx, Ti, M0);
                    M1 = v3fma(wx, Ji, M1);
                    M2 = v3fma(wx, Ki, M2);
                }
                const float nv[3] = {nvp.xy.x, nvp.xy.y, nvp.z};
                float nF[9] = {nF0.xy.x, nF1.xy.x, nF2.xy.x, nF0.xy.y, nF1.xy.y, nF2.xy.y, nF0.z, nF1.z, nF2.z};
                const float M[9] = {M0.xy.x, M1.xy.x, M2.xy.x, M0.xy.y, M1.xy.y, M2.xy.y, M0.z, M1.z, M2.z};
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
        // each warp writes out the records its own lanes staged
        __syncwarp();
        if (ch.w >= 0) {
            // each warp writes its own 32 records, contiguous in each of the
            // three arrays, with coalesced float4 stores: quads 0-3 to a and
            // 4-7 to b (four per record), quads 8-9 to f (two per record)
            const int w0 = (int)(threadIdx.x & ~31u);
            const int np = max(0, min(min(32, ch.z - w0), ws.n - ch.y - w0));
            const int64_t p0 = (int64_t)ch.y + w0;
            const float4 *src = sm.outrec + w0 * kOutStride;
            const int lane = (int)(threadIdx.x & 31u);
            for (int l = lane; l < 4 * np; l += 32) {
                const float4 *rq = src + (l >> 2) * kOutStride + (l & 3);
                out.a[p0 * 4 + l] = rq[0];
                out.b[p0 * 4 + l] = rq[4];
            }
            for (int l = lane; l < 2 * np; l += 32) out.f[p0 * 2 + l] = src[(l >> 1) * kOutStride + 8 + (l & 1)];
        }
        // outrec and this half of the buffer are rewritten only after the next
        // iteration's barrier, which every warp reaches after its write-out
        c = cn; ch = chn; slot = slotn;
        cn = cnn; chn = chnn; slotn = slotnn;
        buf ^= 1;
    }
    cp_async_wait0();
}

static int persistent_grid(const Ctx &cx, int per_sm) {
    int g = cx.num_sms * per_sm;
    return g < cx.ws.max_chunks ? g : (cx.ws.max_chunks > 0 ? cx.ws.max_chunks : 1);
}

// One wave of persistent CTAs: as many as fit on the GPU at once (the
// occupancy of this instance, looked up once per device).  A second wave
// would start only as the first one exits, so the first wave's chunks would
// spread over the whole list instead of sweeping it as one band, and the L2
// reuse with P2G (the chunk list walked from its end) would fall: 200.2 ->
// 198.8 us per substep on the 1M column against twice the resident count.
template <int CH, bool DEFER>
static cudaError_t g2p_t(const Ctx &cx, float dt) {
    // more than the 48 KB of static shared memory: opt in once per instance and device
    static int resident[64] = {0};
    const int bytes = (int)sizeof(G2PSmem<CH>);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (resident[dev] == 0) {
        e = cudaFuncSetAttribute(g2p_kernel<CH, DEFER>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        int nb = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, g2p_kernel<CH, DEFER>, CH, bytes);
        if (e != cudaSuccess) return e;
        resident[dev] = nb > 0 ? nb : 1;
    }
    const int grid = persistent_grid(cx, resident[dev]);
    g2p_kernel<CH, DEFER><<<grid, CH, bytes, cx.stream>>>(cx.scenes, cx.st, cx.st2, cx.ws, dt, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_p2g(const Ctx &cx, float dt, float4 *partials, int *blk_index) {
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
    // up to 32 single-warp CTAs per SM, several times the resident ones: the
    // rest start as others finish, which balances blocks of unequal size;
    // warps loop over blocks when there are more blocks than warps
    int64_t want = (cx.total_blocks + kP2GWarps - 1) / kP2GWarps;
    int grid = (int)(want < (int64_t)cx.num_sms * 32 ? want : (int64_t)cx.num_sms * 32);
    if (grid < 1) grid = 1;
    p2g_kernel<<<grid, kP2GWarps * 32, bytes, cx.stream>>>(cx.scenes, cx.n_scenes, cx.st, cx.ws, dt,
                                                           cx.status, partials, blk_index);
    return cudaGetLastError();
}

cudaError_t launch_grid(const Ctx &cx, float time, float dt) {
    int64_t want = (cx.total_blocks + 3) / 4;
    int grid = (int)(want < (int64_t)cx.num_sms * 8 ? want : (int64_t)cx.num_sms * 8);
    if (grid < 1) grid = 1;
    grid_kernel<<<grid, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws, time, dt);
    return cudaGetLastError();
}

cudaError_t launch_advance_colliders(MpmScene *scenes, int n_scenes, float time, float dt, cudaStream_t stream) {
    const int slots = n_scenes * MPM_MAX_COLLIDERS;
    if (slots <= 0) return cudaSuccess;
    advance_colliders_kernel<<<(slots + 127) / 128, 128, 0, stream>>>(scenes, n_scenes, time, dt);
    return cudaGetLastError();
}

template <bool DEFER>
static cudaError_t g2p_sized(const Ctx &cx, float dt) {
    switch (cx.ws.chunk_size) {
        case 32: return g2p_t<32, DEFER>(cx, dt);
        case 64: return g2p_t<64, DEFER>(cx, dt);
        case 128: return g2p_t<128, DEFER>(cx, dt);
        case 256: return g2p_t<256, DEFER>(cx, dt);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_g2p(const Ctx &cx, float dt, bool defer_stress) {
    return defer_stress ? g2p_sized<true>(cx, dt) : g2p_sized<false>(cx, dt);
}

}  // namespace mpm
