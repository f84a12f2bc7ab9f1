// Per-substep particle ordering by grid cell, grouped by 4x4x4 grid block.
//
// The reference scatters every particle straight into global memory
// (p2g_apic_stress_given, engine_stress/mpm_utils.py:190-227: 7 float
// atomics per node, 189 per particle).  Here particles are ordered by the
// cell of their stencil base, block-major, so P2G can accumulate a block's
// nodes in shared memory and find each cell's particles as one range.  The
// order is a two-level counting (radix) sort on the cell key
// block * 64 + cell:
//   keys + histograms -- written by G2P for the next substep (block and
//                        cell counts), or by key_kernel after a load moved
//                        particles
//   scan_tiles        -- per-tile sums of the block counts; the last CTA to
//                        finish scans the tile sums (atomic ticket, no spin)
//   scan_finish       -- block offsets, the P2G block list and the G2P chunk
//                        list; for each non-empty block, its 64 cell offsets
//   scatter           -- order[] via warp-aggregated cell-cursor atomics
// G2P then writes every record to the other state buffer at its sorted
// position, so order[] stays close to the identity from one substep to the
// next and the gathers through it stay coalesced.
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

// keys + histogram straight from x0 + u (used after loads)
__global__ void key_kernel(const MpmScene *__restrict__ scenes, int n_scenes, PState st, Ws ws,
                           int n, int *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < n) {
        const float4 q0 = ldrec(st, i, 0), q1 = ldrec(st, i, 1), q2 = ldrec(st, i, 2);
        const int uid = __float_as_int(q1.y);
        const MpmScene &S = scenes[scene_of_particle(scenes, n_scenes, uid)];
        bool ok;
        key = particle_key(S, q0.x, q0.y, q0.z, q2.x, q2.y, q2.z, ws.nbk - 1, ok);
        if (!ok) atomicOr(status, MPM_ST_OUT_OF_DOMAIN);
        st.key[i] = key;
    }
    warp_histogram(ws.counts, ws.cell_counts, key);
}

__device__ __forceinline__ int4 add4(int4 a, int4 b) {
    return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// inclusive scan of an int4 triple over the kScanThreads threads of a CTA;
// returns the thread's inclusive value and leaves the CTA total in *total
constexpr int kScanWarps = kScanThreads / 32;
__device__ __forceinline__ int4 cta_scan4(int4 v, int4 *wsum /* [kScanWarps] shared */, int4 &total) {
    int4 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int4 y;
        y.x = __shfl_up_sync(0xffffffffu, x.x, o);
        y.y = __shfl_up_sync(0xffffffffu, x.y, o);
        y.z = __shfl_up_sync(0xffffffffu, x.z, o);
        y.w = 0;
        if ((threadIdx.x & 31) >= o) x = add4(x, y);
    }
    if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
    __syncthreads();
    int4 pre = make_int4(0, 0, 0, 0);
    total = make_int4(0, 0, 0, 0);
    for (int w = 0; w < kScanWarps; ++w) {
        if (w < (int)(threadIdx.x >> 5)) pre = add4(pre, wsum[w]);
        total = add4(total, wsum[w]);
    }
    __syncthreads();
    return add4(pre, x);
}

// per-bucket triple: (particles, G2P chunks, non-empty blocks) -- the
// sentinel bucket (out-of-domain particles) gets copy chunks but no block
__device__ __forceinline__ int4 bucket_triple(const Ws &ws, int b, int cnt) {
    const int ch = (cnt + ws.chunk_size - 1) / ws.chunk_size;
    if (b >= ws.nbk - 1) return make_int4(cnt, ch, 0, 0);
    return make_int4(cnt, ch, cnt > 0 ? 1 : 0, 0);
}

// Phase 1: per-tile sums.  The last CTA to finish (atomic ticket; nobody
// waits) scans the tile sums into exclusive tile offsets and publishes the
// work-list lengths.
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(Ws ws) {
    __shared__ int4 wsum[kScanWarps];
    __shared__ bool last;
    const int tile = blockIdx.x;
    const int b0 = tile * kScanTile + threadIdx.x * kScanPerThread;
    int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll
    for (int j = 0; j < kScanPerThread; ++j) {
        int b = b0 + j;
        if (b < ws.nbk) acc = add4(acc, bucket_triple(ws, b, ws.counts[b]));
    }
    int4 total;
    cta_scan4(acc, wsum, total);
    if (threadIdx.x == 0) {
        ws.tile_sums[tile] = total;
        __threadfence();
        unsigned t = atomicAdd(ws.ticket, 1u);
        last = (t == (unsigned)gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    int4 carry = make_int4(0, 0, 0, 0);
    for (int base = 0; base < ws.n_tiles; base += kScanThreads) {
        const int t = base + threadIdx.x;
        int4 v = t < ws.n_tiles ? __ldcg(ws.tile_sums + t) : make_int4(0, 0, 0, 0);
        int4 tot;
        int4 inc = cta_scan4(v, wsum, tot);
        if (t < ws.n_tiles) {
            int4 ex = add4(carry, make_int4(inc.x - v.x, inc.y - v.y, inc.z - v.z, 0));
            ws.tile_sums[t] = ex;
        }
        carry = add4(carry, tot);
    }
    if (threadIdx.x == 0) {
        // counts always sum to n when the stages run in order; the clamps keep
        // a mis-sequenced call from walking past the work lists
        *ws.n_chunks = min(carry.y, ws.max_chunks);
        *ws.n_blocks = min(carry.z, ws.nbk - 1);
        *ws.ticket = 0u;  // re-arm for the next substep
    }
}

// Phase 2: bucket offsets / cursors, the G2P chunk list and the P2G block
// list; zeroes the histogram for the next substep.  Each thread first finds
// the offsets of its buckets (a CTA scan on top of the tile's exclusive
// prefix); then the CTA's warps take its non-empty buckets one at a time and
// write the 64 cell offsets of each with a warp scan (two cells per lane),
// and its chunk-list entries with one lane per chunk.
__global__ void __launch_bounds__(kScanThreads) scan_finish_kernel(const MpmScene *__restrict__ scenes,
                                                          int n_scenes, Ws ws) {
    __shared__ int4 wsum[kScanWarps];
    __shared__ int s_off[kScanTile], s_coff[kScanTile], s_boff[kScanTile], s_cnt[kScanTile];
    __shared__ int s_list[kScanTile];
    __shared__ int s_nlist;
    const int tile = blockIdx.x;
    const int b0 = tile * kScanTile + threadIdx.x * kScanPerThread;
    if (threadIdx.x == 0) s_nlist = 0;
    const int4 pre = ws.tile_sums[tile];  // loaded beside the counts: one round trip for both
    int cnt[kScanPerThread];
    int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll
    for (int j = 0; j < kScanPerThread; ++j) {
        int b = b0 + j;
        cnt[j] = b < ws.nbk ? ws.counts[b] : 0;
        if (b < ws.nbk) acc = add4(acc, bucket_triple(ws, b, cnt[j]));
    }
    int4 total;
    int4 inc = cta_scan4(acc, wsum, total);  // its barriers also order s_nlist = 0
    int off = pre.x + inc.x - acc.x, coff = pre.y + inc.y - acc.y, boff = pre.z + inc.z - acc.z;
#pragma unroll
    for (int j = 0; j < kScanPerThread; ++j) {
        const int b = b0 + j;
        if (b >= ws.nbk) break;
        ws.counts[b] = 0;
        const int li = threadIdx.x * kScanPerThread + j;
        s_off[li] = off;
        s_coff[li] = coff;
        s_boff[li] = boff;
        s_cnt[li] = cnt[j];
        // the out-of-domain bucket always gets its cursor (its particles sort
        // after every other one; G2P's copy chunks count them again)
        if (cnt[j] > 0 || b == ws.nbk - 1) s_list[atomicAdd(&s_nlist, 1)] = li;
        const int4 t = bucket_triple(ws, b, cnt[j]);
        off += t.x;
        coff += t.y;
        boff += t.z;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int nlist = s_nlist;
    const int cs = ws.chunk_size;
    // a warp takes kScanPrefetch of the tile's non-empty buckets at a time and
    // loads all their cell counts before scanning any, so the loads' round
    // trips overlap instead of queueing one after another
    constexpr int kScanPrefetch = 8;
    const int warp = (int)(threadIdx.x >> 5);
    for (int i0 = warp; i0 < nlist; i0 += kScanWarps * kScanPrefetch) {
        int lis[kScanPrefetch];
        int2 ks[kScanPrefetch];
#pragma unroll
        for (int u = 0; u < kScanPrefetch; ++u) {
            const int i = i0 + u * kScanWarps;
            lis[u] = i < nlist ? s_list[i] : -1;
            ks[u] = lis[u] >= 0
                        ? reinterpret_cast<const int2 *>(ws.cell_counts + (int64_t)(tile * kScanTile + lis[u]) * 64)[lane]
                        : make_int2(0, 0);
        }
#pragma unroll
        for (int u = 0; u < kScanPrefetch; ++u) {
            const int li = lis[u];
            if (li < 0) break;  // uniform over the warp
            const int b = tile * kScanTile + li;
            const int bo = s_off[li], n_b = s_cnt[li];
            // cell offsets of the block: lane owns cells 2 lane, 2 lane + 1
            const int2 k = ks[u];
            const int sum = k.x + k.y;
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int st = bo + incl - sum;
            const int2 st2 = make_int2(st, st + k.x);
            reinterpret_cast<int2 *>(ws.cell_start + (int64_t)b * 64)[lane] = st2;
            reinterpret_cast<int2 *>(ws.cell_cursor + (int64_t)b * 64)[lane] = st2;
            reinterpret_cast<int2 *>(ws.cell_counts + (int64_t)b * 64)[lane] = make_int2(0, 0);
            if (n_b > 0) {
                const bool real = b < ws.nbk - 1;
                const int sc = real ? scene_of_block(scenes, n_scenes, b) : -1;  // -1: copy chunk
                if (real && lane == 0 && s_boff[li] < ws.nbk - 1) ws.blocks[s_boff[li]] = make_int4(b, bo, n_b, sc);
                const int nch = (n_b + cs - 1) / cs;
                for (int c = lane; c < nch; c += 32) {
                    const int at = s_coff[li] + c;
                    if (at < ws.max_chunks) ws.chunks[at] = make_int4(b, bo + c * cs, min(cs, n_b - c * cs), sc);
                }
            }
        }
    }
    if (tile == 0 && threadIdx.x == 0) {
        *ws.n_active_prev = *ws.n_active;
        *ws.n_active = 0;
    }
}

// order[cell_cursor[key]++] = slot, warp-aggregated.  Each thread takes
// kScatterPer keys (strided by the grid's thread count) so that their
// cursor atomics are in flight together.  Also zeroes the grid accumulator
// of the previous substep's active blocks (kept until now so grid mass and
// momentum stay readable between substeps).
constexpr int kScatterPer = 4;

__global__ void __launch_bounds__(256) scatter_kernel(PState st, Ws ws, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    int key[kScatterPer], base[kScatterPer];
    unsigned peers[kScatterPer];
    // the keys' loads first, so their round trip overlaps the clearing below
#pragma unroll
    for (int r = 0; r < kScatterPer; ++r) {
        const int64_t idx = (int64_t)i + (int64_t)r * stride;
        key[r] = idx < n ? __ldcs(st.key + idx) : -1;
    }
    const int nclear = *ws.n_active_prev * kBlockNodes;
    for (int j = i; j < nclear; j += stride)
        ws.grid_acc[(int64_t)ws.active_list[j >> 6] * kBlockNodes + (j & 63)] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int r = 0; r < kScatterPer; ++r) {
        peers[r] = __match_any_sync(0xffffffffu, key[r]);
        const int leader = __ffs(peers[r]) - 1;
        base[r] = 0;
        if (key[r] >= 0 && lane == leader) base[r] = atomicAdd(ws.cell_cursor + key[r], __popc(peers[r]));
    }
#pragma unroll
    for (int r = 0; r < kScatterPer; ++r) {
        const int leader = __ffs(peers[r]) - 1;
        const int b = __shfl_sync(0xffffffffu, base[r], leader);
        const int pos = b + __popc(peers[r] & ((1u << lane) - 1u));
        const int64_t idx = (int64_t)i + (int64_t)r * stride;
        if (key[r] >= 0 && pos < n) ws.order[pos] = (int)idx;
    }
}

cudaError_t launch_keys(const Ctx &cx) {
    if (cx.n == 0) return cudaSuccess;
    key_kernel<<<(cx.n + 255) / 256, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.st, cx.ws,
                                                           cx.n, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_sort(const Ctx &cx) {
    scan_tiles_kernel<<<cx.ws.n_tiles, kScanThreads, 0, cx.stream>>>(cx.ws);
    scan_finish_kernel<<<cx.ws.n_tiles, kScanThreads, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws);
    const int per = 256 * kScatterPer;
    const int sgrid = cx.n > 0 ? (cx.n + per - 1) / per : 1;
    scatter_kernel<<<sgrid, 256, 0, cx.stream>>>(cx.st, cx.ws, cx.n);
    return cudaGetLastError();
}


}  // namespace mpm
