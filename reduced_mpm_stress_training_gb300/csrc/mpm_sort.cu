// Per-substep particle ordering by 4x4x4 grid block ("bucket").
//
// The reference scatters every particle straight into global memory
// (p2g_apic_stress_given, engine_stress/mpm_utils.py:190-227: 7 float
// atomics per node, 189 per particle).  Here particles are grouped by the
// grid block that holds their base cell, so P2G can accumulate a block's
// nodes in shared memory.  The order is a single-digit counting (radix)
// sort on the block key:
//   keys + histogram  -- written by G2P for the next substep, or by
//                        key_kernel after a load moved particles
//   scan_tiles        -- per-tile sums of (count, chunks); the last CTA
//                        to finish scans the tile sums (ticket, no spin)
//   scan_finish       -- bucket offsets, cursors, the chunk work list
//   scatter           -- order[] via warp-aggregated cursor atomics
//   permute           -- every k substeps, physically reorder the state
//                        so the order[] gathers stay coalesced
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

// keys + histogram straight from x0 + u (used after loads)
__global__ void key_kernel(const MpmScene *__restrict__ scenes, int n_scenes, PState st, Ws ws,
                           int n, int *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < n) {
        int uid = st.uid[i];
        const MpmScene &S = scenes[scene_of_particle(scenes, n_scenes, uid)];
        const int64_t sd = st.stride;
        bool ok;
        key = particle_key(S, st.x0[i], st.x0[i + sd], st.x0[i + 2 * sd], st.u[i], st.u[i + sd],
                           st.u[i + 2 * sd], ws.nbk - 1, ok);
        if (!ok) atomicOr(status, MPM_ST_OUT_OF_DOMAIN);
        st.key[i] = key;
    }
    warp_histogram(ws.counts, key);
}

// Phase 1: per-tile sums of (count, ceil(count/chunk)).  The last CTA
// (atomic ticket; nobody waits) scans the tile sums into exclusive offsets
// and publishes the chunk total.
__global__ void __launch_bounds__(256) scan_tiles_kernel(Ws ws) {
    __shared__ int2 red[8];
    __shared__ bool last;
    const int tile = blockIdx.x;
    const int b0 = tile * kScanTile + threadIdx.x * 8;
    const int cs = ws.chunk_size;
    int c = 0, k = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int b = b0 + j;
        if (b < ws.nbk - 1) {  // the sentinel bucket gets no chunks
            int v = ws.counts[b];
            c += v;
            k += (v + cs - 1) / cs;
        } else if (b == ws.nbk - 1) {
            c += ws.counts[b];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_down_sync(0xffffffffu, c, o);
        k += __shfl_down_sync(0xffffffffu, k, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_int2(c, k);
    __syncthreads();
    if (threadIdx.x == 0) {
        int2 s = make_int2(0, 0);
        for (int w = 0; w < 8; ++w) { s.x += red[w].x; s.y += red[w].y; }
        ws.tile_sums[tile] = s;
        __threadfence();
        unsigned t = atomicAdd(ws.ticket, 1u);
        last = (t == (unsigned)gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    // last CTA: exclusive scan of the tile sums (n_tiles <= a few thousand)
    __threadfence();
    __shared__ int2 carry;
    if (threadIdx.x == 0) carry = make_int2(0, 0);
    __syncthreads();
    for (int base = 0; base < ws.n_tiles; base += 256) {
        int t = base + threadIdx.x;
        int2 v = t < ws.n_tiles ? __ldcg(ws.tile_sums + t) : make_int2(0, 0);
        int x = v.x, y = v.y;
        // inclusive warp scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int xs = __shfl_up_sync(0xffffffffu, x, o), ys = __shfl_up_sync(0xffffffffu, y, o);
            if ((threadIdx.x & 31) >= o) { x += xs; y += ys; }
        }
        __shared__ int2 wsum[8];
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = make_int2(x, y);
        __syncthreads();
        int2 pre = carry;
        for (int w = 0; w < (threadIdx.x >> 5); ++w) { pre.x += wsum[w].x; pre.y += wsum[w].y; }
        if (t < ws.n_tiles) ws.tile_sums[t] = make_int2(pre.x + x - v.x, pre.y + y - v.y);
        __syncthreads();
        if (threadIdx.x == 255) carry = make_int2(pre.x + x, pre.y + y);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *ws.n_chunks = carry.y;
        *ws.ticket = 0u;  // re-arm for the next substep
    }
}

// Phase 2: bucket offsets / cursors, chunk list, zero the histogram.
__global__ void __launch_bounds__(256) scan_finish_kernel(const MpmScene *__restrict__ scenes,
                                                          int n_scenes, Ws ws) {
    const int tile = blockIdx.x;
    const int b0 = tile * kScanTile + threadIdx.x * 8;
    const int cs = ws.chunk_size;
    int cnt[8];
    int c = 0, k = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int b = b0 + j;
        cnt[j] = b < ws.nbk ? ws.counts[b] : 0;
        c += cnt[j];
        if (b < ws.nbk - 1) k += (cnt[j] + cs - 1) / cs;
    }
    // block-wide exclusive scan of (c, k)
    int x = c, y = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int xs = __shfl_up_sync(0xffffffffu, x, o), ys = __shfl_up_sync(0xffffffffu, y, o);
        if ((threadIdx.x & 31) >= o) { x += xs; y += ys; }
    }
    __shared__ int2 wsum[8];
    if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = make_int2(x, y);
    __syncthreads();
    int2 pre = ws.tile_sums[tile];
    for (int w = 0; w < (threadIdx.x >> 5); ++w) { pre.x += wsum[w].x; pre.y += wsum[w].y; }
    int off = pre.x + x - c, coff = pre.y + y - k;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int b = b0 + j;
        if (b >= ws.nbk) break;
        ws.offsets[b] = off;
        ws.cursor[b] = off;
        ws.counts[b] = 0;
        if (b < ws.nbk - 1 && cnt[j] > 0) {
            int sc = scene_of_block(scenes, n_scenes, b);
            for (int s = 0; s < cnt[j]; s += cs) {
                if (coff < ws.max_chunks)
                    ws.chunks[coff] = make_int4(b, off + s, min(cs, cnt[j] - s), sc);
                ++coff;
            }
        }
        off += cnt[j];
    }
    if (tile == 0 && threadIdx.x == 0) {
        *ws.n_active_prev = *ws.n_active;
        *ws.n_active = 0;
    }
}

// order[cursor[key]++] = slot, warp-aggregated.  Also zeroes the grid
// accumulator of the previous substep's active blocks (kept until now so
// grid mass/momentum stay readable between substeps).
__global__ void scatter_kernel(PState st, Ws ws, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nclear = *ws.n_active_prev * kBlockNodes;
    for (int j = i; j < nclear; j += gridDim.x * blockDim.x)
        ws.grid_acc[(int64_t)ws.active_list[j >> 6] * kBlockNodes + (j & 63)] = make_float4(0.f, 0.f, 0.f, 0.f);
    int key = i < n ? st.key[i] : -1;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(ws.cursor + key, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) ws.order[base + __popc(peers & ((1u << lane) - 1u))] = i;
}

// physical re-sort: dst[i] = src[order[i]] for every field; order := identity
__global__ void permute_kernel(PState src, PState dst, Ws ws, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = ws.order[i];
    const int64_t s = src.stride;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        dst.x0[i + c * s] = src.x0[j + c * s];
        dst.u[i + c * s] = src.u[j + c * s];
        dst.v[i + c * s] = src.v[j + c * s];
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        dst.C[i + c * s] = src.C[j + c * s];
        dst.F[i + c * s] = src.F[j + c * s];
        dst.tau[i + c * s] = src.tau[j + c * s];
    }
    dst.mass[i] = src.mass[j];
    dst.vol[i] = src.vol[j];
    dst.yld[i] = src.yld[j];
    dst.uid[i] = src.uid[j];
    dst.key[i] = src.key[j];  // G2P rewrites all but the out-of-domain ones
    ws.order[i] = i;
}

cudaError_t launch_keys(const Ctx &cx) {
    if (cx.n == 0) return cudaSuccess;
    key_kernel<<<(cx.n + 255) / 256, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.st, cx.ws,
                                                           cx.n, cx.status);
    return cudaGetLastError();
}

cudaError_t launch_sort(const Ctx &cx) {
    scan_tiles_kernel<<<cx.ws.n_tiles, 256, 0, cx.stream>>>(cx.ws);
    scan_finish_kernel<<<cx.ws.n_tiles, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws);
    const int sgrid = cx.n > 0 ? (cx.n + 255) / 256 : 1;
    scatter_kernel<<<sgrid, 256, 0, cx.stream>>>(cx.st, cx.ws, cx.n);
    return cudaGetLastError();
}

cudaError_t launch_permute(const Ctx &cx, const PState &dst) {
    if (cx.n == 0) return cudaSuccess;
    permute_kernel<<<(cx.n + 255) / 256, 256, 0, cx.stream>>>(cx.st, dst, cx.ws, cx.n);
    return cudaGetLastError();
}

}  // namespace mpm
