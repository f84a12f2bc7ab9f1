// Ordered P2G: grid sums that do not depend on the order in which warps run.
//
// The regular P2G (p2g_kernel) is exact up to float32 rounding, but two
// things make its rounding vary from run to run: the sort's scatter places
// the particles of one cell in the order in which warps reach the cell's
// cursor, and the per-block tiles are flushed into the grid with float
// atomics from up to eight warps per node.  A finite-difference check of a
// gradient compares two forward runs whose inputs differ by 1e-3 relative;
// that needs the forward to be a deterministic function of its inputs.
// This mode removes both sources:
//   canonical_cells_kernel -- each cell's range of order[] sorted by particle
//                             uid (the user's index), so every run sums its
//                             particles in the same order
//   p2g_kernel (ordered)   -- each non-empty block's 6x6x6 tile written whole
//                             to its own slot instead of atomics
//   gather_partials_kernel -- each node of an active grid block sums the
//                             <= 8 tiles that cover it in a fixed order
//                             (source block offsets (0,0,0), (0,0,1), ...,
//                             (1,1,1)) into grid_acc
// The grid update and G2P that follow are per node / per particle and
// deterministic already.  Results equal the regular P2G's up to float32
// rounding (the same terms, summed in another order).
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

namespace {

constexpr int64_t kAlignBytes = 256;
inline int64_t align_up(int64_t x) { return (x + kAlignBytes - 1) / kAlignBytes * kAlignBytes; }

__device__ __forceinline__ int rec_uid(const PState &st, int slot) {
    return __float_as_int(ldrec(st, slot, 1).y);
}

// one thread per (work-list block, cell): insertion sort of the cell's range
// of order[] by uid.  Cells hold a handful of particles; the sort is
// quadratic in the cell's count.
__global__ void __launch_bounds__(256) canonical_cells_kernel(PState st, Ws ws) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int bi = (int)(t >> 6), c = (int)(t & 63);
    if (bi >= *ws.n_blocks) return;
    const int4 be = ws.blocks[bi];
    if ((unsigned)be.x >= (unsigned)(ws.nbk - 1)) return;
    const int64_t cell = (int64_t)be.x * 64 + c;
    const int s = ws.cell_start[cell], e = ws.cell_cursor[cell];
    if (s < 0 || e > ws.n || e - s < 2) return;
    int *o = ws.order;
    for (int i = s + 1; i < e; ++i) {
        const int slot = o[i];
        if ((unsigned)slot >= (unsigned)ws.n) return;  // damaged list: leave it
        const int uid = rec_uid(st, slot);
        int j = i - 1;
        while (j >= s) {
            const int sj = o[j];
            if (rec_uid(st, sj) <= uid) break;
            o[j + 1] = sj;
            --j;
        }
        o[j + 1] = slot;
    }
}

// one thread per node of each active grid block: grid_acc = the sum of the
// tiles of the (up to 8) non-empty blocks whose 6x6x6 tile covers the node,
// in the fixed order of the source block offsets
__global__ void __launch_bounds__(256) gather_partials_kernel(const MpmScene *__restrict__ scenes, int n_scenes,
                                                              Ws ws, const float4 *__restrict__ partials,
                                                              const int *__restrict__ blk_index) {
    const int n_active = *ws.n_active;
    const int l = threadIdx.x & 63;
    for (int base = blockIdx.x * 4; base < n_active; base += gridDim.x * 4) {
        const int li = base + (threadIdx.x >> 6);
        if (li >= n_active) continue;
        const int gb = ws.active_list[li];
        const MpmScene &S = scenes[scene_of_block(scenes, n_scenes, gb)];
        const int nb = S.n_blocks_axis;
        int bx, by, bz;
        chunk_block(S, gb, bx, by, bz);
        const int lx = l >> 4, ly = (l >> 2) & 3, lz = l & 3;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int dx = d >> 2, dy = (d >> 1) & 1, dz = d & 1;
            const int sx = bx - dx, sy = by - dy, sz = bz - dz;
            const int tx = 4 * dx + lx, ty = 4 * dy + ly, tz = 4 * dz + lz;
            if (sx < 0 || sy < 0 || sz < 0 || tx >= kTile || ty >= kTile || tz >= kTile) continue;
            const int64_t sb = S.block_begin + ((int64_t)(sx * nb + sy) * nb + sz);
            const int idx = blk_index[sb];
            if (idx < 0) continue;
            const float4 p = partials[(int64_t)idx * kTileNodes + (tx * kTile + ty) * kTile + tz];
            acc.x += p.x;
            acc.y += p.y;
            acc.z += p.z;
            acc.w += p.w;
        }
        ws.grid_acc[(int64_t)gb * kBlockNodes + l] = acc;
    }
}

}  // namespace

int64_t ordered_scratch_bytes(int64_t total_blocks) {
    return align_up(total_blocks * kTileNodes * 16) + align_up(total_blocks * 4);
}

cudaError_t launch_p2g_ordered(const Ctx &cx, float dt, void *scratch) {
    float4 *partials = static_cast<float4 *>(scratch);
    int *blk_index = reinterpret_cast<int *>(static_cast<char *>(scratch) +
                                             align_up(cx.total_blocks * kTileNodes * 16));
    cudaError_t e = cudaMemsetAsync(blk_index, 0xff, (size_t)cx.total_blocks * sizeof(int), cx.stream);
    if (e != cudaSuccess) return e;
    const int64_t threads = cx.total_blocks * 64;
    if (threads > 0) {
        canonical_cells_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, cx.stream>>>(cx.st, cx.ws);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = launch_p2g(cx, dt, partials, blk_index)) != cudaSuccess) return e;
    int64_t want = (cx.total_blocks + 3) / 4;
    int grid = (int)(want < (int64_t)cx.num_sms * 8 ? want : (int64_t)cx.num_sms * 8);
    if (grid < 1) grid = 1;
    gather_partials_kernel<<<grid, 256, 0, cx.stream>>>(cx.scenes, cx.n_scenes, cx.ws, partials, blk_index);
    return cudaGetLastError();
}

}  // namespace mpm
