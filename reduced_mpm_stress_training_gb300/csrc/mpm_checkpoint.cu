// Saved grids for the reverse pass: the part of the workspace that the
// adjoint of a substep and the substep's G2P read (sorted order, active-block
// list, G2P chunk list, the active blocks' grid momentum + mass and
// velocity), copied out after the substep's grid update and back in before
// its reverse pass (or before re-running its G2P).  Only active blocks are
// copied.  Blob layout (offsets in bytes, each aligned to 256):
//   0                          int n_active, int n_chunks
//   256                        int active_list[total_blocks]
//   L                          int order[n_particles]
//   H                          int4 chunks[max_chunks]
//   A                          float4 acc[total_blocks * 64]   (packed in list order)
//   A + total_blocks * 1024    float4 vel[total_blocks * 64]
#include "mpm_launch.h"

namespace mpm {
namespace ckpt {

struct Blob {
    int *n_active;
    int *n_chunks;
    int *list;
    int *order;
    int4 *chunks;
    float4 *acc;
    float4 *vel;
};

__host__ __device__ inline int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

inline Blob blob_view(void *base, int64_t total_blocks, int64_t n, int64_t max_chunks) {
    char *p = static_cast<char *>(base);
    Blob b;
    int64_t o = 0;
    b.n_active = reinterpret_cast<int *>(p + o);
    b.n_chunks = b.n_active + 1;
    o += 256;
    b.list = reinterpret_cast<int *>(p + o);
    o += align256(total_blocks * 4);
    b.order = reinterpret_cast<int *>(p + o);
    o += align256(n * 4 > 0 ? n * 4 : 4);
    b.chunks = reinterpret_cast<int4 *>(p + o);
    o += align256(max_chunks * 16);
    b.acc = reinterpret_cast<float4 *>(p + o);
    o += total_blocks * kBlockNodes * 16;
    b.vel = reinterpret_cast<float4 *>(p + o);
    return b;
}

// SAVE: workspace -> blob; otherwise blob -> workspace, in one launch.
// Counts and the active-block list are read from the side being copied from.
template <bool SAVE>
__global__ void blob_kernel(Ws ws, Blob b, int n) {
    const int na = SAVE ? *ws.n_active : *b.n_active;
    const int nc = min(SAVE ? *ws.n_chunks : *b.n_chunks, ws.max_chunks);
    const int *list = SAVE ? ws.active_list : b.list;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if (tid == 0) {
        if (SAVE) {
            *b.n_active = na;
            *b.n_chunks = nc;
        } else {
            *ws.n_active = na;
            *ws.n_chunks = nc;
        }
    }
    for (int64_t i = tid; i < na; i += stride) {
        if (SAVE) b.list[i] = ws.active_list[i];
        else ws.active_list[i] = b.list[i];
    }
    for (int64_t i = tid; i < n; i += stride) {
        if (SAVE) b.order[i] = ws.order[i];
        else ws.order[i] = b.order[i];
    }
    for (int64_t i = tid; i < nc; i += stride) {
        if (SAVE) b.chunks[i] = ws.chunks[i];
        else ws.chunks[i] = b.chunks[i];
    }
    const int64_t total = (int64_t)na * kBlockNodes;
    for (int64_t i = tid; i < total; i += stride) {
        const int64_t g = (int64_t)list[i / kBlockNodes] * kBlockNodes + (i % kBlockNodes);
        if (SAVE) {
            b.acc[i] = ws.grid_acc[g];
            b.vel[i] = ws.grid_v[g];
        } else {
            ws.grid_acc[g] = b.acc[i];
            ws.grid_v[g] = b.vel[i];
        }
    }
}

}  // namespace ckpt

int64_t substep_grid_bytes(int64_t total_blocks, int64_t n, int64_t max_chunks) {
    return 256 + ckpt::align256(total_blocks * 4) + ckpt::align256(n * 4 > 0 ? n * 4 : 4) +
           ckpt::align256(max_chunks * 16) + 2 * total_blocks * kBlockNodes * 16;
}

cudaError_t launch_save_grid(const Ctx &cx, void *dst) {
    using namespace ckpt;
    Blob b = blob_view(dst, cx.total_blocks, cx.n, cx.ws.max_chunks);
    blob_kernel<true><<<cx.num_sms * 8, 256, 0, cx.stream>>>(cx.ws, b, (int)cx.n);
    return cudaGetLastError();
}

cudaError_t launch_load_grid(const Ctx &cx, const void *src) {
    using namespace ckpt;
    Blob b = blob_view(const_cast<void *>(src), cx.total_blocks, cx.n, cx.ws.max_chunks);
    blob_kernel<false><<<cx.num_sms * 8, 256, 0, cx.stream>>>(cx.ws, b, (int)cx.n);
    return cudaGetLastError();
}

cudaError_t launch_clear_grid(const Ctx &cx) {
    cudaError_t e = cudaMemsetAsync(cx.ws.grid_acc, 0, (size_t)cx.total_blocks * kBlockNodes * 16, cx.stream);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(cx.ws.n_active, 0, sizeof(int), cx.stream);
}

}  // namespace mpm
