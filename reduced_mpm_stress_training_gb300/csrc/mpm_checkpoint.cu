// Saved grids for the reverse pass: the part of the workspace that the
// adjoint of a substep reads (sorted order, active-block list, the active
// blocks' grid momentum + mass and velocity), copied out after the substep's
// grid update and back in before its reverse pass.  Only active blocks are
// copied.  Blob layout (offsets in bytes, each aligned to 256):
//   0                          int n_active
//   256                        int active_list[total_blocks]
//   L                          int order[n_particles]
//   A                          float4 acc[total_blocks * 64]   (packed in list order)
//   A + total_blocks * 1024    float4 vel[total_blocks * 64]
#include "mpm_launch.h"

namespace mpm {
namespace ckpt {

struct Blob {
    int *n_active;
    int *list;
    int *order;
    float4 *acc;
    float4 *vel;
};

__host__ __device__ inline int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

inline Blob blob_view(void *base, int64_t total_blocks, int64_t n) {
    char *p = static_cast<char *>(base);
    Blob b;
    int64_t o = 0;
    b.n_active = reinterpret_cast<int *>(p + o);
    o += 256;
    b.list = reinterpret_cast<int *>(p + o);
    o += align256(total_blocks * 4);
    b.order = reinterpret_cast<int *>(p + o);
    o += align256(n * 4 > 0 ? n * 4 : 4);
    b.acc = reinterpret_cast<float4 *>(p + o);
    o += total_blocks * kBlockNodes * 16;
    b.vel = reinterpret_cast<float4 *>(p + o);
    return b;
}

__global__ void save_list_kernel(Ws ws, Blob b, int64_t total_blocks) {
    const int na = *ws.n_active;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total_blocks; i += (int64_t)gridDim.x * blockDim.x)
        if (i < na) b.list[i] = ws.active_list[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *b.n_active = na;
}

__global__ void load_list_kernel(Ws ws, Blob b, int64_t total_blocks) {
    const int na = *b.n_active;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total_blocks; i += (int64_t)gridDim.x * blockDim.x)
        if (i < na) ws.active_list[i] = b.list[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *ws.n_active = na;
}

// SAVE: workspace -> blob; otherwise blob -> workspace.  The active count is
// read from the side being copied from.
template <bool SAVE>
__global__ void blocks_kernel(Ws ws, Blob b) {
    const int na = SAVE ? *ws.n_active : *b.n_active;
    const int *list = SAVE ? ws.active_list : b.list;
    const int64_t total = (int64_t)na * kBlockNodes;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
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

int64_t substep_grid_bytes(int64_t total_blocks, int64_t n) {
    return 256 + ckpt::align256(total_blocks * 4) + ckpt::align256(n * 4 > 0 ? n * 4 : 4) +
           2 * total_blocks * kBlockNodes * 16;
}

cudaError_t launch_save_grid(const Ctx &cx, void *dst) {
    using namespace ckpt;
    Blob b = blob_view(dst, cx.total_blocks, cx.n);
    const int g = cx.num_sms * 4;
    save_list_kernel<<<g, 256, 0, cx.stream>>>(cx.ws, b, cx.total_blocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (cx.n > 0) {
        e = cudaMemcpyAsync(b.order, cx.ws.order, (size_t)cx.n * 4, cudaMemcpyDeviceToDevice, cx.stream);
        if (e != cudaSuccess) return e;
    }
    blocks_kernel<true><<<g * 2, 256, 0, cx.stream>>>(cx.ws, b);
    return cudaGetLastError();
}

cudaError_t launch_load_grid(const Ctx &cx, const void *src) {
    using namespace ckpt;
    Blob b = blob_view(const_cast<void *>(src), cx.total_blocks, cx.n);
    const int g = cx.num_sms * 4;
    load_list_kernel<<<g, 256, 0, cx.stream>>>(cx.ws, b, cx.total_blocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (cx.n > 0) {
        e = cudaMemcpyAsync(cx.ws.order, b.order, (size_t)cx.n * 4, cudaMemcpyDeviceToDevice, cx.stream);
        if (e != cudaSuccess) return e;
    }
    blocks_kernel<false><<<g * 2, 256, 0, cx.stream>>>(cx.ws, b);
    return cudaGetLastError();
}

cudaError_t launch_clear_grid(const Ctx &cx) {
    cudaError_t e = cudaMemsetAsync(cx.ws.grid_acc, 0, (size_t)cx.total_blocks * kBlockNodes * 16, cx.stream);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(cx.ws.n_active, 0, sizeof(int), cx.stream);
}

}  // namespace mpm
