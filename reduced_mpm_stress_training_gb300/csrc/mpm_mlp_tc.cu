// Stress-surrogate network forward on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).  Same network, parameter blob
// and bf16 rounding points as mlp_forward_kernel (mpm_mlp.cu):
//   Z_l = H_{l-1} W_l^T + b_l (fp32 accumulate), H_l = bf16(silu(Z_l)).
//
// One CTA = 128 threads = one 128-row tile at a time (persistent over
// tiles).  Operands live in shared memory in the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, K-adjacent core matrices
// 128 B apart (leading byte offset), 8-row groups 256 B apart (stride byte
// offset), one 16-wide K slab per MMA.  A single thread issues the MMAs of a
// layer (M = 128, N = 128 or 16, K = 16 each) into a 128-column TMEM
// accumulator and commits them to an mbarrier; every thread then reads its
// own row (TMEM lane = row) with tcgen05.ld, adds the bias, applies SiLU and
// writes the bf16 activations back as the next layer's A operand.
// Every mbarrier wait is bounded: on timeout the kernel raises an error flag,
// stops issuing work, frees its tensor memory and returns.
#include "mpm_mlp_tc.cuh"
#include "mpm_launch.h"

namespace mpm {
namespace mlptc {

struct TcIO {
    const float *x;        // [n][12]
    float *y;              // [n][6] or null
    const float *target;   // [n][6] or null
    __nv_bfloat16 *z;      // [3][n][128] or null
    __nv_bfloat16 *dy;     // [n][16] or null
    float *loss;           // or null
    float grad_scale;
    int64_t n;
};

__global__ void __launch_bounds__(kThreads, 2) mlp_forward_tc_kernel(const __nv_bfloat16 *__restrict__ w,
                                                                  const float *__restrict__ b, TcIO io,
                                                                  int *__restrict__ err) {
    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    TcSmem &s = *reinterpret_cast<TcSmem *>(tc_smem_raw);
    const int tid = threadIdx.x;
    const uint32_t tbase = tc_setup(s, w, b);
    uint32_t phase = 0;
    bool ok = true;
    const int64_t tiles = (io.n + kRows - 1) / kRows;
    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t row = tile * kRows + (tid & (kRows - 1));
        const bool valid = row < io.n;
        const bool lead = tid < kRows;  // the thread that owns the row's inputs and outputs
        if (lead) {
            float v[12];
#pragma unroll
            for (int k = 0; k < 12; ++k) v[k] = valid ? io.x[row * IN + k] : 0.0f;
            tc_store_inputs(s, v);
        }
        __nv_bfloat16 *z[3] = {nullptr, nullptr, nullptr};
        if (io.z && valid)
            for (int l = 0; l < 3; ++l) z[l] = io.z + (int64_t)l * io.n * H + row * H;
        float out[16];
        ok = tc_tile_forward(s, tbase, phase, out, io.z ? z : nullptr);
        if (!ok) break;
        float lsum = 0.0f;
#pragma unroll
        for (int c = 0; c < N4; ++c) {
            float d = 0.0f;
            if (!lead) break;
            if (valid && c < OUT) {
                if (io.y) io.y[row * OUT + c] = out[c];
                if (io.target) {
                    const float r = out[c] - io.target[row * OUT + c];
                    lsum += r * r;
                    d = io.grad_scale * r;
                }
            }
            if (io.dy && valid) io.dy[row * N4 + c] = __float2bfloat16_rn(d);
        }
        if (io.loss) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
            if ((tid & 31) == 0) atomicAdd(io.loss, lsum);
        }
    }
    if (!ok && tid == 0) atomicOr(err, 1);
    tc_teardown(s, tbase, ok, phase);
}

}  // namespace mlptc

int64_t mlp_tc_smem_bytes() { return (int64_t)sizeof(mlptc::TcSmem); }

cudaError_t launch_mlp_forward_tc(const void *params, const float *x, float *y, const float *target, void *zsave,
                                  void *dy, float *loss, float grad_scale, int64_t n, int *err, int num_sms,
                                  cudaStream_t stream) {
    using namespace mlptc;
    if (n <= 0) return cudaSuccess;
    static bool attr_set[64] = {false};
    const int bytes = (int)mlp_tc_smem_bytes();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(mlp_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(params);
    const float *b = reinterpret_cast<const float *>(static_cast<const char *>(params) + (int64_t)mlp::W_COUNT * 2);
    TcIO io{x, y, target, static_cast<__nv_bfloat16 *>(zsave), static_cast<__nv_bfloat16 *>(dy), loss, grad_scale, n};
    const int64_t tiles = (n + kRows - 1) / kRows;
    const int grid = (int)(tiles < 2 * (int64_t)num_sms ? tiles : 2 * (int64_t)num_sms);
    mlp_forward_tc_kernel<<<grid, kThreads, bytes, stream>>>(w, b, io, err);
    return cudaGetLastError();
}

}  // namespace mpm
