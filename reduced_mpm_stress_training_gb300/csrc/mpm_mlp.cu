// Stress surrogate MLP: 12 -> 128 -> 128 -> 128 -> 6, SiLU, BF16 weights and
// activations, FP32 accumulation, on the BF16 tensor cores (mma.sync m16n8k16).
//
// Parameters live in one device buffer (mpm_mlp_param_bytes):
//   W1 bf16 [128][16]   (input padded 12 -> 16 with zero columns)
//   W2 bf16 [128][128], W3 bf16 [128][128]
//   W4 bf16 [16][128]   (output padded 6 -> 16 with zero rows)
//   b1, b2, b3 f32 [128], b4 f32 [16]
// Kernels:
//   mlp_forward_kernel  fused 4-layer forward, one warp per 16 rows, all
//                       activations register-resident (the m16n8 accumulator
//                       fragments of one layer are the A fragments of the
//                       next); optional loss gradient and saved pre-activations
//   mlp_dgrad_kernel    dZ_l = (dZ_{l+1} W_{l+1}) * silu'(Z_l)
//   mlp_wgrad_kernel    dW_l += dZ_l^T H_{l-1}, db_l += sum dZ_l   (row-split, fp32 atomics)
//   mlp_adam_kernel     Adam on fp32 master weights, refreshes the bf16 copy
#include "mpm_mlp.cuh"
#include "mpm_launch.h"

namespace mpm {
namespace mlp {

// Forward of a warp's 16 rows whose 12 inputs are x(row, i); writes outputs y(row, j).
// Optional: save Z1..Z3 (training) and the loss gradient dY = 2 (y - target) * scale.
struct FwdIO {
    const float *x;        // [n][12]
    float *y;              // [n][6]
    const float *target;   // [n][6] or null
    __nv_bfloat16 *z;      // [3][n][128] or null
    __nv_bfloat16 *dy;     // [n][16] loss gradient (bf16) or null
    float *loss;           // sum of squared errors (atomic) or null
    float grad_scale;      // d(loss)/dy = grad_scale * (y - target)
    int64_t n;
};

__device__ __forceinline__ void mlp_rows(const WSmem &s, const uint32_t a1[1][4], int64_t row0,
                                         const FwdIO &io) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float out[2][4];
    mlp_core(s, a1, out, io.z, row0, io.n);
    float lsum = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // rows g, g+8
            const int64_t row = row0 + g + 8 * h;
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int col = nt * 8 + 2 * t + e;
                const float yv = out[nt][2 * h + e];
                float d = 0.0f;
                if (col < OUT && row < io.n) {
                    if (io.y) io.y[row * OUT + col] = yv;
                    if (io.target) {
                        const float r = yv - io.target[row * OUT + col];
                        lsum += r * r;
                        d = io.grad_scale * r;
                    }
                }
                if (io.dy && row < io.n) io.dy[row * N4 + col] = __float2bfloat16_rn(d);
            }
        }
    }
    if (io.loss) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if (lane == 0) atomicAdd(io.loss, lsum);
    }
}

// A fragment (16 rows x 16 inputs, inputs 12..15 zero) from a row-major [n][12] f32 array
__device__ __forceinline__ void a1_from_x(uint32_t a1[1][4], const float *x, int64_t row0, int64_t n) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float v[2][2][2];  // [row half][k half][pair]
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int kh = 0; kh < 2; ++kh)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int64_t row = row0 + g + 8 * h;
                const int k = 2 * t + e + 8 * kh;
                v[h][kh][e] = (row < n && k < IN) ? x[row * IN + k] : 0.0f;
            }
    a1[0][0] = pack_bf16(v[0][0][0], v[0][0][1]);
    a1[0][1] = pack_bf16(v[1][0][0], v[1][0][1]);
    a1[0][2] = pack_bf16(v[0][1][0], v[0][1][1]);
    a1[0][3] = pack_bf16(v[1][1][0], v[1][1][1]);
}

__global__ void __launch_bounds__(256) mlp_forward_kernel(const __nv_bfloat16 *__restrict__ w,
                                                          const float *__restrict__ b, FwdIO io) {
    extern __shared__ __align__(16) unsigned char mlp_smem[];
    WSmem &s = *reinterpret_cast<WSmem *>(mlp_smem);
    load_weights(s, w, b);
    __syncthreads();
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int64_t tiles = (io.n + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * nwarps + warp; tile < tiles; tile += (int64_t)gridDim.x * nwarps) {
        uint32_t a1[1][4];
        a1_from_x(a1, io.x, tile * 16, io.n);
        mlp_rows(s, a1, tile * 16, io);
    }
}

// ---------------------------------------------------------------------------
// Backward.  dgrad: dZ_l[rows][128] = (dZ_{l+1}[rows][Nn] W_{l+1}) * silu'(Z_l)
// with W_{l+1} stored [Nn][128] row-major (= the B operand [k = Nn][n = 128]).
// One warp per 16 rows; dZ_{l+1} rows and W_{l+1} staged in shared memory.
// ---------------------------------------------------------------------------
template <int NN>  // width of dZ_{l+1}: 128 (hidden) or 16 (output, padded)
__global__ void __launch_bounds__(128) mlp_dgrad_kernel(const __nv_bfloat16 *__restrict__ dz_next,
                                                        const __nv_bfloat16 *__restrict__ wnext,
                                                        const __nv_bfloat16 *__restrict__ z,
                                                        __nv_bfloat16 *__restrict__ dz, int64_t n) {
    constexpr int LDA = NN + 8;
    extern __shared__ __align__(16) unsigned char mlp_smem[];
    __nv_bfloat16 *ws = reinterpret_cast<__nv_bfloat16 *>(mlp_smem);  // [NN][LDW]
    __nv_bfloat16 (*as)[16 * LDA] = reinterpret_cast<__nv_bfloat16 (*)[16 * LDA]>(ws + NN * LDW);
    for (int i = threadIdx.x; i < NN * (H / 8); i += blockDim.x)
        *reinterpret_cast<uint4 *>(ws + (i / (H / 8)) * LDW + (i % (H / 8)) * 8) =
            reinterpret_cast<const uint4 *>(wnext)[i];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __syncthreads();
    const int64_t tiles = (n + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * 4 + warp; tile < tiles; tile += (int64_t)gridDim.x * 4) {
        const int64_t row0 = tile * 16;
        __nv_bfloat16 *a_s = as[warp];
        for (int i = lane; i < 16 * (NN / 8); i += 32) {
            const int r = i / (NN / 8), c = i % (NN / 8);
            const uint4 v = (row0 + r < n) ? reinterpret_cast<const uint4 *>(dz_next + (row0 + r) * NN)[c]
                                           : make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4 *>(a_s + r * LDA + c * 8) = v;
        }
        __syncwarp();
        float acc[16][4];
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < NN / 16; ++kt) {
            uint32_t a[4];
            {
                const int r = (lane & 7) + ((lane >> 3) & 1) * 8, c = (lane >> 4) * 8;
                ldsm_x4(a, a_s + r * LDA + kt * 16 + c);
            }
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) {
                uint32_t bb[2];
                const int l = lane & 15;
                ldsm_x2_trans(bb, ws + (kt * 16 + (l & 7) + ((l >> 3) << 3)) * LDW + nt * 8);
                mma16816(acc[nt], a, bb[0], bb[1]);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
            const int col = nt * 8 + 2 * t;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t row = row0 + g + 8 * h;
                if (row < n) {
                    const float2 zz = unpack_bf16(*reinterpret_cast<const uint32_t *>(z + row * H + col));
                    *reinterpret_cast<uint32_t *>(dz + row * H + col) =
                        pack_bf16(acc[nt][2 * h] * silu_grad(zz.x), acc[nt][2 * h + 1] * silu_grad(zz.y));
                }
            }
        }
        __syncwarp();
    }
}

// wgrad: dW[NO][KI] += sum_rows dZ[rows][NO]^T * Hp[rows][KI], Hp = silu(Zp) (or the
// input x for the first layer), db[NO] += sum_rows dZ.  A CTA takes a slab of
// rows; 16 warps = 4 x 4 tiles of the (NO x KI) output when both are 128.
template <int NO, int KI, bool FIRST>
__global__ void __launch_bounds__(128) mlp_wgrad_kernel(const __nv_bfloat16 *__restrict__ dz,
                                                        const __nv_bfloat16 *__restrict__ zp,
                                                        const float *__restrict__ x, float *__restrict__ dw,
                                                        float *__restrict__ db, int64_t n, int rows_per_cta) {
    constexpr int LDD = NO + 8, LDH = KI + 8, RT = 32;  // rows staged per step
    __shared__ __align__(16) __nv_bfloat16 ds[RT * LDD];
    __shared__ __align__(16) __nv_bfloat16 hs[RT * LDH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // warp tile of the output: MT m16 tiles x NT n8 tiles
    constexpr int MT_ALL = NO / 16, NT_ALL = KI / 8;
    constexpr int WM = (MT_ALL >= 4) ? 4 : MT_ALL;  // warps along m
    constexpr int WN = 4 / WM;                       // warps along n
    constexpr int MT = MT_ALL / WM, NT = NT_ALL / WN;
    const int wm = warp % WM, wn = warp / WM;
    float acc[MT][NT][4];
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.0f;
    float dbs = 0.0f;  // bias gradient of column threadIdx.x (< NO)
    const int64_t r_begin = (int64_t)blockIdx.x * rows_per_cta;
    const int64_t r_end = min(n, r_begin + rows_per_cta);
    for (int64_t r0 = r_begin; r0 < r_end; r0 += RT) {
        __syncthreads();
        for (int i = threadIdx.x; i < RT * (NO / 8); i += blockDim.x) {
            const int r = i / (NO / 8), c = i % (NO / 8);
            const uint4 v = (r0 + r < r_end) ? reinterpret_cast<const uint4 *>(dz + (r0 + r) * NO)[c]
                                             : make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4 *>(ds + r * LDD + c * 8) = v;
        }
        if (FIRST) {
            for (int i = threadIdx.x; i < RT * KI; i += blockDim.x) {
                const int r = i / KI, c = i % KI;
                const float v = (r0 + r < r_end && c < IN) ? x[(r0 + r) * IN + c] : 0.0f;
                hs[r * LDH + c] = __float2bfloat16_rn(v);
            }
        } else {
            // H = bf16(silu(Z)), eight activations per 16-byte word
            for (int i = threadIdx.x; i < RT * (KI / 8); i += blockDim.x) {
                const int r = i / (KI / 8), c = i % (KI / 8);
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (r0 + r < r_end) {
                    v = reinterpret_cast<const uint4 *>(zp + (r0 + r) * KI)[c];
                    uint32_t *u = reinterpret_cast<uint32_t *>(&v);
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const float2 zz = unpack_bf16(u[k]);
                        u[k] = pack_bf16(silu(zz.x), silu(zz.y));
                    }
                }
                *reinterpret_cast<uint4 *>(hs + r * LDH + c * 8) = v;
            }
        }
        __syncthreads();
        if (threadIdx.x < NO)
            for (int r = 0; r < RT; ++r) dbs += __bfloat162float(ds[r * LDD + threadIdx.x]);
#pragma unroll
        for (int kt = 0; kt < RT / 16; ++kt) {
#pragma unroll
            for (int i = 0; i < MT; ++i) {
                // A = dZ^T: [m = out][k = row], stored as ds[row][out] -> transposed ldmatrix
                uint32_t a[4];
                {
                    const int q = lane >> 3, l = lane & 7;
                    const int krow = kt * 16 + l + ((q >> 1) << 3);
                    const int mcol = (wm * MT + i) * 16 + ((q & 1) << 3);
                    ldsm_x4_trans(a, ds + krow * LDD + mcol);
                }
#pragma unroll
                for (int j = 0; j < NT; ++j) {
                    // B = Hp: [k = row][n = in], stored row-major -> transposed ldmatrix
                    uint32_t bb[2];
                    const int l = lane & 15;
                    ldsm_x2_trans(bb, hs + (kt * 16 + (l & 7) + ((l >> 3) << 3)) * LDH + (wn * NT + j) * 8);
                    mma16816(acc[i][j], a, bb[0], bb[1]);
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int m = (wm * MT + i) * 16 + g, c = (wn * NT + j) * 8 + 2 * t;
            atomicAdd(dw + m * KI + c, acc[i][j][0]);
            atomicAdd(dw + m * KI + c + 1, acc[i][j][1]);
            atomicAdd(dw + (m + 8) * KI + c, acc[i][j][2]);
            atomicAdd(dw + (m + 8) * KI + c + 1, acc[i][j][3]);
        }
    if (threadIdx.x < NO) atomicAdd(db + threadIdx.x, dbs);
}

// Adam on fp32 master parameters (weights then biases, one flat array); refreshes
// the bf16 weight copy.  Padded weight entries (inputs 12..15, outputs 6..15) stay 0.
__global__ void mlp_adam_kernel(float *__restrict__ master, float *__restrict__ m, float *__restrict__ v,
                                const float *__restrict__ grad, __nv_bfloat16 *__restrict__ wbf,
                                float *__restrict__ bias, int count, float lr, float b1, float b2,
                                float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    bool pad = false;
    if (i < W_COUNT) {
        if (i < W2_OFF) pad = (i % K1) >= IN;
        else if (i >= W4_OFF) pad = ((i - W4_OFF) / H) >= OUT;
    } else if (i - W_COUNT >= B4_OFF + OUT) {
        pad = true;
    }
    float p = master[i];
    if (!pad) {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gr;
        const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        p -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    } else {
        p = 0.0f;
    }
    master[i] = p;
    if (i < W_COUNT) wbf[i] = __float2bfloat16_rn(p);
    else bias[i - W_COUNT] = p;
}

}  // namespace mlp
}  // namespace mpm

using namespace mpm::mlp;

static int num_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
        return 1;
    return n;
}

// persistent grids: at most `per_sm` CTAs per SM, never more CTAs than work
static int mlp_grid(int64_t tiles, int tiles_per_cta, int per_sm) {
    const int64_t want = (tiles + tiles_per_cta - 1) / tiles_per_cta;
    const int64_t cap = (int64_t)num_sms() * per_sm;
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

template <int NN>
constexpr int dgrad_smem() { return (NN * LDW + 4 * 16 * (NN + 8)) * 2; }

// Opt the kernels that use more than 48 KB of dynamic shared memory in, once per device.
static cudaError_t mlp_attrs() {
    static bool set[64] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !set[dev]) {
        e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(WSmem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mlp_dgrad_kernel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     dgrad_smem<H>());
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mlp_dgrad_kernel<N4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     dgrad_smem<N4>());
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) set[dev] = true;
    }
    return cudaSuccess;
}


extern "C" {

int64_t mpm_mlp_param_bytes(void) { return PARAM_BYTES; }


// Forward (and, with target != NULL, loss gradient); see include/mpm_gb300.h.
int mpm_mlp_forward(const void *params, const float *x, float *y, const float *target,
                    void *zsave, void *dy, float *loss, float grad_scale, int64_t n, void *stream) {
    if (!params || n < 0 || (n > 0 && !x)) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(params) & 15) return MPM_ERR_ARG;
    if (n == 0) return MPM_OK;
    if (mlp_attrs() != cudaSuccess) return MPM_ERR_CUDA;
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(params);
    const float *b = reinterpret_cast<const float *>(static_cast<const char *>(params) + (int64_t)W_COUNT * 2);
    FwdIO io{x, y, target, static_cast<__nv_bfloat16 *>(zsave), static_cast<__nv_bfloat16 *>(dy), loss,
             grad_scale, n};
    mlp_forward_kernel<<<mlp_grid((n + 15) / 16, 8, 1), 256, sizeof(WSmem), static_cast<cudaStream_t>(stream)>>>(
        w, b, io);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

// Backward for one batch: accumulates (adds) into grad (fp32, same flat layout as
// the parameters: weights then biases).
int mpm_mlp_backward(const void *params, const float *x, const void *zsave, const void *dy, void *work,
                     float *grad, int64_t n, void *stream) {
    if (!params || !x || !zsave || !dy || !work || !grad || n <= 0) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(params) & 15) return MPM_ERR_ARG;
    if (mlp_attrs() != cudaSuccess) return MPM_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(params);
    const __nv_bfloat16 *z = static_cast<const __nv_bfloat16 *>(zsave);
    __nv_bfloat16 *dz3 = static_cast<__nv_bfloat16 *>(work);  // [n][128] x 2 scratch
    __nv_bfloat16 *dz2 = dz3 + n * H;
    float *gw = grad, *gb = grad + W_COUNT;
    // wgrad: at most 2 CTAs per SM, each over a contiguous slab of rows (a multiple of 32)
    int64_t rows64 = (n + 303) / 304;
    rows64 = ((rows64 + 31) / 32) * 32;
    if (rows64 < 64) rows64 = 64;
    const int rows = (int)rows64;
    const int gridw = (int)((n + rows - 1) / rows);
    const int gridd = mlp_grid((n + 15) / 16, 4, 4);
    const __nv_bfloat16 *dyb = static_cast<const __nv_bfloat16 *>(dy);
    // layer 4: dW4 += dY^T H3, dZ3 = (dY W4) * silu'(Z3)
    mlp_wgrad_kernel<N4, H, false><<<gridw, 128, 0, st>>>(dyb, z + 2 * n * H, nullptr, gw + W4_OFF, gb + B4_OFF, n, rows);
    mlp_dgrad_kernel<N4><<<gridd, 128, dgrad_smem<N4>(), st>>>(dyb, w + W4_OFF, z + 2 * n * H, dz3, n);
    // layer 3
    mlp_wgrad_kernel<H, H, false><<<gridw, 128, 0, st>>>(dz3, z + 1 * n * H, nullptr, gw + W3_OFF, gb + B3_OFF, n, rows);
    mlp_dgrad_kernel<H><<<gridd, 128, dgrad_smem<H>(), st>>>(dz3, w + W3_OFF, z + 1 * n * H, dz2, n);
    // layer 2
    mlp_wgrad_kernel<H, H, false><<<gridw, 128, 0, st>>>(dz2, z + 0 * n * H, nullptr, gw + W2_OFF, gb + B2_OFF, n, rows);
    mlp_dgrad_kernel<H><<<gridd, 128, dgrad_smem<H>(), st>>>(dz2, w + W2_OFF, z + 0 * n * H, dz3, n);
    // layer 1: dW1 += dZ1^T X
    mlp_wgrad_kernel<H, K1, true><<<gridw, 128, 0, st>>>(dz3, nullptr, x, gw + W1_OFF, gb + B1_OFF, n, rows);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

int mpm_mlp_adam(float *master, float *m, float *v, const float *grad, void *params, float lr, float beta1,
                 float beta2, float eps, int32_t step, void *stream) {
    if (!master || !m || !v || !grad || !params || step < 1) return MPM_ERR_ARG;
    const int count = W_COUNT + B_COUNT;
    const float c1 = 1.0f / (1.0f - powf(beta1, (float)step));
    const float c2 = 1.0f / (1.0f - powf(beta2, (float)step));
    __nv_bfloat16 *wbf = static_cast<__nv_bfloat16 *>(params);
    float *bias = reinterpret_cast<float *>(static_cast<char *>(params) + (int64_t)W_COUNT * 2);
    mlp_adam_kernel<<<(count + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        master, m, v, grad, wbf, bias, count, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

}  // extern "C"
