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
#include <cuda_bf16.h>
#include <stdint.h>

#include "mpm_launch.h"

namespace mpm {
namespace mlp {

constexpr int IN = 12, K1 = 16, H = 128, OUT = 6, N4 = 16;
constexpr int W1_OFF = 0, W2_OFF = W1_OFF + H * K1, W3_OFF = W2_OFF + H * H, W4_OFF = W3_OFF + H * H,
              W_COUNT = W4_OFF + N4 * H;  // bf16 elements
constexpr int B1_OFF = 0, B2_OFF = H, B3_OFF = 2 * H, B4_OFF = 3 * H, B_COUNT = 3 * H + N4;  // f32
constexpr int64_t PARAM_BYTES = (int64_t)W_COUNT * 2 + (int64_t)B_COUNT * 4;
constexpr int LDW = H + 8;   // padded smem row (bf16) of a 128-wide matrix: conflict-free ldmatrix
constexpr int LDW1 = K1 + 8; // padded smem row of W1

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162 *>(&u);
    return __bfloat1622float2(v);
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(uint32_t r[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_trans(uint32_t r[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(smem_u32(p)));
}

// ---------------------------------------------------------------------------
// Weights in shared memory, rows padded for conflict-free ldmatrix.
// ---------------------------------------------------------------------------
struct WSmem {
    __nv_bfloat16 w1[H * LDW1];
    __nv_bfloat16 w2[H * LDW];
    __nv_bfloat16 w3[H * LDW];
    __nv_bfloat16 w4[N4 * LDW];
    float b[B_COUNT];
};

__device__ void load_weights(WSmem &s, const __nv_bfloat16 *w, const float *b) {
    for (int i = threadIdx.x; i < H * K1; i += blockDim.x) s.w1[(i / K1) * LDW1 + i % K1] = w[W1_OFF + i];
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        s.w2[(i / H) * LDW + i % H] = w[W2_OFF + i];
        s.w3[(i / H) * LDW + i % H] = w[W3_OFF + i];
    }
    for (int i = threadIdx.x; i < N4 * H; i += blockDim.x) s.w4[(i / H) * LDW + i % H] = w[W4_OFF + i];
    for (int i = threadIdx.x; i < B_COUNT; i += blockDim.x) s.b[i] = b[i];
}

// B fragment (n8 x k16, "col" operand) from a weight matrix stored [n][k]:
// lanes 0-7 address rows n0..n0+7 at k0, lanes 8-15 at k0+8.
__device__ __forceinline__ void b_frag(uint32_t r[2], const __nv_bfloat16 *w, int ld, int n0, int k0) {
    const int l = threadIdx.x & 15;
    ldsm_x2(r, w + (n0 + (l & 7)) * ld + k0 + ((l >> 3) << 3));
}

// One dense layer on a warp's 16 rows: acc[nt][4] = A(16 x K) * W^T, W [128][K] in smem.
template <int KT>  // number of k16 steps
__device__ __forceinline__ void layer_mma(float acc[16][4], const uint32_t a[KT][4], const __nv_bfloat16 *w,
                                          int ld) {
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            uint32_t b[2];
            b_frag(b, w, ld, nt * 8, kt * 16);
            mma16816(acc[nt], a[kt], b[0], b[1]);
        }
    }
}

// bias + SiLU on accumulators, then pack as the A fragments (k = the 128 features)
// of the next layer; optionally save the pre-activations Z (bf16, row-major [rows][128]).
__device__ __forceinline__ void act_to_a(float acc[16][4], const float *bias, uint32_t a[8][4],
                                         __nv_bfloat16 *zsave, int64_t row0, int64_t n_rows) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const int col = nt * 8 + 2 * t;
        const float z0 = acc[nt][0] + bias[col], z1 = acc[nt][1] + bias[col + 1];
        const float z2 = acc[nt][2] + bias[col], z3 = acc[nt][3] + bias[col + 1];
        if (zsave) {
            if (row0 + g < n_rows)
                *reinterpret_cast<uint32_t *>(zsave + (row0 + g) * H + col) = pack_bf16(z0, z1);
            if (row0 + g + 8 < n_rows)
                *reinterpret_cast<uint32_t *>(zsave + (row0 + g + 8) * H + col) = pack_bf16(z2, z3);
        }
        acc[nt][0] = silu(z0); acc[nt][1] = silu(z1); acc[nt][2] = silu(z2); acc[nt][3] = silu(z3);
    }
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
        a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
        a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
        a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
        a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
    }
}

// Forward of a warp's 16 rows whose 12 inputs are x(row, i); writes outputs y(row, j).
// Optional: save Z1..Z3 (training) and the loss gradient dY = 2 (y - target) * scale.
struct FwdIO {
    const float *x;        // [n][12] or null (then x comes from a functor in the caller)
    float *y;              // [n][6]
    const float *target;   // [n][6] or null
    __nv_bfloat16 *z;      // [3][n][128] or null
    __nv_bfloat16 *dy;     // [n][16] loss gradient (bf16) or null
    float *loss;           // sum of squared errors (atomic) or null
    float grad_scale;      // d(loss)/dy = grad_scale * (y - target)
    int64_t n;
};

__device__ __forceinline__ void mlp_rows(const WSmem &s, const float xin[2][2][2][2] /*unused*/,
                                         uint32_t a1[1][4], int64_t row0, const FwdIO &io) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[16][4];
    uint32_t a[8][4];
    layer_mma<1>(acc, a1, s.w1, LDW1);
    act_to_a(acc, s.b + B1_OFF, a, io.z ? io.z + 0 * io.n * H : nullptr, row0, io.n);
    layer_mma<8>(acc, a, s.w2, LDW);
    act_to_a(acc, s.b + B2_OFF, a, io.z ? io.z + 1 * io.n * H : nullptr, row0, io.n);
    layer_mma<8>(acc, a, s.w3, LDW);
    act_to_a(acc, s.b + B3_OFF, a, io.z ? io.z + 2 * io.n * H : nullptr, row0, io.n);
    // output layer: N = 16 (two n8 tiles), K = 128
    float out[2][4];
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
        out[nt][0] = out[nt][1] = out[nt][2] = out[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 8; ++kt) {
            uint32_t b[2];
            b_frag(b, s.w4, LDW, nt * 8, kt * 16);
            mma16816(out[nt], a[kt], b[0], b[1]);
        }
    }
    float lsum = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // rows g, g+8
            const int64_t row = row0 + g + 8 * h;
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int col = nt * 8 + 2 * t + e;
                const float yv = out[nt][2 * h + e] + s.b[B4_OFF + col];
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
        mlp_rows(s, nullptr, a1, tile * 16, io);
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
    for (int i = threadIdx.x; i < NN * H; i += blockDim.x) ws[(i / H) * LDW + i % H] = wnext[i];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __syncthreads();
    const int64_t tiles = (n + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * 4 + warp; tile < tiles; tile += (int64_t)gridDim.x * 4) {
        const int64_t row0 = tile * 16;
        __nv_bfloat16 *a_s = as[warp];
        for (int i = lane; i < 16 * NN; i += 32) {
            const int r = i / NN, c = i % NN;
            a_s[r * LDA + c] = (row0 + r < n) ? dz_next[(row0 + r) * NN + c] : __float2bfloat16_rn(0.0f);
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
        for (int i = threadIdx.x; i < RT * NO; i += blockDim.x) {
            const int r = i / NO, c = i % NO;
            ds[r * LDD + c] = (r0 + r < r_end) ? dz[(r0 + r) * NO + c] : __float2bfloat16_rn(0.0f);
        }
        for (int i = threadIdx.x; i < RT * KI; i += blockDim.x) {
            const int r = i / KI, c = i % KI;
            float v = 0.0f;
            if (r0 + r < r_end) {
                if (FIRST) v = c < IN ? x[(r0 + r) * IN + c] : 0.0f;
                else v = silu(__bfloat162float(zp[(r0 + r) * KI + c]));
            }
            hs[r * LDH + c] = __float2bfloat16_rn(v);
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

static int mlp_grid(int64_t tiles, int per_cta) {
    int64_t want = (tiles + per_cta - 1) / per_cta;
    return (int)(want < 1 ? 1 : (want > 152 * 4 ? 152 * 4 : want));
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
    if (n == 0) return MPM_OK;
    if (mlp_attrs() != cudaSuccess) return MPM_ERR_CUDA;
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(params);
    const float *b = reinterpret_cast<const float *>(static_cast<const char *>(params) + (int64_t)W_COUNT * 2);
    FwdIO io{x, y, target, static_cast<__nv_bfloat16 *>(zsave), static_cast<__nv_bfloat16 *>(dy), loss,
             grad_scale, n};
    mlp_forward_kernel<<<mlp_grid((n + 15) / 16, 8), 256, sizeof(WSmem), static_cast<cudaStream_t>(stream)>>>(
        w, b, io);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

// Backward for one batch: accumulates (adds) into grad (fp32, same flat layout as
// the parameters: weights then biases).
int mpm_mlp_backward(const void *params, const float *x, const void *zsave, const void *dy, void *work,
                     float *grad, int64_t n, void *stream) {
    if (!params || !x || !zsave || !dy || !work || !grad || n <= 0) return MPM_ERR_ARG;
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
    const int gridd = mlp_grid((n + 15) / 16, 4);
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
