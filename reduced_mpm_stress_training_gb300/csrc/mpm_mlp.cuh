// Device core of the stress-surrogate network (12 -> 128 -> 128 -> 128 -> 6,
// SiLU, BF16 operands, FP32 accumulation on mma.sync m16n8k16), shared by the
// training kernels (mpm_mlp.cu) and the in-step surrogate stress kernel
// (mpm_surrogate.cu).  One warp evaluates 16 rows: the accumulator fragments
// of one layer are repacked in registers as the A fragments of the next.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "mpm_device.cuh"

namespace mpm {
namespace mlp {

constexpr int IN = 12, K1 = 16, H = 128, OUT = 6, N4 = 16;
constexpr int W1_OFF = 0, W2_OFF = W1_OFF + H * K1, W3_OFF = W2_OFF + H * H, W4_OFF = W3_OFF + H * H,
              W_COUNT = W4_OFF + N4 * H;  // bf16 elements
constexpr int B1_OFF = 0, B2_OFF = H, B3_OFF = 2 * H, B4_OFF = 3 * H, B_COUNT = 3 * H + N4;  // f32
constexpr int64_t PARAM_BYTES = (int64_t)W_COUNT * 2 + (int64_t)B_COUNT * 4;
constexpr int LDW = H + 8;   // padded smem row (bf16) of a 128-wide matrix: conflict-free ldmatrix
constexpr int LDW1 = K1 + 8; // padded smem row of W1

// SiLU through the hardware tanh (one MUFU op instead of an exponential and a
// division): sigmoid(z) = (1 + tanh(z / 2)) / 2, silu(z) = z sigmoid(z).  The
// approximation's relative error (about 2^-11) is below the bf16 rounding the
// activations get next.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid_fast(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = sigmoid_fast(z);
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

// Weights into shared memory with 16-byte copies (the blob is 16-byte aligned;
// every row of W1..W4 is a whole number of 16-byte words).
__device__ __forceinline__ void load_weights(WSmem &s, const __nv_bfloat16 *w, const float *b) {
    const uint4 *g = reinterpret_cast<const uint4 *>(w);
    for (int i = threadIdx.x; i < H * (K1 / 8); i += blockDim.x) {
        const int r = i / (K1 / 8), c = i % (K1 / 8);
        *reinterpret_cast<uint4 *>(s.w1 + r * LDW1 + c * 8) = g[W1_OFF / 8 + i];
    }
    for (int i = threadIdx.x; i < H * (H / 8); i += blockDim.x) {
        const int r = i / (H / 8), c = i % (H / 8);
        *reinterpret_cast<uint4 *>(s.w2 + r * LDW + c * 8) = g[W2_OFF / 8 + i];
        *reinterpret_cast<uint4 *>(s.w3 + r * LDW + c * 8) = g[W3_OFF / 8 + i];
    }
    for (int i = threadIdx.x; i < N4 * (H / 8); i += blockDim.x) {
        const int r = i / (H / 8), c = i % (H / 8);
        *reinterpret_cast<uint4 *>(s.w4 + r * LDW + c * 8) = g[W4_OFF / 8 + i];
    }
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


// The four layers on one warp's 16 rows: a1 = input fragment (16 rows x 16
// inputs), out = output fragments (two n8 tiles: columns 0..15, bias added).
// zsave (training only): pre-activations of rows row0.. as bf16 [3][n][128].
__device__ __forceinline__ void mlp_core(const WSmem &s, const uint32_t a1[1][4], float out[2][4],
                                         __nv_bfloat16 *zsave, int64_t row0, int64_t n) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    float acc[16][4];
    uint32_t a[8][4];
    layer_mma<1>(acc, a1, s.w1, LDW1);
    act_to_a(acc, s.b + B1_OFF, a, zsave ? zsave + 0 * n * H : nullptr, row0, n);
    layer_mma<8>(acc, a, s.w2, LDW);
    act_to_a(acc, s.b + B2_OFF, a, zsave ? zsave + 1 * n * H : nullptr, row0, n);
    layer_mma<8>(acc, a, s.w3, LDW);
    act_to_a(acc, s.b + B3_OFF, a, zsave ? zsave + 2 * n * H : nullptr, row0, n);
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
        const int col = nt * 8 + 2 * t;
        out[nt][0] = out[nt][2] = s.b[B4_OFF + col];
        out[nt][1] = out[nt][3] = s.b[B4_OFF + col + 1];
#pragma unroll
        for (int kt = 0; kt < 8; ++kt) {
            uint32_t b[2];
            b_frag(b, s.w4, LDW, nt * 8, kt * 16);
            mma16816(out[nt], a[kt], b[0], b[1]);
        }
    }
}

}  // namespace mlp
}  // namespace mpm
