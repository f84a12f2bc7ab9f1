// Stress-surrogate network backward on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).  Same gradients, parameter
// blob and bf16 rounding points as the mma.sync kernels of mpm_mlp.cu:
//   dZ_4 = dY (bf16, from the forward)
//   dH_{l-1} = dZ_l W_l            (fp32 accumulate)
//   dZ_{l-1} = bf16(dH_{l-1} * silu'(Z_{l-1}))
//   dW_l += dZ_l^T H_{l-1},  db_l += sum_rows dZ_l,  H_{l-1} = bf16(silu(Z_{l-1})) (H_0 = bf16(x))
//
// One persistent CTA per SM (256 threads, the whole 512-column tensor
// memory) walks 128-row tiles.  The four weight gradients stay in tensor
// memory across all of the CTA's tiles:
//   columns   0-127  dH (the data gradient of the current layer, per tile)
//   columns 128-255  dW2 [out = lane][in = column]
//   columns 256-383  dW3
//   columns 384-399  dW1 [out][in 0-15]
//   columns 400-415  dW4^T [in = lane][out 0-15]
// so no weight-gradient sum goes through global memory until the end, when
// each CTA adds its four accumulators and its bias sums into grad once.
// Per tile and layer one thread issues the data-gradient MMAs (A = dZ_l
// [rows][out], B = W_l^T [in][out]) and the weight-gradient MMAs (A =
// dZ_l^T [out][rows], B = H_{l-1}^T [in][rows]) and commits them to an
// mbarrier; then every thread reads its row of dH with tcgen05.ld, applies
// silu'(Z) and writes the next dZ in both orientations.  Operands are in the
// canonical K-major layout without swizzle (the forward's layout); the
// transposed copies are written element by element.  Every mbarrier wait is
// bounded: on timeout the kernel raises the error flag, stops issuing work,
// frees its tensor memory after a bounded grace wait and returns.
#include "mpm_mlp_tc.cuh"
#include "mpm_launch.h"

namespace mpm {
namespace mlpbw {

using namespace mpm::mlp;
using namespace mpm::mlptc;

constexpr uint32_t kBwCols = 512;
constexpr uint32_t C_DH = 0, C_W2 = 128, C_W3 = 256, C_W1 = 384, C_W4 = 400;

struct BwSmem {
    alignas(128) unsigned char w2t[8 * kWSlab];   // W2^T as B: [in 128][K = out 128]
    alignas(128) unsigned char w3t[8 * kWSlab];   // W3^T
    alignas(128) unsigned char w4t[kWSlab];       // W4^T: [in 128][K = out 16]
    alignas(128) unsigned char dz[8 * kSlab];     // dZ_l as A of the data gradient: [rows][K = out]
    alignas(128) unsigned char dzt[8 * kSlab];    // dZ_l^T as A of the weight gradient: [out 128][K = rows]
    alignas(128) unsigned char ht[8 * kSlab];     // H_{l-1}^T as B (and A for layer 4): [in 128][K = rows]
    alignas(128) unsigned char dz4t[8 * kW4Slab]; // dY^T as B of dW4^T: [out 16][K = rows]
    alignas(128) unsigned char xt[8 * kW4Slab];   // x^T as B of dW1: [in 16][K = rows]
    alignas(8) unsigned long long mbar;
    uint32_t tmem_base;
};

// byte offset of element (row, k) of a K-major operand with `slab_bytes` per 16-wide K slab
__device__ __forceinline__ uint32_t elem_off(int row, int k, int slab_bytes) {
    return chunk_off(row, k >> 3, slab_bytes) + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ void st_bf16(unsigned char *base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
}

// W_l [out][in] row-major (the blob) -> W_l^T as a K-major B operand [in][K = out];
// eight weights per 16-byte load
__device__ __forceinline__ void stage_wt(unsigned char *dst, const __nv_bfloat16 *w, int n_out, int slab_bytes) {
    for (int i = threadIdx.x; i < n_out * (H / 8); i += blockDim.x) {
        const int o = i / (H / 8), in0 = (i % (H / 8)) * 8;
        const uint4 v = reinterpret_cast<const uint4 *>(w)[i];
        const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
        for (int j = 0; j < 8; ++j) *reinterpret_cast<__nv_bfloat16 *>(dst + elem_off(in0 + j, o, slab_bytes)) = e[j];
    }
}

// this thread's 64 columns [c0, c0 + 64) of a saved pre-activation row (zeros past n)
struct ZHalf {
    uint4 v[8];
};
__device__ __forceinline__ void load_zhalf(ZHalf &z, const __nv_bfloat16 *zrow, int c0) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
        z.v[q] = zrow ? *reinterpret_cast<const uint4 *>(zrow + c0 + 8 * q) : make_uint4(0u, 0u, 0u, 0u);
}

// H_{l-1}^T from the pre-activations Z_{l-1} of this thread's row (columns
// [c0, c0 + 64)): H = bf16(silu(Z)), written transposed
__device__ __forceinline__ void stage_ht(BwSmem &s, const ZHalf &z, int row, int c0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t *u = reinterpret_cast<const uint32_t *>(&z.v[q]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 zz = unpack_bf16(u[e]);
            const int c = c0 + 8 * q + 2 * e;
            st_bf16(s.ht, elem_off(c, row, kSlab), silu(zz.x));
            st_bf16(s.ht, elem_off(c + 1, row, kSlab), silu(zz.y));
        }
    }
}

// commit the issued MMAs and wait (every thread); uniform outcome
__device__ __forceinline__ bool bw_wait(BwSmem &s, uint32_t &phase) {
    const bool ok = __syncthreads_and(mbar_wait(&s.mbar, phase) ? 1 : 0) != 0;
    phase ^= 1u;
    tc_after_sync();
    return ok;
}

__device__ __forceinline__ void bw_sync() {
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
}

// column c of dZ^T summed over the tile's rows (threads c < n_out)
__device__ __forceinline__ float sum_row_t(const unsigned char *t, int c, int slab_bytes) {
    float acc = 0.0f;
#pragma unroll 4
    for (int k8 = 0; k8 < kRows / 8; ++k8) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + chunk_off(c, k8, slab_bytes));
        const uint32_t *u = reinterpret_cast<const uint32_t *>(&v);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 f = unpack_bf16(u[e]);
            acc += f.x + f.y;
        }
    }
    return acc;
}

__global__ void __launch_bounds__(kThreads, 1) mlp_backward_tc_kernel(const __nv_bfloat16 *__restrict__ w,
                                                                   const float *__restrict__ x,
                                                                   const __nv_bfloat16 *__restrict__ zsave,
                                                                   const __nv_bfloat16 *__restrict__ dy,
                                                                   float *__restrict__ grad, int64_t n,
                                                                   int *__restrict__ err) {
    extern __shared__ __align__(128) unsigned char bw_smem_raw[];
    BwSmem &s = *reinterpret_cast<BwSmem *>(bw_smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & (kRows - 1), half = tid >> 7;
    // set-up: transposed weights, mbarrier, the whole tensor memory
    stage_wt(s.w2t, w + W2_OFF, H, kWSlab);
    stage_wt(s.w3t, w + W3_OFF, H, kWSlab);
    stage_wt(s.w4t, w + W4_OFF, N4, kWSlab);
    if (tid == 0) {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(&s.mbar);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s.tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst),
                     "r"(kBwCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    bw_sync();
    const uint32_t tbase = s.tmem_base;
    const uint32_t tlane = tbase + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's TMEM lane quarter
    uint32_t phase = 0;
    bool ok = true, first = true;
    float db[3] = {0.0f, 0.0f, 0.0f};  // bias sums of layers 1-3, column tid (< 128)
    float db4 = 0.0f;                 // bias sum of layer 4, column tid (< 16)
    const uint32_t idH = idesc_bf16(kRows, H), id16 = idesc_bf16(kRows, N4);
    const int64_t tiles = (n + kRows - 1) / kRows;
    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t grow = tile * kRows + row;
        const bool valid = grow < n;
        // ---- layer 4: dZ4 = dY; H3^T ----
        if (half == 0) {
            uint4 d0 = make_uint4(0u, 0u, 0u, 0u), d1 = d0;
            if (valid) {
                d0 = reinterpret_cast<const uint4 *>(dy + grow * N4)[0];
                d1 = reinterpret_cast<const uint4 *>(dy + grow * N4)[1];
            }
            *reinterpret_cast<uint4 *>(s.dz + chunk_off(row, 0, kSlab)) = d0;
            *reinterpret_cast<uint4 *>(s.dz + chunk_off(row, 1, kSlab)) = d1;
            const __nv_bfloat16 *dv0 = reinterpret_cast<const __nv_bfloat16 *>(&d0);
            const __nv_bfloat16 *dv1 = reinterpret_cast<const __nv_bfloat16 *>(&d1);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                *reinterpret_cast<__nv_bfloat16 *>(s.dz4t + elem_off(c, row, kW4Slab)) = dv0[c];
                *reinterpret_cast<__nv_bfloat16 *>(s.dz4t + elem_off(c + 8, row, kW4Slab)) = dv1[c];
            }
        }
        // the row's three saved pre-activations (this thread's half), loaded
        // together up front so one round trip serves the whole tile
        ZHalf z3, z2, z1;
        load_zhalf(z3, valid ? zsave + 2 * n * H + grow * H : nullptr, half * 64);
        load_zhalf(z2, valid ? zsave + 1 * n * H + grow * H : nullptr, half * 64);
        load_zhalf(z1, valid ? zsave + grow * H : nullptr, half * 64);
        stage_ht(s, z3, row, half * 64);
        bw_sync();
        if (tid < N4) db4 += sum_row_t(s.dz4t, tid, kW4Slab);
        if (tid == 0) {
            mma_bf16(tbase + C_DH, smem_desc(s.dz), smem_desc(s.w4t), idH, false);  // dH3 = dZ4 W4
#pragma unroll 1
            for (int ks = 0; ks < 8; ++ks)  // dW4^T += H3^T dZ4
                mma_bf16(tbase + C_W4, smem_desc(s.ht + ks * kSlab), smem_desc(s.dz4t + ks * kW4Slab), id16,
                         !first || ks > 0);
            mma_commit(&s.mbar);
        }
        if (!(ok = bw_wait(s, phase))) break;
        // ---- layers 3, 2: dZ_l = dH_l * silu'(Z_l); then dgrad + wgrad of layer l ----
#pragma unroll
        for (int l = 3; l >= 2; --l) {
            const ZHalf &zl = l == 3 ? z3 : z2;  // Z_l of this row
            const ZHalf &zp = l == 3 ? z2 : z1;  // Z_{l-1}: H_{l-1}^T for dW_l
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int c0 = half * 64 + 32 * h2;
                float acc[32];
                tmem_ld32(tlane + C_DH + (uint32_t)c0, acc);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint32_t *zu = reinterpret_cast<const uint32_t *>(&zl.v[4 * h2 + q]);
                    uint32_t dv[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 zz = unpack_bf16(zu[e]);
                        const int c = q * 8 + 2 * e;
                        const float g0 = valid ? acc[c] * silu_grad(zz.x) : 0.0f;
                        const float g1 = valid ? acc[c + 1] * silu_grad(zz.y) : 0.0f;
                        dv[e] = pack_bf16(g0, g1);
                        const float2 r = unpack_bf16(dv[e]);  // the bf16 values, for the transpose
                        st_bf16(s.dzt, elem_off(c0 + c, row, kSlab), r.x);
                        st_bf16(s.dzt, elem_off(c0 + c + 1, row, kSlab), r.y);
                    }
                    *reinterpret_cast<uint4 *>(s.dz + chunk_off(row, (c0 >> 3) + q, kSlab)) =
                        make_uint4(dv[0], dv[1], dv[2], dv[3]);
                }
            }
            stage_ht(s, zp, row, half * 64);
            bw_sync();
            if (tid < H) db[l - 1] += sum_row_t(s.dzt, tid, kSlab);
            if (tid == 0) {
                const unsigned char *wt = l == 3 ? s.w3t : s.w2t;
                const uint32_t cw = l == 3 ? C_W3 : C_W2;
#pragma unroll 1
                for (int ks = 0; ks < 8; ++ks) {
                    // dH_{l-1} = dZ_l W_l
                    mma_bf16(tbase + C_DH, smem_desc(s.dz + ks * kSlab), smem_desc(wt + ks * kWSlab), idH, ks > 0);
                    // dW_l += dZ_l^T H_{l-1}
                    mma_bf16(tbase + cw, smem_desc(s.dzt + ks * kSlab), smem_desc(s.ht + ks * kSlab), idH,
                             !first || ks > 0);
                }
                mma_commit(&s.mbar);
            }
            if (!(ok = bw_wait(s, phase))) break;
        }
        if (!ok) break;
        // ---- layer 1: dZ1 = dH1 * silu'(Z1); dW1 += dZ1^T x ----
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int c0 = half * 64 + 32 * h2;
            float acc[32];
            tmem_ld32(tlane + C_DH + (uint32_t)c0, acc);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t *zu = reinterpret_cast<const uint32_t *>(&z1.v[4 * h2 + q]);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float2 zz = unpack_bf16(zu[e]);
                    const int c = q * 8 + 2 * e;
                    const float g0 = valid ? acc[c] * silu_grad(zz.x) : 0.0f;
                    const float g1 = valid ? acc[c + 1] * silu_grad(zz.y) : 0.0f;
                    st_bf16(s.dzt, elem_off(c0 + c, row, kSlab), g0);
                    st_bf16(s.dzt, elem_off(c0 + c + 1, row, kSlab), g1);
                }
            }
        }
        if (half == 1) {  // x^T: inputs 0-11, 12-15 zero
#pragma unroll
            for (int k = 0; k < K1; ++k)
                st_bf16(s.xt, elem_off(k, row, kW4Slab), (valid && k < IN) ? x[grow * IN + k] : 0.0f);
        }
        bw_sync();
        if (tid < H) db[0] += sum_row_t(s.dzt, tid, kSlab);
        if (tid == 0) {
#pragma unroll 1
            for (int ks = 0; ks < 8; ++ks)
                mma_bf16(tbase + C_W1, smem_desc(s.dzt + ks * kSlab), smem_desc(s.xt + ks * kW4Slab), id16,
                         !first || ks > 0);
            mma_commit(&s.mbar);
        }
        if (!(ok = bw_wait(s, phase))) break;
        first = false;
        tc_before_sync();
    }
    if (ok && !first) {
        // the CTA's weight gradients and bias sums into grad (once per CTA)
#pragma unroll 1
        for (int m = 0; m < 2; ++m) {
            const uint32_t cw = m == 0 ? C_W2 : C_W3;
            float *g = grad + (m == 0 ? W2_OFF : W3_OFF) + row * H;
#pragma unroll 1
            for (int c0 = half * 64; c0 < half * 64 + 64; c0 += 32) {
                float acc[32];
                tmem_ld32(tlane + cw + (uint32_t)c0, acc);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    atomicAdd(reinterpret_cast<float4 *>(g + c0) + q,
                              make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]));
            }
        }
        {
            float acc[32];  // columns 384-415: dW1 row (out = row, in 0-15), dW4^T row (in = row, out 0-15)
            tmem_ld32(tlane + C_W1, acc);
            if (half == 0) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    atomicAdd(reinterpret_cast<float4 *>(grad + W1_OFF + row * K1) + q,
                              make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]));
            } else {
#pragma unroll
                for (int o = 0; o < N4; ++o) atomicAdd(grad + W4_OFF + o * H + row, acc[16 + o]);
            }
        }
        float *gb = grad + W_COUNT;
        if (tid < H) {
            atomicAdd(gb + B1_OFF + tid, db[0]);
            atomicAdd(gb + B2_OFF + tid, db[1]);
            atomicAdd(gb + B3_OFF + tid, db[2]);
        }
        if (tid < N4) atomicAdd(gb + B4_OFF + tid, db4);
    }
    if (!ok && tid == 0) atomicOr(err, 1);
    // tear-down: after a timed-out wait the MMAs may still be in flight, so they
    // get a bounded grace period before the tensor memory is released
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) {
        if (!ok) mbar_wait(&s.mbar, phase ^ 1u);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(kBwCols)
                     : "memory");
    }
}

}  // namespace mlpbw

int64_t mlp_bw_tc_smem_bytes() { return (int64_t)sizeof(mlpbw::BwSmem); }

cudaError_t launch_mlp_backward_tc(const void *params, const float *x, const void *zsave, const void *dy,
                                   float *grad, int64_t n, int *err, int num_sms, cudaStream_t stream) {
    using namespace mlpbw;
    if (n <= 0) return cudaSuccess;
    static bool attr_set[64] = {false};
    const int bytes = (int)mlp_bw_tc_smem_bytes();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(mlp_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(params);
    const int64_t tiles = (n + kRows - 1) / kRows;
    // one CTA per SM (each holds all 512 tensor-memory columns)
    const int grid = (int)(tiles < (int64_t)num_sms ? tiles : (int64_t)num_sms);
    mlp_backward_tc_kernel<<<grid, kThreads, bytes, stream>>>(w, x, static_cast<const __nv_bfloat16 *>(zsave),
                                                              static_cast<const __nv_bfloat16 *>(dy), grad, n, err);
    return cudaGetLastError();
}

}  // namespace mpm
