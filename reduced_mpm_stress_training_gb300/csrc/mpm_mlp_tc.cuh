// Device core of the tcgen05 network forward, shared by the standalone
// forward (mpm_mlp_tc.cu) and the in-step surrogate stage (mpm_surrogate.cu).
// See mpm_mlp_tc.cu for the operand layout and the synchronisation scheme.
#pragma once

#include "mpm_mlp.cuh"

namespace mpm {
namespace mlptc {

using namespace mpm::mlp;

constexpr int kRows = 128;                 // tile rows = TMEM lanes
constexpr int kThreads = 256;              // two threads per row: each takes half of the columns
constexpr int kSlab = kRows * 16 * 2;      // bytes of one 128 x 16 bf16 K slab (4 KB)
constexpr int kWSlab = H * 16 * 2;         // bytes of one 128(N) x 16 weight slab (4 KB)
constexpr int kW4Slab = N4 * 16 * 2;       // 16(N) x 16 weight slab (512 B)
constexpr uint32_t kTmemCols = 128;
constexpr long long kWaitLimit = 20000000; // mbarrier polls before giving up

struct TcSmem {  // every operand region 128-byte aligned (the descriptors need 16)
    alignas(128) unsigned char w1[kWSlab];       // W1: 1 slab
    alignas(128) unsigned char w2[8 * kWSlab];   // W2: 8 slabs
    alignas(128) unsigned char w3[8 * kWSlab];
    alignas(128) unsigned char w4[8 * kW4Slab];
    alignas(128) unsigned char x[kSlab];         // input tile: 1 slab
    alignas(128) unsigned char h[8 * kSlab];     // activations: 8 slabs
    float bias[B_COUNT];
    alignas(8) unsigned long long mbar;
    uint32_t tmem_base;
};

// byte offset of (row, k) 16-byte chunk (k8 = k / 8) inside a K slab set
// with `slab_bytes` per 16-wide K slab
__device__ __forceinline__ uint32_t chunk_off(int row, int k8, int slab_bytes) {
    return (uint32_t)((k8 >> 1) * slab_bytes + ((row >> 3) * 2 + (k8 & 1)) * 128 + (row & 7) * 16);
}

__device__ __forceinline__ uint64_t smem_desc(const void *p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint64_t d = 0;
    d |= (uint64_t)((a >> 4) & 0x3FFF);                 // start address
    d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;        // leading byte offset: K-adjacent core matrices
    d |= (uint64_t)((256u >> 4) & 0x3FFF) << 32;        // stride byte offset: 8-row groups
    d |= (uint64_t)1 << 46;                             // descriptor version
    return d;                                           // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((int)acc));
}

__device__ __forceinline__ void mma_commit(unsigned long long *mbar) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(mbar);
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(a)
                 : "memory");
}

// bounded wait for the mbarrier phase with the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(unsigned long long *mbar, uint32_t parity) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(mbar);
    for (long long it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// weights, row-major [n][k] in the blob -> K-major core-matrix layout
__device__ __forceinline__ void stage_weights(TcSmem &s, const __nv_bfloat16 *w, const float *b) {
    const uint4 *g = reinterpret_cast<const uint4 *>(w);
    for (int i = threadIdx.x; i < H * (K1 / 8); i += blockDim.x) {  // W1 [128][16]
        const int n = i / (K1 / 8), k8 = i % (K1 / 8);
        *reinterpret_cast<uint4 *>(s.w1 + chunk_off(n, k8, kWSlab)) = g[W1_OFF / 8 + i];
    }
    for (int i = threadIdx.x; i < H * (H / 8); i += blockDim.x) {   // W2, W3 [128][128]
        const int n = i / (H / 8), k8 = i % (H / 8);
        *reinterpret_cast<uint4 *>(s.w2 + chunk_off(n, k8, kWSlab)) = g[W2_OFF / 8 + i];
        *reinterpret_cast<uint4 *>(s.w3 + chunk_off(n, k8, kWSlab)) = g[W3_OFF / 8 + i];
    }
    for (int i = threadIdx.x; i < N4 * (H / 8); i += blockDim.x) {  // W4 [16][128]
        const int n = i / (H / 8), k8 = i % (H / 8);
        *reinterpret_cast<uint4 *>(s.w4 + chunk_off(n, k8, kW4Slab)) = g[W4_OFF / 8 + i];
    }
    for (int i = threadIdx.x; i < B_COUNT; i += blockDim.x) s.bias[i] = b[i];
}

// bias + SiLU of 32 accumulator columns of this thread's row; writes the bf16
// activations (columns c0..c0+31) into the A slabs and, if given, Z to zrow
__device__ __forceinline__ void act_chunk(TcSmem &s, const float acc[32], const float *bias, int row, int c0,
                                          __nv_bfloat16 *zrow) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // 4 chunks of 8 columns = 16 bytes
        uint32_t hv[4], zv[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = q * 8 + 2 * e;
            const float z0 = acc[c] + bias[c0 + c], z1 = acc[c + 1] + bias[c0 + c + 1];
            zv[e] = pack_bf16(z0, z1);
            hv[e] = pack_bf16(silu(z0), silu(z1));
        }
        const int k8 = (c0 >> 3) + q;
        *reinterpret_cast<uint4 *>(s.h + chunk_off(row, k8, kSlab)) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
        if (zrow) *reinterpret_cast<uint4 *>(zrow + c0 + q * 8) = make_uint4(zv[0], zv[1], zv[2], zv[3]);
    }
}


// CTA set-up: weights into the K-major layout, mbarrier, 128 TMEM columns.
// All 128 threads call it; returns the TMEM base address.
__device__ __forceinline__ uint32_t tc_setup(TcSmem &s, const __nv_bfloat16 *w, const float *b) {
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weights(s, w, b);
    if (tid == 0) {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(&s.mbar);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s.tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    return s.tmem_base;
}

// CTA tear-down: after a timed-out wait the MMAs may still be in flight, so
// they get a bounded grace period before the tensor memory is released.
__device__ __forceinline__ void tc_teardown(TcSmem &s, uint32_t tbase, bool ok, uint32_t phase) {
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if ((threadIdx.x >> 5) == 0) {
        if (!ok) mbar_wait(&s.mbar, phase ^ 1u);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(kTmemCols)
                     : "memory");
    }
}

// Row t's inputs into the input slab (12 features + 4 zeros); threads t < 128 only.
__device__ __forceinline__ void tc_store_inputs(TcSmem &s, const float v[12]) {
    const int t = threadIdx.x;
    *reinterpret_cast<uint4 *>(s.x + chunk_off(t, 0, kSlab)) =
        make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
    *reinterpret_cast<uint4 *>(s.x + chunk_off(t, 1, kSlab)) =
        make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), 0u, 0u);
}

// The four layers on the 128-row tile whose inputs are in s.x.  Threads t and
// t + 128 share row t (TMEM lanes are reachable from warps w and w + 4) and
// take columns 0-63 and 64-127 of the hidden layers.  Thread t < 128 gets row
// t's 16 (padded) outputs, bias added, in out; with z != null the bf16
// pre-activations of layer l go to z[l] (row pointers, null for padding
// rows).  Returns false (uniformly) on a timed-out wait.
__device__ __forceinline__ bool tc_tile_forward(TcSmem &s, uint32_t tbase, uint32_t &phase, float out[16],
                                                __nv_bfloat16 *const z[3]) {
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & (kRows - 1), half = tid >> 7;
    const uint32_t tlane = tbase + ((uint32_t)((warp & 3) * 32) << 16);
    for (int layer = 0; layer < 4; ++layer) {
        fence_async_smem();
        tc_before_sync();
        __syncthreads();
        tc_after_sync();
        if (tid == 0) {
            if (layer == 0) {
                mma_bf16(tbase, smem_desc(s.x), smem_desc(s.w1), idesc_bf16(kRows, H), false);
            } else {
                const unsigned char *wl = layer == 1 ? s.w2 : layer == 2 ? s.w3 : s.w4;
                const int wslab = layer == 3 ? kW4Slab : kWSlab;
                const uint32_t id = idesc_bf16(kRows, layer == 3 ? N4 : H);
#pragma unroll 1
                for (int ks = 0; ks < 8; ++ks)
                    mma_bf16(tbase, smem_desc(s.h + ks * kSlab), smem_desc(wl + ks * wslab), id, ks > 0);
            }
            mma_commit(&s.mbar);
        }
        // every thread waits; the outcome is made uniform so that no warp
        // enters the warp-wide tensor-memory loads alone
        const bool ok = __syncthreads_and(mbar_wait(&s.mbar, phase) ? 1 : 0) != 0;
        phase ^= 1u;
        tc_after_sync();
        if (!ok) return false;
        if (layer < 3) {
            // the layer's MMAs are done reading s.h: overwrite it with the next activations
#pragma unroll 1
            for (int c0 = half * (H / 2); c0 < (half + 1) * (H / 2); c0 += 32) {
                float acc[32];
                tmem_ld32(tlane + (uint32_t)c0, acc);
                act_chunk(s, acc, s.bias + layer * H, row, c0, z ? z[layer] : nullptr);
            }
        } else {
            float acc[32];
            tmem_ld32(tlane, acc);
#pragma unroll
            for (int c = 0; c < N4; ++c) out[c] = acc[c] + s.bias[B4_OFF + c];
        }
        tc_before_sync();
    }
    return true;
}

}  // namespace mlptc
}  // namespace mpm
