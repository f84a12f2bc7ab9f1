// The reference's stress decoder NetDec
// (offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301, 434-525)
// evaluated on the GPU: Prepare (standardise or clip the position), five
// Linear layers of width `hidden` with ELU or sin(omega_0 x) activations,
// the output Linear to the six stress components [xx, xy, xz, yy, yz, zz]
// and invStandardizeQ.  Two forms:
//   decoder_rows_kernel   -- NetDec.forward on caller rows (lbl + 3 + mu_dim
//                            floats each) -> 6 floats per row
//   decoder_stress_kernel -- the reduced-order loop's stress source: one
//                            frame label for all particles, each particle's
//                            x_initial from its state record and its mu row
//                            by uid; the symmetric stress goes straight into
//                            the record's stress words, which the next P2G
//                            reads (the reference loads it with
//                            load_uvstress_from_tensor, mpm_solver_warp.py:253-266).
// FP32 throughout, as the reference's PyTorch module.  One thread per row;
// the parameters (zero-padded to HP neurons) sit in shared memory and are
// read as broadcasts, the activations stay in registers.
#include "mpm_launch.h"
#include "mpm_mlp_tc.cuh"

namespace mpm {

namespace {

constexpr int kDecThreads = 128;

struct DecLayout {  // float offsets of the shared-memory copy (HP-padded)
    int w0, b0, wh, bh, we, be, prep, qm, qs, c0, total;
};

__host__ __device__ inline DecLayout dec_layout(int hp, int in) {
    DecLayout L;
    int o = 0;
    L.w0 = o; o += hp * in;
    L.b0 = o; o += hp;
    L.wh = o; o += 4 * hp * hp;
    L.bh = o; o += 4 * hp;
    L.we = o; o += 6 * hp;
    L.be = o; o += 8;
    L.prep = o; o += 8;
    L.qm = o; o += 8;
    L.qs = o; o += 8;
    L.c0 = o; o += hp;  // layer-0 bias plus the frame label's part (stress form)
    L.total = o;
    return L;
}

// offsets in the caller's packed (unpadded) parameter blob
struct BlobLayout {
    int w0, b0, wh, bh, we, be, prep, qm, qs, total;
};

__host__ __device__ inline BlobLayout blob_layout(int h, int in) {
    BlobLayout B;
    int o = 0;
    B.w0 = o; o += h * in;
    B.b0 = o; o += h;
    B.wh = o; o += 4 * h * h;
    B.bh = o; o += 4 * h;
    B.we = o; o += 6 * h;
    B.be = o; o += 6;
    B.prep = o; o += 6;
    B.qm = o; o += 6;
    B.qs = o; o += 6;
    B.total = o;
    return B;
}

// exp(x) - 1 for x <= 0: on [-0.5, 0] the Taylor series through x^8 / 8!
// (truncation below 1.1e-8 of the result), below that exp(x) - 1, whose
// magnitude is then at least 0.39, so the 2^-21 relative error of the fast
// exponential stays under 1e-6 of it
__device__ __forceinline__ float expm1_nonpos(float x) {
    if (x > -0.5f) {
        float p = 1.0f / 40320.0f;
        p = fmaf(p, x, 1.0f / 5040.0f);
        p = fmaf(p, x, 1.0f / 720.0f);
        p = fmaf(p, x, 1.0f / 120.0f);
        p = fmaf(p, x, 1.0f / 24.0f);
        p = fmaf(p, x, 1.0f / 6.0f);
        p = fmaf(p, x, 0.5f);
        p = fmaf(p, x, 1.0f);
        return p * x;
    }
    return __expf(x) - 1.0f;
}

__device__ __forceinline__ float dec_act(float x, bool siren, float omega_0) {
    if (siren) return sinf(__fmul_rn(omega_0, x));  // actSIN, :462-463
    return x > 0.0f ? x : expm1_nonpos(x);          // actELU (F.elu, alpha 1), :459-460
}

// copy the blob into shared memory, padding every layer to hp neurons with zeros
__device__ void dec_stage(const MpmStressDecoder &d, int hp, float *sm) {
    const int h = d.hidden, in = d.label_dim + 3 + d.mu_dim;
    const DecLayout L = dec_layout(hp, in);
    const BlobLayout B = blob_layout(h, in);
    const float *P = d.params;
    for (int i = threadIdx.x; i < hp * in; i += blockDim.x) {
        const int r = i / in, c = i % in;
        sm[L.w0 + i] = r < h ? P[B.w0 + r * in + c] : 0.0f;
    }
    for (int i = threadIdx.x; i < hp; i += blockDim.x) sm[L.b0 + i] = i < h ? P[B.b0 + i] : 0.0f;
    for (int i = threadIdx.x; i < 4 * hp * hp; i += blockDim.x) {
        const int l = i / (hp * hp), r = (i / hp) % hp, c = i % hp;
        sm[L.wh + i] = (r < h && c < h) ? P[B.wh + (l * h + r) * h + c] : 0.0f;
    }
    for (int i = threadIdx.x; i < 4 * hp; i += blockDim.x) {
        const int l = i / hp, r = i % hp;
        sm[L.bh + i] = r < h ? P[B.bh + l * h + r] : 0.0f;
    }
    for (int i = threadIdx.x; i < 6 * hp; i += blockDim.x) {
        const int r = i / hp, c = i % hp;
        sm[L.we + i] = c < h ? P[B.we + r * h + c] : 0.0f;
    }
    for (int i = threadIdx.x; i < 6; i += blockDim.x) {
        sm[L.be + i] = P[B.be + i];
        sm[L.prep + i] = P[B.prep + i];
        sm[L.qm + i] = P[B.qm + i];
        sm[L.qs + i] = P[B.qs + i];
    }
}

// Prepare (:507-525): clipX 2 (x - min) / (max - min) - 1 for SIREN, else
// standardizeX (x - mean) / std; prep holds (min, max) or (mean, std)
__device__ __forceinline__ float dec_prep(const float *prep, int d, float x, bool siren) {
    if (siren) return __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fsub_rn(x, prep[d])), __fsub_rn(prep[3 + d], prep[d])), 1.0f);
    return __fdiv_rn(__fsub_rn(x, prep[d]), prep[3 + d]);
}

// hidden layers dec1..dec4 and the output layer enc + invStandardizeQ (:476-477)
template <int HP>
__device__ __forceinline__ void dec_tail(const float *sm, const DecLayout &L, float h[HP], bool siren, float omega_0,
                                         float q[6]) {
#pragma unroll 1
    for (int l = 0; l < 4; ++l) {
        const float *W = sm + L.wh + l * HP * HP;
        const float *b = sm + L.bh + l * HP;
        float g[HP];
        // the 64-wide form keeps one output row per iteration (g in local memory): a full
        // unroll of 64 x 64 multiply-adds costs minutes of compile time
        constexpr int kJUnroll = HP <= 32 ? HP : 1;
#pragma unroll kJUnroll
        for (int j = 0; j < HP; ++j) {
            float acc = b[j];
            const float4 *w4 = reinterpret_cast<const float4 *>(W + j * HP);
#pragma unroll
            for (int k = 0; k < HP / 4; ++k) {
                const float4 w = w4[k];
                acc = fmaf(w.x, h[4 * k + 0], acc);
                acc = fmaf(w.y, h[4 * k + 1], acc);
                acc = fmaf(w.z, h[4 * k + 2], acc);
                acc = fmaf(w.w, h[4 * k + 3], acc);
            }
            g[j] = dec_act(acc, siren, omega_0);
        }
#pragma unroll
        for (int j = 0; j < HP; ++j) h[j] = g[j];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        float acc = sm[L.be + c];
        const float4 *w4 = reinterpret_cast<const float4 *>(sm + L.we + c * HP);
#pragma unroll
        for (int k = 0; k < HP / 4; ++k) {
            const float4 w = w4[k];
            acc = fmaf(w.x, h[4 * k + 0], acc);
            acc = fmaf(w.y, h[4 * k + 1], acc);
            acc = fmaf(w.z, h[4 * k + 2], acc);
            acc = fmaf(w.w, h[4 * k + 3], acc);
        }
        q[c] = __fadd_rn(sm[L.qm + c], __fmul_rn(acc, sm[L.qs + c]));
    }
}

}  // namespace

// NetDec.forward (:288-291) on rows (label_dim + 3 + mu_dim floats) -> 6 floats
template <int HP>
__global__ void __launch_bounds__(kDecThreads) decoder_rows_kernel(MpmStressDecoder d, const float *__restrict__ rows,
                                                                   float *__restrict__ out, int64_t n) {
    extern __shared__ float4 sm4[];
    float *sm = reinterpret_cast<float *>(sm4);
    const int L0 = d.label_dim, in = L0 + 3 + d.mu_dim;
    const DecLayout L = dec_layout(HP, in);
    dec_stage(d, HP, sm);
    __syncthreads();
    const bool siren = d.siren != 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const float *x = rows + r * in;
        float h[HP];
#pragma unroll
        for (int j = 0; j < HP; ++j) h[j] = sm[L.b0 + j];
        for (int k = 0; k < in; ++k) {
            float v = x[k];
            if (k >= L0 && k < L0 + 3) v = dec_prep(sm + L.prep, k - L0, v, siren);
#pragma unroll
            for (int j = 0; j < HP; ++j) h[j] = fmaf(sm[L.w0 + j * in + k], v, h[j]);
        }
#pragma unroll
        for (int j = 0; j < HP; ++j) h[j] = dec_act(h[j], siren, d.omega_0);
        float q[6];
        dec_tail<HP>(sm, L, h, siren, d.omega_0, q);
#pragma unroll
        for (int c = 0; c < 6; ++c) out[r * 6 + c] = q[c];
    }
}

// The decoder as the stress source of a substep: label (label_dim floats, the
// frame's latent), each particle's x_initial from its record and mu row
// (mu_dim floats, user order) by uid; writes the symmetric stress
// [q0 q1 q2; q1 q3 q4; q2 q4 q5] into the record (mpm_solver_warp.py:383 order).
template <int HP>
__global__ void __launch_bounds__(kDecThreads) decoder_stress_kernel(MpmStressDecoder d, PState st,
                                                                     const float *__restrict__ label,
                                                                     const float *__restrict__ mu, int n) {
    extern __shared__ float4 sm4[];
    float *sm = reinterpret_cast<float *>(sm4);
    const int L0 = d.label_dim, M = d.mu_dim, in = L0 + 3 + M;
    const DecLayout L = dec_layout(HP, in);
    dec_stage(d, HP, sm);
    __syncthreads();
    // the label's part of layer 0 is the same for every particle of the frame
    for (int j = threadIdx.x; j < HP; j += blockDim.x) {
        float acc = sm[L.b0 + j];
        for (int k = 0; k < L0; ++k) acc = fmaf(sm[L.w0 + j * in + k], label[k], acc);
        sm[L.c0 + j] = acc;
    }
    __syncthreads();
    const bool siren = d.siren != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q0 = ldrec(st, i, 0), q1 = ldrec(st, i, 1);
        const int uid = __float_as_int(q1.y);
        float h[HP];
#pragma unroll
        for (int j = 0; j < HP; ++j) h[j] = sm[L.c0 + j];
        const float xp[3] = {dec_prep(sm + L.prep, 0, q0.x, siren), dec_prep(sm + L.prep, 1, q0.y, siren),
                             dec_prep(sm + L.prep, 2, q0.z, siren)};
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int j = 0; j < HP; ++j) h[j] = fmaf(sm[L.w0 + j * in + L0 + k], xp[k], h[j]);
        for (int k = 0; k < M; ++k) {
            const float v = mu[(int64_t)uid * M + k];
#pragma unroll
            for (int j = 0; j < HP; ++j) h[j] = fmaf(sm[L.w0 + j * in + L0 + 3 + k], v, h[j]);
        }
#pragma unroll
        for (int j = 0; j < HP; ++j) h[j] = dec_act(h[j], siren, d.omega_0);
        float q[6];
        dec_tail<HP>(sm, L, h, siren, d.omega_0, q);
        const float4 q5 = ldrec(st, i, 5);
        strec(st, i, 5, make_float4(q5.x, q5.y, q5.z, q[0]));
        strec(st, i, 6, make_float4(q[1], q[2], q[1], q[3]));
        strec(st, i, 7, make_float4(q[4], q[2], q[4], q[5]));
    }
}

// ---------------------------------------------------------------------------
// Tensor-core form of decoder_stress_kernel for widths up to 32 (the
// reference's default is 30).  The four 32 x 32 hidden layers carry 85 % of the
// multiply-adds.  They run as tcgen05 MMAs on 128-particle tiles, with FP32
// accumulators in tensor memory.
//
// FP32 accuracy comes from BF16 operands: every activation and weight is
// split exactly into three BF16 pieces (x = x0 + x1 + x2, 8 significant bits
// each).  The six products x_i w_j with i + j <= 2 are accumulated, smallest
// first.  Each of the three dropped products is below 2^-24 |x| |w|.
//
// Layer 0 stays on the CUDA cores: the label's part once per CTA, then the
// position and mu columns per particle.  The 6-wide output layer does too.
//
// One thread per tile row (TMEM lane).  Each layer's epilogue (bias,
// activation, split into the next layer's A operand) runs on the CUDA cores
// between the MMAs.  Every mbarrier wait is bounded; a timeout sets
// MPM_ST_INTERNAL and the CTA stops.
// ---------------------------------------------------------------------------
namespace dtc {

constexpr int kRows = 128;              // particles per tile = TMEM lanes = threads
constexpr int kHP = 32;                 // padded width
constexpr int kParts = 3;               // BF16 pieces per FP32 value
constexpr int kASlab = kRows * 16 * 2;  // one 128 x 16 BF16 K slab (4 KB)
constexpr int kWSlab = kHP * 16 * 2;    // one 32 x 16 BF16 K slab (1 KB)
constexpr int kKSlabs = kHP / 16;
constexpr uint32_t kTmemCols = 32;
constexpr int kMaxCols = 3 + 4;         // per-particle layer-0 columns: position + mu

// P tile pipelines per CTA (P x 128 threads), each with its own activations,
// tensor-memory columns, mbarrier and named barrier; the weights are shared
template <int P>
struct Smem {
    alignas(128) unsigned char a[P][kParts][kKSlabs * kASlab];  // each pipeline's activations
    alignas(128) unsigned char w[4][kParts][kKSlabs * kWSlab];  // hidden-layer weights
    alignas(16) float w0p[kMaxCols][kHP];  // layer 0, position and mu columns, [k][j]
    alignas(16) float c0[kHP];             // layer-0 bias + the label's part
    alignas(16) float bh[4][kHP];
    alignas(16) float we[6][kHP];
    float be[6], prep[6], qm[6], qs[6];
    alignas(8) unsigned long long mbar[P];
    uint32_t tmem_base;
};

// two values -> their three BF16 pieces, packed in pairs (exact: each
// difference is representable in FP32, the last one in BF16)
__device__ __forceinline__ void split3(float x, float y, uint32_t &p0, uint32_t &p1, uint32_t &p2) {
    p0 = mlp::pack_bf16(x, y);
    const float2 f0 = mlp::unpack_bf16(p0);
    const float rx = __fsub_rn(x, f0.x), ry = __fsub_rn(y, f0.y);
    p1 = mlp::pack_bf16(rx, ry);
    const float2 f1 = mlp::unpack_bf16(p1);
    p2 = mlp::pack_bf16(__fsub_rn(rx, f1.x), __fsub_rn(ry, f1.y));
}

// row's 32 activations -> the three A operands (K-major core-matrix layout)
__device__ __forceinline__ void store_row(unsigned char (&a)[kParts][kKSlabs * kASlab], int row,
                                          const float v[kHP]) {
#pragma unroll
    for (int q = 0; q < kHP / 8; ++q) {
        uint32_t h0[4], h1[4], h2[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) split3(v[q * 8 + 2 * e], v[q * 8 + 2 * e + 1], h0[e], h1[e], h2[e]);
        const uint32_t off = mlptc::chunk_off(row, q, kASlab);
        *reinterpret_cast<uint4 *>(a[0] + off) = make_uint4(h0[0], h0[1], h0[2], h0[3]);
        *reinterpret_cast<uint4 *>(a[1] + off) = make_uint4(h1[0], h1[1], h1[2], h1[3]);
        *reinterpret_cast<uint4 *>(a[2] + off) = make_uint4(h2[0], h2[1], h2[2], h2[3]);
    }
}

// the parameters: hidden weights as BF16 pieces, the rest FP32, zero-padded to 32
template <int P>
__device__ void stage(const MpmStressDecoder &d, const float *label, Smem<P> &s) {
    const int h = d.hidden, L0 = d.label_dim, M = d.mu_dim, in = L0 + 3 + M;
    const BlobLayout B = blob_layout(h, in);
    const float *Pm = d.params;
    for (int i = threadIdx.x; i < 4 * kHP * kHP; i += blockDim.x) {
        const int l = i / (kHP * kHP), j = (i / kHP) % kHP, k = i % kHP;
        const float w = (j < h && k < h) ? Pm[B.wh + (l * h + j) * h + k] : 0.0f;
        const __nv_bfloat16 b0 = __float2bfloat16_rn(w);
        const float r = __fsub_rn(w, __bfloat162float(b0));
        const __nv_bfloat16 b1 = __float2bfloat16_rn(r);
        const __nv_bfloat16 b2 = __float2bfloat16_rn(__fsub_rn(r, __bfloat162float(b1)));
        const uint32_t off = mlptc::chunk_off(j, k >> 3, kWSlab) + (k & 7) * 2;
        *reinterpret_cast<__nv_bfloat16 *>(s.w[l][0] + off) = b0;
        *reinterpret_cast<__nv_bfloat16 *>(s.w[l][1] + off) = b1;
        *reinterpret_cast<__nv_bfloat16 *>(s.w[l][2] + off) = b2;
    }
    for (int i = threadIdx.x; i < kMaxCols * kHP; i += blockDim.x) {
        const int k = i / kHP, j = i % kHP;
        s.w0p[k][j] = (j < h && k < 3 + M) ? Pm[B.w0 + j * in + L0 + k] : 0.0f;
    }
    for (int j = threadIdx.x; j < kHP; j += blockDim.x) {
        float acc = j < h ? Pm[B.b0 + j] : 0.0f;
        for (int k = 0; k < L0 && j < h; ++k) acc = fmaf(Pm[B.w0 + j * in + k], label[k], acc);
        s.c0[j] = acc;
    }
    for (int i = threadIdx.x; i < 4 * kHP; i += blockDim.x) {
        const int l = i / kHP, j = i % kHP;
        s.bh[l][j] = j < h ? Pm[B.bh + l * h + j] : 0.0f;
    }
    for (int i = threadIdx.x; i < 6 * kHP; i += blockDim.x) {
        const int c = i / kHP, j = i % kHP;
        s.we[c][j] = j < h ? Pm[B.we + c * h + j] : 0.0f;
    }
    for (int i = threadIdx.x; i < 6; i += blockDim.x) {
        s.be[i] = Pm[B.be + i];
        s.prep[i] = Pm[B.prep + i];
        s.qm[i] = Pm[B.qm + i];
        s.qs[i] = Pm[B.qs + i];
    }
}

// the 128 threads of pipeline `pipe`: a barrier, and one whose outcome is the
// AND of every thread's flag (named barriers 1 and 2; 0 is __syncthreads)
// (barrier ids are immediates, so the kernel reserves three barriers, not sixteen)
__device__ __forceinline__ void pipe_sync(int pipe) {
    if (pipe == 0) asm volatile("bar.sync 1, 128;\n" ::: "memory");
    else asm volatile("bar.sync 2, 128;\n" ::: "memory");
}
__device__ __forceinline__ bool pipe_and(int pipe, bool v) {
    uint32_t r;
    if (pipe == 0)
        asm volatile(
            "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, 1, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(r)
            : "r"((uint32_t)v)
            : "memory");
    else
        asm volatile(
            "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, 2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(r)
            : "r"((uint32_t)v)
            : "memory");
    return r != 0;
}

}  // namespace dtc

template <int P>
__global__ void __launch_bounds__(P * dtc::kRows, P == 2 ? 3 : 4) decoder_stress_tc_kernel(MpmStressDecoder d, PState st,
                                                                          const float *__restrict__ label,
                                                                          const float *__restrict__ mu, int n,
                                                                          int *status) {
    using namespace dtc;
    extern __shared__ __align__(128) unsigned char dtc_smem_raw[];
    Smem<P> &s = *reinterpret_cast<Smem<P> *>(dtc_smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, pipe = tid >> 7, row = tid & (kRows - 1);
    const int M = d.mu_dim;
    const bool siren = d.siren != 0;
    stage(d, label, s);
    if (tid < P) {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(&s.mbar[tid]);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s.tmem_base);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst),
                     "r"(kTmemCols * P)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    mlptc::fence_async_smem();
    mlptc::tc_before_sync();
    __syncthreads();
    mlptc::tc_after_sync();
    const uint32_t tbase = s.tmem_base + (uint32_t)(pipe * kTmemCols);  // this pipeline's columns
    const uint32_t tlane = tbase + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t id = mlptc::idesc_bf16(kRows, kHP);
    unsigned long long *mbar = &s.mbar[pipe];
    auto &a = s.a[pipe];
    // the six piece products, smallest first: (activation piece, weight piece)
    constexpr int kPa[6] = {2, 1, 0, 1, 0, 0}, kPw[6] = {0, 1, 2, 0, 1, 0};
    uint32_t phase = 0;
    bool ok = true;
    const int n_tiles = (n + kRows - 1) / kRows;
    for (int tile = blockIdx.x * P + pipe; tile < n_tiles && ok; tile += gridDim.x * P) {
        const int i = tile * kRows + row;
        const bool live = i < n;
        // layer 0 (dec0 + act): the label part is in c0; position and mu per particle
        float xin[kMaxCols];
#pragma unroll
        for (int k = 0; k < kMaxCols; ++k) xin[k] = 0.0f;
        if (live) {
            const float4 q0 = ldrec(st, i, 0), q1 = ldrec(st, i, 1);
            xin[0] = dec_prep(s.prep, 0, q0.x, siren);
            xin[1] = dec_prep(s.prep, 1, q0.y, siren);
            xin[2] = dec_prep(s.prep, 2, q0.z, siren);
            const int uid = __float_as_int(q1.y);
#pragma unroll
            for (int k = 0; k < kMaxCols - 3; ++k)
                if (k < M) xin[3 + k] = mu[(int64_t)uid * M + k];
        }
        float h[kHP];
#pragma unroll
        for (int j = 0; j < kHP; ++j) h[j] = s.c0[j];
#pragma unroll
        for (int k = 0; k < kMaxCols; ++k) {
            if (k >= 3 + M) break;
            const float4 *w4 = reinterpret_cast<const float4 *>(s.w0p[k]);
#pragma unroll
            for (int q = 0; q < kHP / 4; ++q) {
                const float4 w = w4[q];
                h[4 * q + 0] = fmaf(w.x, xin[k], h[4 * q + 0]);
                h[4 * q + 1] = fmaf(w.y, xin[k], h[4 * q + 1]);
                h[4 * q + 2] = fmaf(w.z, xin[k], h[4 * q + 2]);
                h[4 * q + 3] = fmaf(w.w, xin[k], h[4 * q + 3]);
            }
        }
#pragma unroll
        for (int j = 0; j < kHP; ++j) h[j] = dec_act(h[j], siren, d.omega_0);
        store_row(a, row, h);
        // dec1..dec4 + act on the tensor cores
        for (int l = 0; l < 4; ++l) {
            mlptc::fence_async_smem();
            mlptc::tc_before_sync();
            pipe_sync(pipe);
            mlptc::tc_after_sync();
            if (row == 0) {
                bool acc = false;
#pragma unroll
                for (int t = 0; t < 6; ++t)
#pragma unroll
                    for (int ks = 0; ks < kKSlabs; ++ks) {
                        mlptc::mma_bf16(tbase, mlptc::smem_desc(a[kPa[t]] + ks * kASlab),
                                        mlptc::smem_desc(s.w[l][kPw[t]] + ks * kWSlab), id, acc);
                        acc = true;
                    }
                mlptc::mma_commit(mbar);
            }
            ok = pipe_and(pipe, mlptc::mbar_wait(mbar, phase));
            phase ^= 1u;
            mlptc::tc_after_sync();
            if (!ok) break;  // uniform over the pipeline
            float acc[kHP];
            mlptc::tmem_ld32(tlane, acc);
#pragma unroll
            for (int j = 0; j < kHP; ++j) h[j] = dec_act(acc[j] + s.bh[l][j], siren, d.omega_0);
            // the layer's MMAs are done reading the A operands: overwrite them
            if (l < 3) store_row(a, row, h);
            mlptc::tc_before_sync();
        }
        if (!ok) break;
        // enc + invStandardizeQ
        float q[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float acc = s.be[c];
            const float4 *w4 = reinterpret_cast<const float4 *>(s.we[c]);
#pragma unroll
            for (int k = 0; k < kHP / 4; ++k) {
                const float4 w = w4[k];
                acc = fmaf(w.x, h[4 * k + 0], acc);
                acc = fmaf(w.y, h[4 * k + 1], acc);
                acc = fmaf(w.z, h[4 * k + 2], acc);
                acc = fmaf(w.w, h[4 * k + 3], acc);
            }
            q[c] = __fadd_rn(s.qm[c], __fmul_rn(acc, s.qs[c]));
        }
        if (live) {
            const float4 q5 = ldrec(st, i, 5);
            strec(st, i, 5, make_float4(q5.x, q5.y, q5.z, q[0]));
            strec(st, i, 6, make_float4(q[1], q[2], q[1], q[3]));
            strec(st, i, 7, make_float4(q[4], q[2], q[4], q[5]));
        }
    }
    if (!ok && row == 0) {
        atomicOr(status, MPM_ST_INTERNAL);
        // after a timed-out wait the MMAs may still run: a bounded grace period
        // before the tensor memory is released
        mlptc::mbar_wait(mbar, phase ^ 1u);
    }
    mlptc::tc_before_sync();
    __syncthreads();
    mlptc::tc_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(s.tmem_base),
                     "r"(kTmemCols * P)
                     : "memory");
}

int64_t decoder_param_floats(const MpmStressDecoder &d) {
    return blob_layout(d.hidden, d.label_dim + 3 + d.mu_dim).total;
}

static int dec_hp(int hidden) { return hidden <= 32 ? 32 : 64; }

static size_t dec_smem(const MpmStressDecoder &d) {
    return (size_t)dec_layout(dec_hp(d.hidden), d.label_dim + 3 + d.mu_dim).total * sizeof(float);
}

// opt each kernel in to the largest shared-memory copy once per device (not a
// stream operation, so launches stay capturable in CUDA graphs afterwards)
template <typename K>
static cudaError_t dec_prepare(K kernel, int slot) {
    static bool done[4][64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (done[slot][dev]) return cudaSuccess;
    const int in_max = 64 + 3 + 4;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(dec_layout(64, in_max).total * sizeof(float)));
    if (e == cudaSuccess) done[slot][dev] = true;
    return e;
}

cudaError_t launch_decoder_rows(const MpmStressDecoder &d, const float *rows, float *out, int64_t n, int num_sms,
                                cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const size_t smem = dec_smem(d);
    const int64_t want = (n + kDecThreads - 1) / kDecThreads;
    const int grid = (int)(want < (int64_t)num_sms * 8 ? want : (int64_t)num_sms * 8);
    cudaError_t e;
    if (dec_hp(d.hidden) == 32) {
        if ((e = dec_prepare(decoder_rows_kernel<32>, 0)) != cudaSuccess) return e;
        decoder_rows_kernel<32><<<grid, kDecThreads, smem, stream>>>(d, rows, out, n);
    } else {
        if ((e = dec_prepare(decoder_rows_kernel<64>, 1)) != cudaSuccess) return e;
        decoder_rows_kernel<64><<<grid, kDecThreads, smem, stream>>>(d, rows, out, n);
    }
    return cudaGetLastError();
}

cudaError_t launch_decoder_stress(const Ctx &cx, const MpmStressDecoder &d, const float *label, const float *mu) {
    if (cx.n == 0) return cudaSuccess;
    const size_t smem = dec_smem(d);
    const int want = (cx.n + kDecThreads - 1) / kDecThreads;
    const int grid = want < cx.num_sms * 8 ? want : cx.num_sms * 8;
    cudaError_t e;
    if (dec_hp(d.hidden) == 32) {
        // tensor cores: persistent CTAs of two tile pipelines sharing one weight
        // copy, three per SM (74 KB of shared memory and 64 tensor-memory columns
        // each); measured 8 % faster than one pipeline per CTA, four CTAs per SM
        constexpr int P = 2, per_sm = 3;
        static bool attr[64];
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
        const int bytes = (int)sizeof(dtc::Smem<P>);
        if (!attr[dev]) {
            e = cudaFuncSetAttribute(decoder_stress_tc_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
            attr[dev] = true;
        }
        const int tiles = (cx.n + dtc::kRows - 1) / dtc::kRows;
        const int groups = (tiles + P - 1) / P;
        const int tgrid = groups < cx.num_sms * per_sm ? groups : cx.num_sms * per_sm;
        decoder_stress_tc_kernel<P><<<tgrid, P * dtc::kRows, bytes, cx.stream>>>(d, cx.st, label, mu, cx.n,
                                                                                 cx.status);
    } else {
        if ((e = dec_prepare(decoder_stress_kernel<64>, 3)) != cudaSuccess) return e;
        decoder_stress_kernel<64><<<grid, kDecThreads, smem, cx.stream>>>(d, cx.st, label, mu, cx.n);
    }
    return cudaGetLastError();
}

}  // namespace mpm
