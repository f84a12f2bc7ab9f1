// C ABI of libmpm_gb300.so (declared in include/mpm_gb300.h): buffer layout,
// argument checks, and the launch sequence of the substep.
#include <nvtx3/nvToolsExt.h>
#include <stdio.h>
#include <string.h>

#include "mpm_launch.h"

namespace {

thread_local char g_cuda_err[256] = "";

int fail_cuda(cudaError_t e) {
    snprintf(g_cuda_err, sizeof(g_cuda_err), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return MPM_ERR_CUDA;
}

// NVTX range over one entry point, so a profiler's timeline shows the library's
// stages by name (header-only NVTX 3: a no-op unless a tool is attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

#define MPM_CHECK(expr)                          \
    do {                                         \
        cudaError_t e_ = (expr);                 \
        if (e_ != cudaSuccess) return fail_cuda(e_); \
    } while (0)

int num_sms() {
    static int cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (cache[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 148;
        cache[dev] = v;
    }
    return cache[dev];
}

constexpr int64_t kAlign = 256;
inline int64_t align_up(int64_t x, int64_t a = kAlign) { return (x + a - 1) / a * a; }

// particle-state buffer: `stride` records of 160 B, then `stride` int keys
constexpr int64_t kStateBytesPerParticle = mpm::kRecWords * 4 + 4;

struct WsLayout {
    int64_t order, counts, cell_counts, cell_start, cell_cursor, tile_sums, ticket, chunks, n_chunks,
        blocks, n_blocks, grid_acc, grid_v, block_flag, active_list, n_active, n_active_prev, staging,
        slot_of_uid, total;
    int nbk, n_tiles;
};

WsLayout ws_layout(const MpmPlan &p) {
    WsLayout L;
    const int64_t n = p.particle_stride;
    const int64_t nbk = p.total_blocks + 1;
    L.nbk = (int)nbk;
    L.n_tiles = (int)((nbk + mpm::kScanTile - 1) / mpm::kScanTile);
    int64_t o = 0;
    auto take = [&](int64_t bytes) { int64_t at = o; o = align_up(o + bytes); return at; };
    L.order = take(n * 4);
    L.counts = take(nbk * 4);
    L.cell_counts = take(nbk * 64 * 4);
    L.cell_start = take(nbk * 64 * 4);
    L.cell_cursor = take(nbk * 64 * 4);
    L.tile_sums = take((int64_t)L.n_tiles * 16);
    L.ticket = take(4);
    L.chunks = take(p.max_chunks * 16);
    L.n_chunks = take(4);
    L.blocks = take((p.total_blocks + 1) * 16);
    L.n_blocks = take(4);
    L.grid_acc = take(p.total_blocks * mpm::kBlockNodes * 16);
    L.grid_v = take(p.total_blocks * mpm::kBlockNodes * 16);
    L.block_flag = take(p.total_blocks * 4);
    L.active_list = take(p.total_blocks * 4);
    L.n_active = take(4);
    L.n_active_prev = take(4);
    // host transfers: [u, v, stress in: 15 n][u, v, F_disp, stress out: 2 x 24 n] (disjoint, so
    // the next step's input copy and export may run while this step's output copy is in flight)
    L.staging = take(n * 63 * 4);
    L.slot_of_uid = take(n * 4);
    L.total = o;
    return L;
}

}  // namespace

namespace mpm {
int record_cuda_error(cudaError_t e) { return fail_cuda(e); }
}  // namespace mpm

// bytes at the start of the workspace that a substep touches: everything
// but the host-transfer staging and the slot-of-uid table, which come last
int64_t mpm::substep_workspace_bytes(const MpmPlan &p) { return ws_layout(p).staging; }

namespace {

// [quads 0-3 of every slot][quads 4-7][quads 8-9][cell keys]; stride is a
// multiple of 64 slots, so every array starts 4 KB-aligned
mpm::PState state_view(void *base, int64_t stride) {
    mpm::PState s;
    char *p = static_cast<char *>(base);
    s.stride = stride;
    s.a = reinterpret_cast<float4 *>(p);
    s.b = reinterpret_cast<float4 *>(p + stride * 64);
    s.f = reinterpret_cast<float4 *>(p + stride * 128);
    s.key = reinterpret_cast<int *>(p + stride * mpm::kRecWords * 4);
    return s;
}

mpm::Ctx make_ctx(const MpmBuffers *b, void *stream, int which) {
    const MpmPlan &p = b->plan;
    WsLayout L = ws_layout(p);
    char *w = static_cast<char *>(b->workspace);
    mpm::Ctx cx;
    cx.scenes = static_cast<const MpmScene *>(b->scenes);
    cx.n_scenes = p.n_scenes;
    cx.st = state_view(b->state[which], p.particle_stride);
    cx.st2 = state_view(b->state[which ^ 1], p.particle_stride);
    mpm::Ws &ws = cx.ws;
    ws.order = reinterpret_cast<int *>(w + L.order);
    ws.counts = reinterpret_cast<int *>(w + L.counts);
    ws.cell_counts = reinterpret_cast<int *>(w + L.cell_counts);
    ws.cell_start = reinterpret_cast<int *>(w + L.cell_start);
    ws.cell_cursor = reinterpret_cast<int *>(w + L.cell_cursor);
    ws.tile_sums = reinterpret_cast<int4 *>(w + L.tile_sums);
    ws.ticket = reinterpret_cast<unsigned *>(w + L.ticket);
    ws.chunks = reinterpret_cast<int4 *>(w + L.chunks);
    ws.n_chunks = reinterpret_cast<int *>(w + L.n_chunks);
    ws.blocks = reinterpret_cast<int4 *>(w + L.blocks);
    ws.n_blocks = reinterpret_cast<int *>(w + L.n_blocks);
    ws.grid_acc = reinterpret_cast<float4 *>(w + L.grid_acc);
    ws.grid_v = reinterpret_cast<float4 *>(w + L.grid_v);
    ws.block_flag = reinterpret_cast<int *>(w + L.block_flag);
    ws.active_list = reinterpret_cast<int *>(w + L.active_list);
    ws.n_active = reinterpret_cast<int *>(w + L.n_active);
    ws.n_active_prev = reinterpret_cast<int *>(w + L.n_active_prev);
    ws.staging = reinterpret_cast<float *>(w + L.staging);
    ws.slot_of_uid = reinterpret_cast<int *>(w + L.slot_of_uid);
    ws.nbk = L.nbk;
    ws.n_tiles = L.n_tiles;
    ws.max_chunks = (int)p.max_chunks;
    ws.chunk_size = p.chunk_size;
    ws.n = (int)p.n_particles;
    cx.n = (int)p.n_particles;
    cx.status = b->status;
    cx.stream = static_cast<cudaStream_t>(stream);
    cx.num_sms = num_sms();
    cx.total_blocks = p.total_blocks;
    return cx;
}

bool buffers_ok(const MpmBuffers *b) {
    return b && b->state[0] && b->state[1] && b->workspace && b->scenes && b->status &&
           b->plan.n_scenes >= 1 && (b->cur == 0 || b->cur == 1);
}

}  // namespace

extern "C" {

int mpm_abi_version(void) { return MPM_ABI_VERSION; }

void mpm_struct_sizes(int64_t *out) {
    if (!out) return;
    out[0] = sizeof(MpmCollider);
    out[1] = sizeof(MpmScene);
    out[2] = sizeof(MpmPlan);
    out[3] = sizeof(MpmBuffers);
    out[4] = sizeof(MpmReducedGrid);
    out[5] = sizeof(MpmStressDecoder);
}

const char *mpm_error_string(int code) {
    switch (code) {
        case MPM_OK: return "ok";
        case MPM_ERR_ARG: return "invalid argument";
        case MPM_ERR_CUDA: return "CUDA runtime error";
        case MPM_ERR_SIZE: return "size exceeds the planned buffers";
        default: return "unknown error";
    }
}

const char *mpm_last_cuda_error(void) { return g_cuda_err; }

int mpm_plan(MpmScene *scenes, int32_t n_scenes, int64_t n_particles, int32_t chunk_size,
             MpmPlan *plan) {
    if (!scenes || !plan || n_scenes < 1 || n_particles < 0) return MPM_ERR_ARG;
    if (chunk_size == 0) chunk_size = 128;
    if (chunk_size != 32 && chunk_size != 64 && chunk_size != 128 && chunk_size != 256)
        return MPM_ERR_ARG;
    if (n_particles >= (int64_t)1 << 30) return MPM_ERR_SIZE;
    int64_t next_particle = 0, blocks = 0;
    for (int s = 0; s < n_scenes; ++s) {
        MpmScene &S = scenes[s];
        if (S.n_grid < 3 || S.n_grid > 4096 || !(S.dx > 0.0f) || !(S.inv_dx > 0.0f)) return MPM_ERR_ARG;
        if (S.material < MPM_JELLY || S.material > MPM_SAND) return MPM_ERR_ARG;
        if (S.n_colliders < 0 || S.n_colliders > MPM_MAX_COLLIDERS) return MPM_ERR_ARG;
        if (S.particle_begin != next_particle || S.particle_count < 0) return MPM_ERR_ARG;
        next_particle += S.particle_count;
        S.n_blocks_axis = (S.n_grid + 3) / 4;
        S.block_begin = blocks;
        blocks += (int64_t)S.n_blocks_axis * S.n_blocks_axis * S.n_blocks_axis;
    }
    if (next_particle != n_particles) return MPM_ERR_ARG;
    if (blocks + 1 >= ((int64_t)1 << 31) / mpm::kBlockNodes) return MPM_ERR_SIZE;
    MpmPlan p;
    memset(&p, 0, sizeof(p));
    p.n_particles = n_particles;
    p.particle_stride = align_up(n_particles > 0 ? n_particles : 1, 64);
    p.total_blocks = blocks;
    p.chunk_size = chunk_size;
    p.n_scenes = n_scenes;
    const int64_t nonempty = n_particles < blocks ? n_particles : blocks;
    // G2P chunks of the blocks, plus the out-of-domain copy chunks
    p.max_chunks = 2 * (n_particles / chunk_size) + nonempty + 2;
    p.state_bytes = kStateBytesPerParticle * p.particle_stride;
    p.workspace_bytes = ws_layout(p).total;
    *plan = p;
    return MPM_OK;
}

int mpm_init(MpmBuffers *b, void *stream) {
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPM_CHECK(cudaMemsetAsync(b->state[0], 0, b->plan.state_bytes, st));
    MPM_CHECK(cudaMemsetAsync(b->state[1], 0, b->plan.state_bytes, st));
    MPM_CHECK(cudaMemsetAsync(b->workspace, 0, b->plan.workspace_bytes, st));
    MPM_CHECK(cudaMemsetAsync(b->status, 0, sizeof(int32_t), st));
    b->cur = 0;
    b->keys_valid = 0;
    b->substep = 0;
    mpm::Ctx cx = make_ctx(b, stream, 0);
    mpm::PState other = state_view(b->state[1], b->plan.particle_stride);
    MPM_CHECK(mpm::launch_init_state(cx, other));
    return MPM_OK;
}

int mpm_upload_scenes(MpmBuffers *b, const MpmScene *scenes, int32_t n_scenes, void *stream) {
    if (!b || !b->scenes || !scenes || n_scenes != b->plan.n_scenes) return MPM_ERR_ARG;
    int flags = 0;
    for (int s = 0; s < n_scenes; ++s) {
        if (scenes[s].n_colliders < 0 || scenes[s].n_colliders > MPM_MAX_COLLIDERS) return MPM_ERR_ARG;
        for (int k = 0; k < scenes[s].n_colliders; ++k) {
            const int kind = scenes[s].colliders[k].kind;
            if (kind < MPM_COLLIDER_SURFACE || kind > MPM_COLLIDER_SPHERE) return MPM_ERR_ARG;
            if (kind >= MPM_COLLIDER_VPLANE) flags |= MPM_CF_EXTENDED;
            if (kind == MPM_COLLIDER_VPLANE || kind == MPM_COLLIDER_CIRCLE || kind == MPM_COLLIDER_CUBE ||
                kind == MPM_COLLIDER_SPHERE)
                flags |= MPM_CF_MOVING;
        }
    }
    b->collider_flags = flags;
    MPM_CHECK(cudaMemcpyAsync(b->scenes, scenes, sizeof(MpmScene) * (size_t)n_scenes,
                              cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_load(MpmBuffers *b, int32_t field, const float *src, int32_t src_on_host, void *stream) {
    if (!buffers_ok(b) || (!src && b->plan.n_particles > 0) || field < MPM_FIELD_X_INITIAL ||
        field > MPM_FIELD_YIELD)
        return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    const float *from = src;
    if (src_on_host) {
        size_t bytes = (size_t)cx.n * mpm::field_components(field) * sizeof(float);
        if (bytes) MPM_CHECK(cudaMemcpyAsync(cx.ws.staging, src, bytes, cudaMemcpyHostToDevice, cx.stream));
        from = cx.ws.staging;
    }
    MPM_CHECK(mpm::launch_load(cx, field, from));
    if (field == MPM_FIELD_X_INITIAL || field == MPM_FIELD_U) b->keys_valid = 0;
    return MPM_OK;
}

int mpm_export(MpmBuffers *b, int32_t field, float *dst, int32_t dst_on_host, void *stream) {
    if (!buffers_ok(b) || (!dst && b->plan.n_particles > 0) || field < MPM_FIELD_X_INITIAL ||
        field > MPM_FIELD_F_DISP)
        return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    float *to = dst_on_host ? cx.ws.staging : dst;
    MPM_CHECK(mpm::launch_export(cx, field, to));
    if (dst_on_host) {
        size_t bytes = (size_t)cx.n * mpm::field_components(field) * sizeof(float);
        if (bytes) MPM_CHECK(cudaMemcpyAsync(dst, to, bytes, cudaMemcpyDeviceToHost, cx.stream));
        MPM_CHECK(cudaStreamSynchronize(cx.stream));
    }
    return MPM_OK;
}

// Side streams per device for the host copies of mpm_load_uvstress (input
// lane) and mpm_export_uvFstress (output lane), and the events that order
// them against the caller's stream.  An input copy waits only until the
// previous load kernel has consumed the input staging.  Exports alternate
// between two output staging halves: an output copy waits for its export
// kernel, and an export kernel waits only for the copy that last drained
// its half (two exports back).  So the input copy of one step, the output
// copy of the step before and the substep itself can all run at once, and
// the output copies run back to back.
namespace {
struct CopyLane {
    cudaStream_t stream = nullptr;
    cudaEvent_t ready = nullptr, done[2] = {nullptr, nullptr};
    int parity = 0;
};
CopyLane g_in[64], g_out[64];

cudaError_t lane_of(CopyLane *lanes, CopyLane *&lane) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    CopyLane &L = lanes[dev];
    if (!L.stream) {
        if ((e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking)) != cudaSuccess) return e;
        if ((e = cudaEventCreateWithFlags(&L.ready, cudaEventDisableTiming)) != cudaSuccess) return e;
        for (cudaEvent_t &d : L.done)
            if ((e = cudaEventCreateWithFlags(&d, cudaEventDisableTiming)) != cudaSuccess) return e;
    }
    lane = &L;
    return cudaSuccess;
}
}  // namespace

int mpm_sync_transfers(void) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPM_ERR_CUDA;
    for (CopyLane *L : {&g_in[dev], &g_out[dev]})
        if (L->stream) MPM_CHECK(cudaStreamSynchronize(L->stream));
    return MPM_OK;
}

int mpm_load_uvstress(MpmBuffers *b, const float *u, const float *v, const float *stress, int32_t src_on_host,
                      void *stream) {
    NvtxRange nvtx_("mpm_load_uvstress");
    if (!buffers_ok(b) || (b->plan.n_particles > 0 && (!u || !v || !stress))) return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    if (cx.n == 0) return MPM_OK;
    if (!src_on_host) {
        MPM_CHECK(mpm::launch_load_uvstress(cx, u, v, stress));
        b->keys_valid = 0;  // u moved the particles
        return MPM_OK;
    }
    const size_t n = (size_t)cx.n;
    float *s = cx.ws.staging;  // input region: u, v, stress
    CopyLane *L = nullptr;
    MPM_CHECK(lane_of(g_in, L));
    MPM_CHECK(cudaStreamWaitEvent(L->stream, L->done[0], 0));  // no-op before the first load
    MPM_CHECK(cudaMemcpyAsync(s, u, n * 12, cudaMemcpyHostToDevice, L->stream));
    MPM_CHECK(cudaMemcpyAsync(s + 3 * n, v, n * 12, cudaMemcpyHostToDevice, L->stream));
    MPM_CHECK(cudaMemcpyAsync(s + 6 * n, stress, n * 36, cudaMemcpyHostToDevice, L->stream));
    MPM_CHECK(cudaEventRecord(L->ready, L->stream));
    MPM_CHECK(cudaStreamWaitEvent(cx.stream, L->ready, 0));
    MPM_CHECK(mpm::launch_load_uvstress(cx, s, s + 3 * n, s + 6 * n));
    MPM_CHECK(cudaEventRecord(L->done[0], cx.stream));  // input staging consumed
    b->keys_valid = 0;
    return MPM_OK;
}

int mpm_export_uvFstress(MpmBuffers *b, float *u, float *v, float *F_disp, float *stress, int32_t dst_on_host,
                         void *stream) {
    NvtxRange nvtx_("mpm_export_uvFstress");
    if (!buffers_ok(b) || (b->plan.n_particles > 0 && (!u || !v || !F_disp || !stress))) return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    if (cx.n == 0) return MPM_OK;
    const size_t n = (size_t)cx.n;
    if (!dst_on_host) {
        MPM_CHECK(mpm::launch_export_uvFstress(cx, u, v, F_disp, stress));
        return MPM_OK;
    }
    CopyLane *L = nullptr;
    MPM_CHECK(lane_of(g_out, L));
    const int h = L->parity;
    L->parity ^= 1;
    float *s = cx.ws.staging + 15 * n + (size_t)h * 24 * n;  // output half h: u, v, F_disp, stress
    MPM_CHECK(cudaStreamWaitEvent(cx.stream, L->done[h], 0));  // the copy that last used half h drained it
    MPM_CHECK(mpm::launch_export_uvFstress(cx, s, s + 3 * n, s + 6 * n, s + 15 * n));
    MPM_CHECK(cudaEventRecord(L->ready, cx.stream));
    MPM_CHECK(cudaStreamWaitEvent(L->stream, L->ready, 0));
    MPM_CHECK(cudaMemcpyAsync(u, s, n * 12, cudaMemcpyDeviceToHost, L->stream));
    MPM_CHECK(cudaMemcpyAsync(v, s + 3 * n, n * 12, cudaMemcpyDeviceToHost, L->stream));
    MPM_CHECK(cudaMemcpyAsync(F_disp, s + 6 * n, n * 36, cudaMemcpyDeviceToHost, L->stream));
    MPM_CHECK(cudaMemcpyAsync(stress, s + 15 * n, n * 36, cudaMemcpyDeviceToHost, L->stream));
    MPM_CHECK(cudaEventRecord(L->done[h], L->stream));
    if (dst_on_host == 1) MPM_CHECK(cudaEventSynchronize(L->done[h]));
    return MPM_OK;
}

int mpm_export_frame(MpmBuffers *b, float *out, void *stream) {
    NvtxRange nvtx_("mpm_export_frame");
    if (!buffers_ok(b) || (b->plan.n_particles > 0 && !out)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_export_frame(make_ctx(b, stream, b->cur), out));
    return MPM_OK;
}

int mpm_sort(MpmBuffers *b, void *stream) {
    NvtxRange nvtx_("mpm_sort");
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    if (!b->keys_valid) {
        MPM_CHECK(cudaMemsetAsync(cx.ws.counts, 0, (size_t)cx.ws.nbk * sizeof(int), cx.stream));
        MPM_CHECK(cudaMemsetAsync(cx.ws.cell_counts, 0, (size_t)cx.ws.nbk * 64 * sizeof(int), cx.stream));
        MPM_CHECK(mpm::launch_keys(cx));
        b->keys_valid = 1;
    }
    MPM_CHECK(mpm::launch_sort(cx));
    return MPM_OK;
}

int mpm_p2g(MpmBuffers *b, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g");
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_p2g(make_ctx(b, stream, b->cur), dt));
    return MPM_OK;
}

int mpm_grid_update(MpmBuffers *b, float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_grid_update");
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_grid(make_ctx(b, stream, b->cur), time, dt));
    if (b->collider_flags & MPM_CF_MOVING)  // after every node used the old points
        MPM_CHECK(mpm::launch_advance_colliders(static_cast<MpmScene *>(b->scenes), b->plan.n_scenes, time, dt,
                                                static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_g2p(MpmBuffers *b, float dt, void *stream) {
    NvtxRange nvtx_("mpm_g2p");
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_g2p(make_ctx(b, stream, b->cur), dt));
    b->cur ^= 1;  // G2P wrote the sorted, updated records into the other buffer
    b->substep += 1;
    return MPM_OK;
}

int64_t mpm_p2g_ordered_bytes(const MpmPlan *plan) {
    if (!plan || plan->total_blocks < 0) return -1;
    return mpm::ordered_scratch_bytes(plan->total_blocks);
}

int mpm_p2g_ordered(MpmBuffers *b, void *scratch, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g_ordered");
    if (!buffers_ok(b) || !scratch) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_p2g_ordered(make_ctx(b, stream, b->cur), dt, scratch));
    return MPM_OK;
}

int mpm_p2g2p_ordered(MpmBuffers *b, void *scratch, float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g2p_ordered");
    int r = mpm_sort(b, stream);
    if (r) return r;
    if ((r = mpm_p2g_ordered(b, scratch, dt, stream))) return r;
    if ((r = mpm_grid_update(b, time, dt, stream))) return r;
    return mpm_g2p(b, dt, stream);
}

int mpm_p2g2p(MpmBuffers *b, float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g2p");
    int r = mpm_sort(b, stream);
    if (r) return r;
    if ((r = mpm_p2g(b, dt, stream))) return r;
    if ((r = mpm_grid_update(b, time, dt, stream))) return r;
    return mpm_g2p(b, dt, stream);
}

static bool surrogate_cfg_ok(const MpmSurrogateConfig *c) {
    // dgamma_max <= 0.25 keeps the exp series of the plastic F update exact to 1e-8
    return c && c->tol >= 0.0f && c->rho_min >= 0.0f && c->rho_min <= c->rho_max &&
           c->nu_min <= c->nu_max && c->phi_min <= c->phi_max && c->dgamma_max >= 0.0f &&
           c->dgamma_max <= 0.25f;
}

int mpm_surrogate_features(const MpmScene *scene, const float *F, const float *stress, float *x, float *y,
                           int64_t n, void *stream) {
    if (!scene || n < 0 || (n > 0 && (!F || !x || (stress && !y)))) return MPM_ERR_ARG;
    if (!(scene->mu > 0.0f)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_features(*scene, F, stress, x, y, n, static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_mlp_forward_tc(const void *params, const float *x, float *y, const float *target, void *zsave, void *dy,
                       float *loss, float grad_scale, int64_t n, int32_t *err, void *stream) {
    if (!params || !err || n < 0 || (n > 0 && !x)) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(params) & 15) return MPM_ERR_ARG;
    if ((target != nullptr) != (dy != nullptr)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_mlp_forward_tc(params, x, y, target, zsave, dy, loss, grad_scale, n, err, num_sms(),
                                         static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_mlp_backward_tc(const void *params, const float *x, const void *zsave, const void *dy, float *grad,
                        int64_t n, int32_t *err, void *stream) {
    if (!params || !err || !grad || n < 0 || (n > 0 && (!x || !zsave || !dy))) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(params) & 15 || reinterpret_cast<uintptr_t>(grad) & 15 ||
        reinterpret_cast<uintptr_t>(zsave) & 15 || reinterpret_cast<uintptr_t>(dy) & 15)
        return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_mlp_backward_tc(params, x, zsave, dy, grad, n, err, num_sms(),
                                          static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_surrogate_apply(const MpmScene *scene, const void *mlp_params, const MpmSurrogateConfig *cfg,
                        const float *F_trial, float *F, float *stress, int32_t *codes, int64_t n, void *stream) {
    if (!scene || !mlp_params || !surrogate_cfg_ok(cfg) || n < 0) return MPM_ERR_ARG;
    if (n > 0 && (!F_trial || !F || !stress || !codes)) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(mlp_params) & 15) return MPM_ERR_ARG;
    int dev = 0, sms = 0;
    MPM_CHECK(cudaGetDevice(&dev));
    MPM_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MPM_CHECK(mpm::launch_surrogate_apply(*scene, mlp_params, *cfg, F_trial, F, stress, codes, n, sms,
                                          static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_g2p_surrogate(MpmBuffers *b, const void *mlp_params, const MpmSurrogateConfig *cfg, void *fallback,
                      int32_t *stats, float dt, void *stream) {
    NvtxRange nvtx_("mpm_g2p_surrogate");
    if (!buffers_ok(b) || !mlp_params || !surrogate_cfg_ok(cfg) || !stats) return MPM_ERR_ARG;
    if (b->plan.n_particles > 0 && (!fallback || (reinterpret_cast<uintptr_t>(fallback) & 7))) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(mlp_params) & 15) return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    MPM_CHECK(mpm::launch_g2p(cx, dt, true));
    MPM_CHECK(mpm::launch_surrogate(cx, mlp_params, *cfg, static_cast<int2 *>(fallback), stats));
    b->cur ^= 1;  // as mpm_g2p: the updated records are in the other buffer
    b->substep += 1;
    return MPM_OK;
}

int mpm_p2g2p_surrogate(MpmBuffers *b, const void *mlp_params, const MpmSurrogateConfig *cfg, void *fallback,
                        int32_t *stats, float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g2p_surrogate");
    if (!buffers_ok(b) || !mlp_params || !surrogate_cfg_ok(cfg) || !stats) return MPM_ERR_ARG;
    int r = mpm_sort(b, stream);
    if (r) return r;
    if ((r = mpm_p2g(b, dt, stream))) return r;
    if ((r = mpm_grid_update(b, time, dt, stream))) return r;
    return mpm_g2p_surrogate(b, mlp_params, cfg, fallback, stats, dt, stream);
}

int mpm_adjoint_substep(MpmBuffers *b, const float *adj_out, float *adj_in, void *grid_adj, double *theta_bar,
                        float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_adjoint_substep");
    if (!buffers_ok(b) || !theta_bar || !grid_adj) return MPM_ERR_ARG;
    if (b->plan.n_particles > 0 && (!adj_out || !adj_in || adj_out == adj_in)) return MPM_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(grid_adj) & 15) return MPM_ERR_ARG;
    if (b->collider_flags & MPM_CF_EXTENDED) return MPM_ERR_ARG;  // surface and box colliders only
    MPM_CHECK(mpm::launch_adjoint(make_ctx(b, stream, b->cur), adj_out, adj_in, static_cast<float4 *>(grid_adj),
                                  theta_bar, time, dt));
    return MPM_OK;
}

int64_t mpm_substep_grid_bytes(const MpmPlan *plan) {
    if (!plan) return -1;
    return mpm::substep_grid_bytes(plan->total_blocks, plan->n_particles, plan->max_chunks);
}

int mpm_save_substep_grid(MpmBuffers *b, void *dst, void *stream) {
    NvtxRange nvtx_("mpm_save_substep_grid");
    if (!buffers_ok(b) || !dst || (reinterpret_cast<uintptr_t>(dst) & 255)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_save_grid(make_ctx(b, stream, b->cur), dst));
    return MPM_OK;
}

int mpm_load_substep_grid(MpmBuffers *b, const void *src, void *stream) {
    NvtxRange nvtx_("mpm_load_substep_grid");
    if (!buffers_ok(b) || !src || (reinterpret_cast<uintptr_t>(src) & 255)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_load_grid(make_ctx(b, stream, b->cur), src));
    return MPM_OK;
}

int mpm_clear_grid(MpmBuffers *b, void *stream) {
    if (!buffers_ok(b)) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_clear_grid(make_ctx(b, stream, b->cur)));
    return MPM_OK;
}

int mpm_return_map_vjp(const MpmScene *scene, const float *F_trial, const float *F_bar, const float *stress_bar,
                       float *F_trial_bar, double *theta_bar, int64_t n, void *stream) {
    if (!scene || !theta_bar || n < 0) return MPM_ERR_ARG;
    if (n > 0 && (!F_trial || !F_bar || !stress_bar || !F_trial_bar)) return MPM_ERR_ARG;
    if (scene->material != MPM_SAND) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_return_map_vjp(*scene, F_trial, F_bar, stress_bar, F_trial_bar, theta_bar, n,
                                         static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

static int reduced_args_ok(const MpmBuffers *b, const MpmReducedGrid *g) {
    if (!buffers_ok(b) || !g || b->plan.n_scenes != 1) return MPM_ERR_ARG;
    if (g->n_samples < 0 || (g->n_samples > 0 && !g->sample_index) || g->n_grid < 1) return MPM_ERR_ARG;
    if (!g->f_disp || !g->density || !g->grid_acc || !g->grid_m || !g->grid_v_in || !g->grid_v_out ||
        !g->neighboring_cells || !g->neighboring_cells_grid_v)
        return MPM_ERR_ARG;
    if (g->n_samples > ((int64_t)1 << 26) || g->n_grid > 1024) return MPM_ERR_SIZE;
    return MPM_OK;
}

int mpm_p2g2p_reduced(MpmBuffers *b, const MpmReducedGrid *g, float time, float dt, void *stream) {
    NvtxRange nvtx_("mpm_p2g2p_reduced");
    int r = reduced_args_ok(b, g);
    if (r) return r;
    MPM_CHECK(mpm::launch_p2g2p_reduced(make_ctx(b, stream, b->cur), *g, time, dt));
    if (b->collider_flags & MPM_CF_MOVING)  // the reference's modify_bc after each collider sweep
        MPM_CHECK(mpm::launch_advance_colliders(static_cast<MpmScene *>(b->scenes), b->plan.n_scenes, time, dt,
                                                static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_mark_neighboring_cells_grid_v(MpmBuffers *b, const MpmReducedGrid *g, void *stream) {
    NvtxRange nvtx_("mpm_mark_neighboring_cells_grid_v");
    int r = reduced_args_ok(b, g);
    if (r) return r;
    MPM_CHECK(mpm::launch_mark_grid_v(make_ctx(b, stream, b->cur), *g));
    return MPM_OK;
}

int mpm_g2p_sample(MpmBuffers *b, const MpmReducedGrid *g, float dt, void *stream) {
    NvtxRange nvtx_("mpm_g2p_sample");
    int r = reduced_args_ok(b, g);
    if (r) return r;
    MPM_CHECK(mpm::launch_g2p_sample(make_ctx(b, stream, b->cur), *g, dt));
    b->keys_valid = 0;  // the sample points moved
    return MPM_OK;
}

static bool decoder_ok(const MpmStressDecoder *d) {
    return d && d->params && d->label_dim >= 0 && d->label_dim <= 64 && d->mu_dim >= 0 && d->mu_dim <= 4 &&
           d->hidden >= 1 && d->hidden <= 64 && (d->siren == 0 || d->siren == 1) && d->omega_0 == d->omega_0;
}

int64_t mpm_decoder_param_count(const MpmStressDecoder *d) {
    if (!d || d->label_dim < 0 || d->label_dim > 64 || d->mu_dim < 0 || d->mu_dim > 4 || d->hidden < 1 ||
        d->hidden > 64)
        return MPM_ERR_ARG;
    return mpm::decoder_param_floats(*d);
}

int mpm_decoder_forward(const MpmStressDecoder *d, const float *rows, float *out, int64_t n, void *stream) {
    NvtxRange nvtx_("mpm_decoder_forward");
    if (!decoder_ok(d) || n < 0 || (n > 0 && (!rows || !out))) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_decoder_rows(*d, rows, out, n, num_sms(), static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_decoder_stress(MpmBuffers *b, const MpmStressDecoder *d, const float *label, const float *mu,
                       void *stream) {
    NvtxRange nvtx_("mpm_decoder_stress");
    if (!buffers_ok(b) || !decoder_ok(d) || (d->label_dim > 0 && !label) || (d->mu_dim > 0 && !mu))
        return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_decoder_stress(make_ctx(b, stream, b->cur), *d, label, mu));
    return MPM_OK;
}

int mpm_export_grid(MpmBuffers *b, int32_t scene, float *grid_m, float *grid_v_in,
                    float *grid_v_out, void *stream) {
    if (!buffers_ok(b) || scene < 0 || scene >= b->plan.n_scenes) return MPM_ERR_ARG;
    mpm::Ctx cx = make_ctx(b, stream, b->cur);
    MpmScene S;
    MPM_CHECK(cudaMemcpyAsync(&S, cx.scenes + scene, sizeof(S), cudaMemcpyDeviceToHost, cx.stream));
    MPM_CHECK(cudaStreamSynchronize(cx.stream));
    MPM_CHECK(mpm::launch_export_grid(cx, S, scene, grid_m, grid_v_in, grid_v_out));
    return MPM_OK;
}

int mpm_svd3(const float *A, float *U, float *s, float *V, int64_t n, void *stream) {
    if (n < 0 || (n > 0 && (!A || !U || !s || !V))) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_svd3(A, U, s, V, n, static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_return_map(const MpmScene *scene, const float *F_trial, float *yield, float *F,
                   float *stress, int64_t n, void *stream) {
    if (!scene || n < 0 || (n > 0 && (!F_trial || !F || !stress))) return MPM_ERR_ARG;
    if (scene->material == MPM_METAL && n > 0 && !yield) return MPM_ERR_ARG;
    MPM_CHECK(mpm::launch_return_map(*scene, F_trial, yield, F, stress, n,
                                     static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

}  // extern "C"
