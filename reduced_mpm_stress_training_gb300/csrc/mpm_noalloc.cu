// mpm_p2g2p_noalloc: the substep for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc: a host framework that has already
// reserved (nearly) all device memory for its own pool, code running inside
// a stream capture or a real-time loop where allocation is not allowed, or a
// plugin whose host only hands it the particle arrays.  They can still own
// the particle-state buffers, the scene table and the status word (the
// inputs and outputs), but not the substep's scratch (sort keys and offsets,
// work lists, the block-sparse grid).  This entry point keeps that scratch in
// one file-scope device array of fixed size instead of the caller's
// MpmBuffers.workspace.
//
// Limits and behaviour:
//   * The array is kNoAllocWorkspaceBytes (16 MiB) and every GPU that loads
//     the library holds it until the process exits.  It holds the part of
//     the workspace a substep uses (all but the host-transfer staging, which
//     this entry point never touches); plans whose substep part exceeds it
//     are rejected with MPM_ERR_SIZE (16 MiB covers a 64^3 grid -- about
//     11 MiB of grid and cell arrays -- with up to about a million
//     particles at 4-5 bytes each; a 128^3 grid does not fit).
//   * All calls share the array, and it keeps the last call's contents.  Each
//     call therefore clears the part it uses and recomputes the sort keys
//     from the particle positions (a full re-sort every call), so calls from
//     different simulators may alternate.  Calls whose work overlaps on the
//     GPU (different streams, or different host threads) race on the array.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture.  Later calls only enqueue work.
//   * Nothing here calls cudaMalloc, cudaFree or any allocating routine.
#include <mutex>
#include <stdio.h>

#include "mpm_launch.h"

namespace {

constexpr size_t kNoAllocWorkspaceBytes = size_t(16) << 20;

static __device__ __align__(256) unsigned char g_noalloc_workspace[kNoAllocWorkspaceBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[64] = {nullptr};

// device address of g_noalloc_workspace on the current device (set-up once
// per device); nullptr on failure
void *noalloc_workspace(int *err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        *err = mpm::record_cuda_error(e != cudaSuccess ? e : cudaErrorInvalidDevice);
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_workspace);
        if (e != cudaSuccess || !p) {
            *err = mpm::record_cuda_error(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
            return nullptr;
        }
        g_noalloc_ptr[dev] = p;
    }
    return g_noalloc_ptr[dev];
}

}  // namespace

extern "C" int mpm_p2g2p_noalloc(MpmBuffers *b, float time, float dt, void *stream) {
    if (!b || !b->state[0] || !b->state[1] || !b->scenes || !b->status) return MPM_ERR_ARG;
    const int64_t need = mpm::substep_workspace_bytes(b->plan);
    if (need < 0 || (size_t)need > kNoAllocWorkspaceBytes) return MPM_ERR_SIZE;
    int err = MPM_OK;
    void *ws = noalloc_workspace(&err);
    if (!ws) return err;
    // the array holds whatever the last call left: start from a cleared
    // workspace and keys recomputed from the positions
    cudaError_t e = cudaMemsetAsync(ws, 0, (size_t)need, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return mpm::record_cuda_error(e);
    MpmBuffers local = *b;
    local.workspace = ws;
    local.keys_valid = 0;
    const int r = mpm_p2g2p(&local, time, dt, stream);
    b->cur = local.cur;
    b->substep = local.substep;
    b->keys_valid = 0;  // the caller's own workspace holds no histograms for these keys
    return r;
}
