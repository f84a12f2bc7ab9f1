// Data movement between the reference layout (AoS vec3 / mat33 arrays in the
// user's particle order) and the internal sorted particle records, the dense
// grid export, and the batched element kernels (SVD, return map) used for
// unit-level checks.
#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

int field_components(int field) {
    switch (field) {
        case MPM_FIELD_X_INITIAL: case MPM_FIELD_U: case MPM_FIELD_V: case MPM_FIELD_X: return 3;
        case MPM_FIELD_C: case MPM_FIELD_F: case MPM_FIELD_STRESS: case MPM_FIELD_F_DISP: return 9;
        case MPM_FIELD_MASS: case MPM_FIELD_VOL: case MPM_FIELD_YIELD: return 1;
        default: return 0;
    }
}

// record word of component c of a field (see the record layout in mpm_device.cuh)
__device__ __forceinline__ int field_word(int field, int c) {
    switch (field) {
        case MPM_FIELD_X_INITIAL: case MPM_FIELD_X: return rec::X0 + c;
        case MPM_FIELD_U: return rec::U + c;
        case MPM_FIELD_V: return rec::V + c;
        case MPM_FIELD_C: return rec::C + c;
        case MPM_FIELD_STRESS: return rec::TAU + c;
        case MPM_FIELD_F: case MPM_FIELD_F_DISP: return c < 8 ? rec::F0 + c : rec::F8;
        case MPM_FIELD_MASS: return rec::MASS;
        case MPM_FIELD_VOL: return rec::VOL;
        default: return rec::YLD;  // MPM_FIELD_YIELD
    }
}

// initial values of MPM_Simulator_WARP.initialize (mpm_solver_warp.py:52-69):
// zero everything, F = I (as load_from_sampling leaves it, :149), slot = user index
__global__ void init_state_kernel(PState a, PState b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < kRecQuads; ++q) {
        strec(a, i, q, z);
        strec(b, i, q, z);
    }
    recword(a, i, rec::F0) = recword(a, i, rec::F0 + 4) = recword(a, i, rec::F8) = 1.0f;
    recword(b, i, rec::F0) = recword(b, i, rec::F0 + 4) = recword(b, i, rec::F8) = 1.0f;
    recword(a, i, rec::UID) = __int_as_float(i);
    recword(b, i, rec::UID) = __int_as_float(i);
    a.key[i] = -1;
    b.key[i] = -1;
}

__global__ void load_kernel(PState st, int n, int field, int nc, const float *__restrict__ src) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t u = __float_as_int(recword(st, i, rec::UID));
    for (int c = 0; c < nc; ++c) recword(st, i, field_word(field, c)) = src[u * nc + c];
}

__global__ void export_kernel(PState st, int n, int field, int nc, float *__restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t u = __float_as_int(recword(st, i, rec::UID));
    for (int c = 0; c < nc; ++c) {
        float v = recword(st, i, field_word(field, c));
        if (field == MPM_FIELD_X) v = __fadd_rn(v, recword(st, i, rec::U + c));    // x0 + u (:5-7)
        if (field == MPM_FIELD_F_DISP) v = v - ((c % 4 == 0) ? 1.0f : 0.0f);       // F - I (:16-19)
        dst[u * nc + c] = v;
    }
}

// slot_of_uid[uid] = slot for the live state: the two transfer kernels below
// walk the particles in USER order, so their host-side arrays are read and
// written coalesced and only the 160-byte records are gathered (whole
// sectors) -- scattering 12- and 36-byte rows by uid instead leaves partial
// sectors that L2 cannot merge once the arrays outgrow it
__global__ void slot_of_uid_kernel(PState st, int n, int *__restrict__ inv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    inv[__float_as_int(ldrec(st, i, 1).y)] = i;
}

cudaError_t launch_slot_of_uid(const Ctx &cx) {
    if (cx.n == 0) return cudaSuccess;
    slot_of_uid_kernel<<<(unsigned)((cx.n + 255) / 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid);
    return cudaGetLastError();
}

// load_uvstress_from_tensor (mpm_solver_warp.py:253-266) in one pass: u, v
// and stress of user particle `id` into its record (quads 2, 3, 5-7; the C
// words sharing quads 3 and 5 are kept)
__global__ void load_uvstress_kernel(PState st, int n, const int *__restrict__ inv, const float *__restrict__ u,
                                     const float *__restrict__ v, const float *__restrict__ tau) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int i = inv[id];
    const float4 q3 = ldrec(st, i, 3), q5 = ldrec(st, i, 5);
    const float *pu = u + (int64_t)id * 3, *pv = v + (int64_t)id * 3, *pt = tau + (int64_t)id * 9;
    strec(st, i, 2, make_float4(pu[0], pu[1], pu[2], pv[0]));
    strec(st, i, 3, make_float4(pv[1], pv[2], q3.z, q3.w));
    strec(st, i, 5, make_float4(q5.x, q5.y, q5.z, pt[0]));
    strec(st, i, 6, make_float4(pt[1], pt[2], pt[3], pt[4]));
    strec(st, i, 7, make_float4(pt[5], pt[6], pt[7], pt[8]));
}

// export_uvFstress_from_warp (mpm_solver_warp.py:305-310) in one pass: u, v,
// F - I (:16-19) and stress of user particle `id`
__global__ void export_uvFstress_kernel(PState st, int n, const int *__restrict__ inv, float *__restrict__ u,
                                        float *__restrict__ v, float *__restrict__ fd, float *__restrict__ tau) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int i = inv[id];
    const float4 q1 = ldrec(st, i, 1), q2 = ldrec(st, i, 2), q3 = ldrec(st, i, 3), q5 = ldrec(st, i, 5),
                 q6 = ldrec(st, i, 6), q7 = ldrec(st, i, 7), q8 = ldrec(st, i, 8), q9 = ldrec(st, i, 9);
    float *pu = u + (int64_t)id * 3, *pv = v + (int64_t)id * 3, *pf = fd + (int64_t)id * 9,
          *pt = tau + (int64_t)id * 9;
    pu[0] = q2.x; pu[1] = q2.y; pu[2] = q2.z;
    pv[0] = q2.w; pv[1] = q3.x; pv[2] = q3.y;
    pf[0] = q8.x - 1.0f; pf[1] = q8.y; pf[2] = q8.z; pf[3] = q8.w; pf[4] = q9.x - 1.0f;
    pf[5] = q9.y; pf[6] = q9.z; pf[7] = q9.w; pf[8] = q1.w - 1.0f;
    pt[0] = q5.w; pt[1] = q6.x; pt[2] = q6.y; pt[3] = q6.z; pt[4] = q6.w;
    pt[5] = q7.x; pt[6] = q7.y; pt[7] = q7.z; pt[8] = q7.w;
}

// save_data_at_frame's arrays (mpm_solver_warp.py:339-404) in one pass, in the
// frame file's own transposed layout: row c of an array holds component c of
// every particle in user order, so each store instruction of a warp writes 32
// consecutive floats.  out: x_initial (3, n) | q = u (3, n) | masses (1, n) |
// f_tensor = F - I (9, n) | stress components 0,1,2,4,5,8 (6, n) | v (3, n) |
// C (9, n).
__global__ void export_frame_kernel(PState st, int n, const int *__restrict__ inv, float *__restrict__ out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int i = inv[id];
    const float4 q0 = ldrec(st, i, 0), q1 = ldrec(st, i, 1), q2 = ldrec(st, i, 2), q3 = ldrec(st, i, 3),
                 q4 = ldrec(st, i, 4), q5 = ldrec(st, i, 5), q6 = ldrec(st, i, 6), q7 = ldrec(st, i, 7),
                 q8 = ldrec(st, i, 8), q9 = ldrec(st, i, 9);
    const int64_t N = n;
    float *o = out + id;
    const float rows[34] = {
        q0.x, q0.y, q0.z,                                                                    // x
        q2.x, q2.y, q2.z,                                                                    // q
        q0.w,                                                                                // masses
        q8.x - 1.0f, q8.y, q8.z, q8.w, q9.x - 1.0f, q9.y, q9.z, q9.w, q1.w - 1.0f,           // f_tensor
        q5.w, q6.x, q6.y, q6.w, q7.x, q7.w,                                                  // stress
        q2.w, q3.x, q3.y,                                                                    // v
        q3.z, q3.w, q4.x, q4.y, q4.z, q4.w, q5.x, q5.y, q5.z};                               // C
#pragma unroll
    for (int r = 0; r < 34; ++r) o[r * N] = rows[r];
}

// dense (n,n,n) grid_m / grid_v_in from the accumulator (valid after p2g)
__global__ void export_acc_kernel(const float4 *__restrict__ acc, int64_t block_begin, int nb, int n,
                                  float *gm, float *gvin) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)n * n * n;
    if (g >= nn) return;
    int iz = (int)(g % n), iy = (int)((g / n) % n), ix = (int)(g / ((int64_t)n * n));
    float4 a = acc[node_addr(block_begin, nb, ix, iy, iz)];
    if (gm) gm[g] = a.w;
    if (gvin) { gvin[3 * g] = a.x; gvin[3 * g + 1] = a.y; gvin[3 * g + 2] = a.z; }
}

// grid_v_out of the active blocks that belong to one scene (rest stays 0)
__global__ void export_vout_kernel(const float4 *__restrict__ gridv, const int *__restrict__ list,
                                   const int *__restrict__ n_active, MpmScene S, float *gvout) {
    const int na = *n_active;
    const int nb = S.n_blocks_axis, n = S.n_grid;
    const int64_t nblk = (int64_t)nb * nb * nb;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (int64_t)na * kBlockNodes;
         j += (int64_t)gridDim.x * blockDim.x) {
        int gb = list[j >> 6];
        int64_t lb = gb - S.block_begin;
        if (lb < 0 || lb >= nblk) continue;
        int l = (int)(j & 63);
        int bz = (int)(lb % nb), by = (int)((lb / nb) % nb), bx = (int)(lb / ((int64_t)nb * nb));
        int ix = 4 * bx + (l >> 4), iy = 4 * by + ((l >> 2) & 3), iz = 4 * bz + (l & 3);
        if (ix >= n || iy >= n || iz >= n) continue;
        float4 v = gridv[(int64_t)gb * kBlockNodes + l];
        int64_t g = ((int64_t)ix * n + iy) * n + iz;
        gvout[3 * g] = v.x; gvout[3 * g + 1] = v.y; gvout[3 * g + 2] = v.z;
    }
}

__global__ void svd_kernel(const float *__restrict__ A, float *U, float *s, float *V, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = A[9 * i + k];
    Svd d;
    svd3(a, d);
#pragma unroll
    for (int k = 0; k < 9; ++k) { U[9 * i + k] = d.U[k]; V[9 * i + k] = d.V[k]; }
#pragma unroll
    for (int k = 0; k < 3; ++k) s[3 * i + k] = d.s[k];
}

__global__ void return_map_kernel(MpmScene S, const float *__restrict__ Ft, float *yld, float *F,
                                  float *tau, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a[9], fo[9], t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = Ft[9 * i + k];
    float y = yld ? yld[i] : 0.0f;
    return_map_stress(S, a, y, fo, t);
    if (yld) yld[i] = y;
#pragma unroll
    for (int k = 0; k < 9; ++k) { F[9 * i + k] = fo[k]; tau[9 * i + k] = t[k]; }
}

static inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_init_state(const Ctx &cx, const PState &other) {
    if (cx.n == 0) return cudaSuccess;
    init_state_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, other, cx.n);
    return cudaGetLastError();
}

cudaError_t launch_load(const Ctx &cx, int field, const float *src) {
    if (cx.n == 0) return cudaSuccess;
    load_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, field,
                                                               field_components(field), src);
    return cudaGetLastError();
}

cudaError_t launch_export(const Ctx &cx, int field, float *dst) {
    if (cx.n == 0) return cudaSuccess;
    export_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, field,
                                                                 field_components(field), dst);
    return cudaGetLastError();
}

cudaError_t launch_load_uvstress(const Ctx &cx, const float *u, const float *v, const float *tau) {
    if (cx.n == 0) return cudaSuccess;
    slot_of_uid_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid);
    load_uvstress_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid, u, v, tau);
    return cudaGetLastError();
}

cudaError_t launch_export_uvFstress(const Ctx &cx, float *u, float *v, float *fd, float *tau) {
    if (cx.n == 0) return cudaSuccess;
    slot_of_uid_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid);
    export_uvFstress_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid, u, v,
                                                                           fd, tau);
    return cudaGetLastError();
}

cudaError_t launch_export_frame(const Ctx &cx, float *out) {
    if (cx.n == 0) return cudaSuccess;
    slot_of_uid_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid);
    export_frame_kernel<<<blocks_for(cx.n, 256), 256, 0, cx.stream>>>(cx.st, cx.n, cx.ws.slot_of_uid, out);
    return cudaGetLastError();
}

cudaError_t launch_export_grid(const Ctx &cx, const MpmScene &S, int scene_index, float *gm,
                               float *gvin, float *gvout) {
    (void)scene_index;
    const int64_t nn = (int64_t)S.n_grid * S.n_grid * S.n_grid;
    if (gm || gvin)
        export_acc_kernel<<<blocks_for(nn, 256), 256, 0, cx.stream>>>(
            cx.ws.grid_acc, S.block_begin, S.n_blocks_axis, S.n_grid, gm, gvin);
    if (gvout) {
        cudaError_t e = cudaMemsetAsync(gvout, 0, (size_t)nn * 3 * sizeof(float), cx.stream);
        if (e != cudaSuccess) return e;
        export_vout_kernel<<<cx.num_sms * 4, 256, 0, cx.stream>>>(cx.ws.grid_v, cx.ws.active_list,
                                                                   cx.ws.n_active, S, gvout);
    }
    return cudaGetLastError();
}

cudaError_t launch_svd3(const float *A, float *U, float *s, float *V, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    svd_kernel<<<blocks_for(n, 128), 128, 0, st>>>(A, U, s, V, n);
    return cudaGetLastError();
}

cudaError_t launch_return_map(const MpmScene &scene, const float *Ft, float *yld, float *F,
                              float *tau, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    return_map_kernel<<<blocks_for(n, 128), 128, 0, st>>>(scene, Ft, yld, F, tau, n);
    return cudaGetLastError();
}

}  // namespace mpm
