// Internal launch interface between the C-ABI layer (mpm_api.cu) and the
// kernel translation units.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include "mpm_device.cuh"

namespace mpm {

struct Ctx {
    const MpmScene *scenes;  // device scene table
    int n_scenes;
    PState st;               // live state buffer
    PState st2;              // the other state buffer (G2P writes the sorted records there)
    Ws ws;
    int n;                   // particles
    int *status;
    cudaStream_t stream;
    int num_sms;
    int64_t total_blocks;
};

// sort stage (mpm_sort.cu)
cudaError_t launch_keys(const Ctx &cx);
cudaError_t launch_sort(const Ctx &cx);

// transfer stages (mpm_substep.cu)
// partials / blk_index non-null: the ordered mode (see launch_p2g_ordered)
cudaError_t launch_p2g(const Ctx &cx, float dt, float4 *partials = nullptr, int *blk_index = nullptr);
// P2G whose sums do not depend on the order in which warps run (mpm_ordered.cu):
// each cell's particles in uid order, per-block tiles to `scratch`, summed per
// node in a fixed order into grid_acc.  scratch: ordered_scratch_bytes
int64_t ordered_scratch_bytes(int64_t total_blocks);
cudaError_t launch_p2g_ordered(const Ctx &cx, float dt, void *scratch);
cudaError_t launch_grid(const Ctx &cx, float time, float dt);
// defer_stress: store F_trial as F and skip the return map (surrogate stage follows)
cudaError_t launch_g2p(const Ctx &cx, float dt, bool defer_stress = false);

// surrogate stress stage (mpm_surrogate.cu): network stress with exact-invariant
// correction and gating on the records G2P wrote into cx.st2; fallbacks to the
// SVD return map.  stats: 8 device ints (see mpm_g2p_surrogate).
cudaError_t launch_surrogate(const Ctx &cx, const void *mlp_params, const MpmSurrogateConfig &cfg,
                             int2 *fallback, int *stats);
cudaError_t launch_surrogate_apply(const MpmScene &scene, const void *mlp_params, const MpmSurrogateConfig &cfg,
                                   const float *F, float *Fo, float *tau, int *codes, int64_t n, int num_sms,
                                   cudaStream_t stream);
// reverse mode of one substep (mpm_adjoint.cu); see mpm_adjoint_substep
cudaError_t launch_adjoint(const Ctx &cx, const float *adj_out, float *adj_in, float4 *grid_adj, double *thb,
                           float time, float dt);
cudaError_t launch_return_map_vjp(const MpmScene &scene, const float *Ft, const float *Fb, const float *Tb,
                                  float *Ftb, double *thb, int64_t n, cudaStream_t st);
// saved grids for the reverse pass (mpm_checkpoint.cu)
int64_t substep_grid_bytes(int64_t total_blocks, int64_t n, int64_t max_chunks);
int64_t substep_workspace_bytes(const MpmPlan &p);  // the substep's prefix of the workspace
cudaError_t launch_save_grid(const Ctx &cx, void *dst);
cudaError_t launch_load_grid(const Ctx &cx, const void *src);
cudaError_t launch_clear_grid(const Ctx &cx);
// tensor-core (tcgen05) network forward (mpm_mlp_tc.cu)
int64_t mlp_tc_smem_bytes();
cudaError_t launch_mlp_forward_tc(const void *params, const float *x, float *y, const float *target, void *zsave,
                                  void *dy, float *loss, float grad_scale, int64_t n, int *err, int num_sms,
                                  cudaStream_t stream);
// tcgen05 network backward (mpm_mlp_bw_tc.cu)
int64_t mlp_bw_tc_smem_bytes();
cudaError_t launch_mlp_backward_tc(const void *params, const float *x, const void *zsave, const void *dy,
                                   float *grad, int64_t n, int *err, int num_sms, cudaStream_t stream);
cudaError_t launch_features(const MpmScene &scene, const float *F, const float *stress, float *x, float *y,
                            int64_t n, cudaStream_t stream);

// data movement and element kernels (mpm_io.cu)
cudaError_t launch_init_state(const Ctx &cx, const PState &other);
cudaError_t launch_load(const Ctx &cx, int field, const float *src);
cudaError_t launch_export(const Ctx &cx, int field, float *dst);
cudaError_t launch_advance_colliders(MpmScene *scenes, int n_scenes, float time, float dt, cudaStream_t stream);
cudaError_t launch_load_uvstress(const Ctx &cx, const float *u, const float *v, const float *tau);
cudaError_t launch_export_uvFstress(const Ctx &cx, float *u, float *v, float *fd, float *tau);
cudaError_t launch_export_frame(const Ctx &cx, float *out);
cudaError_t launch_export_grid(const Ctx &cx, const MpmScene &host_scene, int scene_index,
                               float *gm, float *gvin, float *gvout);
cudaError_t launch_svd3(const float *A, float *U, float *s, float *V, int64_t n, cudaStream_t st);
cudaError_t launch_return_map(const MpmScene &scene, const float *Ft, float *yld, float *F,
                              float *tau, int64_t n, cudaStream_t st);

// the reference's stress decoder (mpm_decoder.cu); see mpm_decoder_forward / mpm_decoder_stress
int64_t decoder_param_floats(const MpmStressDecoder &d);
cudaError_t launch_decoder_rows(const MpmStressDecoder &d, const float *rows, float *out, int64_t n, int num_sms,
                                cudaStream_t stream);
cudaError_t launch_decoder_stress(const Ctx &cx, const MpmStressDecoder &d, const float *label, const float *mu);

// slot_of_uid[uid] = slot of the live state (mpm_io.cu)
cudaError_t launch_slot_of_uid(const Ctx &cx);

// reduced sampled-quadrature substep (mpm_reduced.cu); see mpm_p2g2p_reduced
cudaError_t launch_p2g2p_reduced(const Ctx &cx, const MpmReducedGrid &g, float time, float dt);
cudaError_t launch_mark_grid_v(const Ctx &cx, const MpmReducedGrid &g);
cudaError_t launch_g2p_sample(const Ctx &cx, const MpmReducedGrid &g, float dt);

int field_components(int field);

// records e for mpm_last_cuda_error() (as every entry point does) and returns MPM_ERR_CUDA
int record_cuda_error(cudaError_t e);

}  // namespace mpm
