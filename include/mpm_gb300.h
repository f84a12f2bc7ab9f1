/*
 * mpm_gb300.h -- C ABI of the GB300 (sm_103a) MPM substep library
 * (libmpm_gb300.so, built from reduced_mpm_stress_training_gb300/csrc).
 *
 * Drop-in boundary for MPM_Simulator_WARP.p2g2p of
 * zeshunzong/reduced_mpm_stress_training (engine_stress/mpm_solver_warp.py).
 * The reference reaches its device code through Warp's wp.launch with the
 * by-value structs MPMModelStruct / MPMStateStruct (engine_stress/warp_utils.py:61-124);
 * these entry points replace those launches.  Every function:
 *   - takes plain pointers and sizes, no torch or Warp types;
 *   - allocates no device memory: the caller owns every buffer
 *     (sizes from mpm_plan);
 *   - enqueues work on the given CUDA stream (cudaStream_t passed as void*,
 *     NULL = legacy default stream) and does not synchronise it, except
 *     where a host pointer is read or written (noted below);
 *   - returns MPM_OK (0) or a negative MPM_ERR_* code.
 * Physics faults (particles leaving the grid, CFL violation, non-finite
 * F or stress) never trap: kernels OR a bit into the device status word
 * (MpmBuffers.status) which the caller reads when it likes.
 * State the library keeps itself: the last CUDA error text (per host
 * thread), the SM count per device, two copy lanes (a side stream and
 * events each, created by the first host-buffer transfer), the 16 MiB
 * device array of mpm_p2g2p_noalloc, and a once-per-device shared-memory
 * opt-in of the decoder kernels.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPM_ABI_VERSION 3
#define MPM_MAX_COLLIDERS 8

/* return codes */
#define MPM_OK 0
#define MPM_ERR_ARG (-1)   /* bad argument (null pointer, size, field id)   */
#define MPM_ERR_CUDA (-2)  /* a CUDA runtime call failed (launch, memcpy)   */
#define MPM_ERR_SIZE (-3)  /* a size exceeds what the buffers were planned for */

/* device status-word bits */
#define MPM_ST_OUT_OF_DOMAIN 1 /* stencil outside [0,n-3]^3 or NaN position: particle frozen */
#define MPM_ST_CFL 2           /* |v_i| > dx/dt (mpm_solver_warp.py:188-192)          */
#define MPM_ST_NONFINITE 4     /* non-finite F or stress after the return map         */
#define MPM_ST_INTERNAL 8      /* a particle was not inside its sorted block (bug)    */
#define MPM_ST_BAD_INPUT 16    /* reduced substep: a sample index outside [0, n) or a
                                  dense grid whose n_grid is not the scene's: skipped */

/* material ids, engine_stress/mpm_solver_warp.py:90-94 */
#define MPM_JELLY 0
#define MPM_METAL 1
#define MPM_SAND 2

/* collider kinds */
#define MPM_COLLIDER_SURFACE 0 /* add_surface_collider(2), mpm_solver_warp.py:407-497      */
#define MPM_COLLIDER_BOX 1     /* add_bounding_box,           mpm_solver_warp.py:499-525    */
#define MPM_COLLIDER_VPLANE 2  /* set_velocity_on_infinite_plane, mpm_solver_warp.py:527-568 */
#define MPM_COLLIDER_CIRCLE 3  /* set_column_moving_as_circle,    mpm_solver_warp.py:570-607 */
#define MPM_COLLIDER_DISK 4    /* set_rotation_on_disk,           mpm_solver_warp.py:609-665 */
#define MPM_COLLIDER_CUBE 5    /* set_velocity_on_cube,           mpm_solver_warp.py:667-695 */
#define MPM_COLLIDER_SPHERE 6  /* add_sphere_leader,              mpm_solver_warp.py:697-720 */

/* Dirichlet_collider (engine_stress/warp_utils.py:126-151).  normal, x_unit
 * and y_unit must be unit length.  A collider is active while
 * start_time <= time < end_time; the moving kinds (VPLANE, CIRCLE, CUBE,
 * SPHERE) advance `point` on the device after each active substep's grid
 * update, as the reference's modify_bc callbacks do on the host. */
typedef struct MpmCollider {
    int32_t kind;         /* MPM_COLLIDER_*                                      */
    int32_t surface_type; /* SURFACE: 0 sticky, 1 slip, 2 separate; all three
                             zero the node velocity, as the reference does (:449) */
    float point[3];
    float normal[3];
    float friction;
    float start_time; /* active while start_time <= time < end_time */
    float end_time;
    int32_t reset;        /* VPLANE, DISK, CUBE: zero velocities shortly after end_time */
    float velocity[3];    /* VPLANE, CUBE, SPHERE: velocity given to the covered nodes */
    float threshold;      /* VPLANE: half-thickness of the slab |(x - point).normal|  */
    float radius;         /* CIRCLE, DISK, SPHERE                                */
    float width;          /* DISK: half-thickness; CUBE: half-width               */
    float height;         /* CIRCLE: half-height of the column                    */
    float v_scale;        /* CIRCLE: speed; DISK: angular speed                   */
    float x_unit[3];      /* DISK: in-plane axes                                  */
    float y_unit[3];
    float R;              /* CIRCLE: orbit radius                                 */
    float pad0;
} MpmCollider; /* 112 bytes */

/* One scene: MPMModelStruct (engine_stress/warp_utils.py:61-81) plus its
 * particle range and grid-block range.  A plain simulator is one scene; the
 * batched form concatenates many.  Fields marked (plan) are filled in by
 * mpm_plan. */
typedef struct MpmScene {
    int32_t n_grid;    /* nodes per axis; grid covers [0, n_grid*dx)^3        */
    int32_t material;  /* MPM_JELLY / MPM_METAL / MPM_SAND                   */
    int32_t hardening; /* von Mises linear hardening on (1) / off (0)        */
    int32_t n_colliders;
    float dx, inv_dx;  /* grid_lim/n_grid and n_grid/grid_lim (:37)          */
    float mu, lam;     /* Lame parameters                                    */
    float alpha;       /* Drucker-Prager alpha from the friction angle (:113-116) */
    float xi;          /* hardening slope                                    */
    float gravity[3];  /* reference: (0, -g, 0) (mpm_utils.py:236)           */
    int32_t n_blocks_axis;  /* (plan) ceil(n_grid/4)                          */
    int64_t particle_begin; /* first particle (user order) of this scene     */
    int64_t particle_count;
    int64_t block_begin;    /* (plan) first global 4x4x4 grid-block id        */
    MpmCollider colliders[MPM_MAX_COLLIDERS];
} MpmScene; /* 976 bytes */

/* Sizes computed by mpm_plan. */
typedef struct MpmPlan {
    int64_t n_particles;     /* total over all scenes                         */
    int64_t particle_stride; /* padded per-field stride of the state (floats) */
    int64_t total_blocks;    /* 4x4x4 grid blocks over all scenes             */
    int64_t max_chunks;      /* upper bound of the per-substep work list      */
    int64_t state_bytes;     /* bytes of ONE particle-state buffer             */
    int64_t workspace_bytes; /* bytes of the workspace                         */
    int32_t chunk_size;      /* particles per work chunk (32..256, power of 2) */
    int32_t n_scenes;
} MpmPlan; /* 56 bytes */

/* Caller-owned device buffers plus the host-side control the library keeps
 * between calls.  All pointers are device pointers (256-byte aligned). */
typedef struct MpmBuffers {
    void *state[2];   /* two particle-state buffers, plan.state_bytes each      */
    void *workspace;  /* plan.workspace_bytes                                  */
    void *scenes;     /* device copy of the MpmScene table (mpm_upload_scenes)  */
    int32_t *status;  /* one device int32, MPM_ST_* bits, OR-accumulated        */
    MpmPlan plan;
    int32_t cur;             /* index of the live state buffer; every substep
                                flips it (G2P writes the updated records, sorted
                                by cell, into the other buffer)                 */
    int32_t keys_valid;      /* 0 after a load that moves particles             */
    int32_t collider_flags;  /* (set by mpm_upload_scenes) MPM_CF_* of the table */
    int32_t pad0;
    int64_t substep;         /* substeps taken since mpm_init                   */
} MpmBuffers;

/* collider_flags bits */
#define MPM_CF_EXTENDED 1 /* a collider of kind VPLANE..SPHERE (no adjoint for those) */
#define MPM_CF_MOVING 2   /* a moving collider: mpm_grid_update advances its point  */

/* State fields for mpm_load / mpm_export.  Layout on the caller side is the
 * reference's: AoS, user particle order, vec3 = 3 floats, mat33 = 9 floats
 * row-major (engine_stress/warp_utils.py:5-43). */
#define MPM_FIELD_X_INITIAL 0 /* vec3  particle_x_initial                     */
#define MPM_FIELD_U 1         /* vec3  particle_u (displacement)               */
#define MPM_FIELD_V 2         /* vec3  particle_v                              */
#define MPM_FIELD_C 3         /* mat33 particle_C (APIC affine)                */
#define MPM_FIELD_F 4         /* mat33 particle_F (elastic deformation grad.)  */
#define MPM_FIELD_STRESS 5    /* mat33 particle_stress (Kirchhoff)             */
#define MPM_FIELD_MASS 6      /* float particle_mass                           */
#define MPM_FIELD_VOL 7       /* float particle_vol                            */
#define MPM_FIELD_YIELD 8     /* float yield_stress (von Mises)                */
#define MPM_FIELD_X 9         /* vec3  particle_x = x_initial + u   (export only) */
#define MPM_FIELD_F_DISP 10   /* mat33 particle_F_disp = F - I      (export only) */

/* ---- layout ---------------------------------------------------------- */

/* Fill scenes[*].n_blocks_axis / block_begin and *plan for n_scenes scenes
 * whose particle ranges tile [0, n_particles).  chunk_size 0 picks the
 * default (128).  Host only.  Replaces the allocation half of
 * MPM_Simulator_WARP.initialize (engine_stress/mpm_solver_warp.py:28-87). */
int mpm_plan(MpmScene *scenes, int32_t n_scenes, int64_t n_particles, int32_t chunk_size,
             MpmPlan *plan);

/* Zero both state buffers and the workspace, set F = I and the identity
 * particle order, clear the status word.  Replaces the initial values of
 * MPM_Simulator_WARP.initialize (engine_stress/mpm_solver_warp.py:52-69). */
int mpm_init(MpmBuffers *b, void *stream);

/* Copy n_scenes host MpmScene records into b->scenes (stream-ordered; reads
 * the host table before returning).  Replaces the by-value MPMModelStruct
 * argument of every wp.launch (engine_stress/mpm_solver_warp.py:157-197) and
 * set_parameters (:89-127) / add_surface_collider (:407) / add_bounding_box (:499). */
int mpm_upload_scenes(MpmBuffers *b, const MpmScene *scenes, int32_t n_scenes, void *stream);

/* ---- particle data in the reference layout --------------------------- */

/* Load one field for all particles from src (reference layout, user order).
 * src_on_host != 0: src is host memory (pinned for asynchrony) and is copied
 * through the workspace.  Replaces load_x_initial_from_tensor (:229-230),
 * load_mass_from_tensor (:231-232), load_uvF_from_tensor (:234-245),
 * load_C_from_tensor (:247-251), load_uvstress_from_tensor (:253-266) and the
 * set_value kernels of set_parameters (:108-124). */
int mpm_load(MpmBuffers *b, int32_t field, const float *src, int32_t src_on_host, void *stream);

/* Export one field for all particles to dst (reference layout, user order).
 * dst_on_host != 0: dst is host memory; the call then waits for the copy.
 * Replaces export_uvFstress_from_warp (:305-310) and the wp.array reads of
 * mpm_state.particle_* (e.g. save_data_at_frame :351-384). */
int mpm_export(MpmBuffers *b, int32_t field, float *dst, int32_t dst_on_host, void *stream);
/* load_uvstress_from_tensor (engine_stress/mpm_solver_warp.py:253-266) in one
 * pass: u (n,3), v (n,3), stress (n,9), user order, host (pinned) or device.
 * From the host the copy runs on a library side stream that waits only for
 * the previous mpm_load_uvstress to have consumed its staging, so it may
 * overlap earlier work on `stream` and an mpm_export_uvFstress copy in
 * flight; the load itself is ordered on `stream`.  The host arrays must stay
 * unchanged until `stream` reaches the load. */
int mpm_load_uvstress(MpmBuffers *b, const float *u, const float *v, const float *stress, int32_t src_on_host,
                      void *stream);
/* export_uvFstress_from_warp (engine_stress/mpm_solver_warp.py:305-310) in one
 * pass: u (n,3), v (n,3), F_disp = F - I (n,9), stress (n,9) in user order.
 * dst_on_host 0: device arrays, ordered on `stream`.  1: host (pinned)
 * arrays, the call returns after the copies landed.  2: host arrays, the
 * copies run on a library side stream after the export kernel and may
 * overlap later work on `stream`; read the arrays after mpm_sync_transfers()
 * or a device synchronize. */
int mpm_export_uvFstress(MpmBuffers *b, float *u, float *v, float *F_disp, float *stress, int32_t dst_on_host,
                         void *stream);
/* Waits (host) for every host copy mpm_load_uvstress / mpm_export_uvFstress
 * left in flight on the current device. */
int mpm_sync_transfers(void);

/* The arrays of one frame file (save_data_at_frame, mpm_solver_warp.py:339-404)
 * in its transposed layout, one pass: out (34 * n floats, device) holds
 * x (3, n) = x_initial, q (3, n) = u, masses (1, n), f_tensor (9, n) = F - I
 * row-major, stress (6, n) = components 0, 1, 2, 4, 5, 8 of the row-major
 * stress, v (3, n), C (9, n) -- row c of each array is component c of every
 * particle in user order. */
#define MPM_FRAME_FLOATS_PER_PARTICLE 34
int mpm_export_frame(MpmBuffers *b, float *out, void *stream);

/* ---- the substep ----------------------------------------------------- */

/* One full substep for every scene: x = x0 + u, cell-block sort, APIC P2G
 * with the stored stress, grid normalisation + gravity + colliders, G2P with
 * APIC C, F update, return mapping and Kirchhoff stress, u = x - x0.
 * `time` gates the colliders.  Replaces MPM_Simulator_WARP.p2g2p
 * (engine_stress/mpm_solver_warp.py:156-203), i.e. the launches of
 * update_x_from_u, zero_grid, p2g_apic_stress_given,
 * grid_normalization_and_gravity, the collider kernels, g2p_apic_and_stress,
 * update_u_from_x and update_F_disp_from_F (engine_stress/mpm_utils.py). */
int mpm_p2g2p(MpmBuffers *b, float time, float dt, void *stream);

/* The substep's stages, for callers that interleave their own work and for
 * per-stage checks.  mpm_p2g2p == sort, p2g, grid_update, g2p. */
int mpm_sort(MpmBuffers *b, void *stream); /* block keys, counting sort, re-sort */
int mpm_p2g(MpmBuffers *b, float dt, void *stream); /* mpm_utils.py:190-227 */
int mpm_grid_update(MpmBuffers *b, float time, float dt, void *stream); /* :229-237 + colliders */
int mpm_g2p(MpmBuffers *b, float dt, void *stream); /* mpm_utils.py:241-306, :4-19 */

/* No counterpart in the reference (its P2G, engine_stress/mpm_utils.py:190-227,
 * adds with float atomics in whatever order threads run, as mpm_p2g does).
 * The P2G stage with sums that do not depend on the order in which warps
 * run: each cell's particles are taken in uid order and the per-block node
 * tiles are summed per node in a fixed order, so the whole substep (with
 * mpm_sort, mpm_grid_update, mpm_g2p) is a deterministic function of its
 * inputs -- what finite-difference checks of gradients need.  Same results
 * as mpm_p2g up to float32 rounding.  `scratch`: caller-owned device memory
 * of mpm_p2g_ordered_bytes(&plan) bytes (a 6x6x6 float4 tile per grid block
 * plus a block index).  mpm_p2g2p_ordered is the substep with it. */
int64_t mpm_p2g_ordered_bytes(const MpmPlan *plan);
int mpm_p2g_ordered(MpmBuffers *b, void *scratch, float dt, void *stream);
int mpm_p2g2p_ordered(MpmBuffers *b, void *scratch, float time, float dt, void *stream);

/* Dense (n,n,n) C-order copy of one scene's grid after the last stage that
 * wrote it: grid_m and grid_v_in (momentum) are valid between mpm_p2g and
 * mpm_grid_update, grid_v_out after mpm_grid_update.  Untouched nodes read 0,
 * as after the reference's zero_grid.  Any pointer may be NULL.  Replaces
 * reads of mpm_state.grid_m / grid_v_in / grid_v_out (warp_utils.py:109-112). */
int mpm_export_grid(MpmBuffers *b, int32_t scene, float *grid_m, float *grid_v_in,
                    float *grid_v_out, void *stream);

/* No counterpart in the reference (its Warp launches always use arrays the
 * simulator allocated).  The substep of mpm_p2g2p for callers that cannot
 * allocate device memory -- e.g. a host framework that has reserved nearly all
 * device memory for its own pool, or code that runs where cudaMalloc is not
 * allowed: b->workspace is ignored (may be NULL) and the scratch lives in one
 * library-owned 16 MiB device array (held by every GPU that loads the
 * library).  Returns MPM_ERR_SIZE if the substep's part of the workspace
 * (everything in b->plan.workspace_bytes but the host-transfer staging, which
 * this call never uses) exceeds 16 MiB: a 64^3 grid fits with up to about a
 * million particles, a 128^3 grid does not.  All calls share that array: each
 * call clears it and re-sorts from the particle positions, and calls that
 * overlap on the GPU race.  The first call on a device looks up the array's
 * address (cudaGetSymbolAddress); make it before any stream capture.  Never
 * allocates. */
int mpm_p2g2p_noalloc(MpmBuffers *b, float time, float dt, void *stream);

/* ---- reduced sampled-quadrature substep ------------------------------
 * MPM_Simulator_WARP.p2g2p_reduced (engine_stress/mpm_solver_warp.py:214-227)
 * and its kernels (engine_stress/mpm_utils.py:318-471): only particles whose
 * stencil base cell lies within two cells of a sample point's base cell
 * scatter, with a stress recomputed from F_disp, into a dense grid that is
 * the product of the call.  Single-scene plans only (MPM_ERR_ARG otherwise).
 * Every array is the caller's device memory in the reference's own layout
 * (warp_utils.py:84-124): particle arrays in the user's particle order,
 * grids dense (n, n, n) C-order, flat index (ix * n + iy) * n + iz. */
typedef struct MpmReducedGrid {
    const int32_t *sample_index; /* n_samples user particle indices:
                                    sample_particle_index_short             */
    int64_t n_samples;
    float *f_disp;               /* (n, 9) particle_F_disp: read by the P2G,
                                    written for the samples by mpm_g2p_sample */
    const float *density;        /* (n) particle_density                    */
    void *grid_acc;              /* n^3 x 16 B scratch (momentum, mass)     */
    float *grid_m;               /* n^3       written by mpm_p2g2p_reduced  */
    float *grid_v_in;            /* n^3 x 3   momentum, same                */
    float *grid_v_out;           /* n^3 x 3   velocity after the colliders  */
    int32_t *neighboring_cells;        /* n^3 marks of the P2G (:318-335)    */
    int32_t *neighboring_cells_grid_v; /* n^3 marks for the gather (:338-351) */
    int32_t n_grid;              /* n: the scene's n_grid, at most 1024     */
    int32_t pad0;
} MpmReducedGrid; /* 88 bytes */

/* p2g2p_reduced (mpm_solver_warp.py:214-227): zero the grids and both mark
 * arrays; mark the 5^3 cells around each sample point's base cell
 * (update_neighboring_cells, mpm_utils.py:318-335); every particle whose
 * base cell is marked sets F = F_disp + I (written to its state), takes the
 * FCR (jelly, metal) or Drucker-Prager (sand) Kirchhoff stress of that F and
 * scatters momentum w m v (no affine term), mass and the force
 * -dt (m / density) stress grad w (p2g_sample_all, :353-402); marked nodes
 * with m > 1e-10 get v_out = v_in / m + dt g, the others 0
 * (grid_normalization_and_gravity_sample_all, :405-413); then the scene's
 * colliders sweep every node and moving ones advance.  Particles are not
 * moved; the caller advances time by dt, as for mpm_p2g2p.  A marked
 * particle whose stencil would leave the grid, or any particle whose base
 * cell is outside it (the reference indexes out of bounds there), is skipped
 * and sets MPM_ST_OUT_OF_DOMAIN. */
int mpm_p2g2p_reduced(MpmBuffers *b, const MpmReducedGrid *g, float time, float dt, void *stream);

/* MPM_Simulator_WARP.experiment_for_C (mpm_solver_warp.py:207-209): mark
 * neighboring_cells_grid_v over offsets -2..4 of each sample point's base
 * cell (update_neighboring_cells_for_grid_v, mpm_utils.py:338-351).  Adds
 * marks: the array is cleared only by mpm_p2g2p_reduced, as zero_grid does. */
int mpm_mark_neighboring_cells_grid_v(MpmBuffers *b, const MpmReducedGrid *g, void *stream);

/* The sample points' gather, g2p_sample (mpm_utils.py:415-471; defined but
 * never launched by the reference): for sample s, particle p =
 * sample_index[s] takes v = sum w v_out, x += dt v, F_trial = (I + dt grad v) F,
 * F = return map(F_trial), u = x - x_initial and F_disp = F - I (written to
 * g->f_disp).  C and the stress are not updated.  As in the reference, the
 * von Mises return map reads (and, with hardening, updates) yield_stress[s],
 * the sample's position in the list, not yield_stress[p] (:464).  Duplicate
 * indices race, as they do there. */
int mpm_g2p_sample(MpmBuffers *b, const MpmReducedGrid *g, float dt, void *stream);

/* ---- the reference's stress decoder in the loop ------------------------
 * NetDec (offline_training_xhat_and_stress_and_mu/CROMnet_secondary.py:203-301,
 * with Prepare :487-525, Activation :447-463 and invStandardizeQ :465-477):
 * rows (label, x, mu) -> Prepare(x) -> 5 x [Linear(hidden), activation] ->
 * Linear(6) -> mean_q + q * std_q, the six stress components
 * [xx, xy, xz, yy, yz, zz] (mpm_solver_warp.py:383).  FP32. */
typedef struct MpmStressDecoder {
    const float *params; /* device, packed float32, PyTorch [out, in] weights:
                            dec0.weight (hidden x in), dec0.bias (hidden),
                            dec1..dec4 weights (hidden x hidden each), their biases
                            (hidden each), enc.weight (6 x hidden), enc.bias (6),
                            prepare (6: min_x, max_x with SIREN, else mean_x, std_x),
                            mean_q (6), std_q (6); in = label_dim + 3 + mu_dim      */
    int32_t label_dim;   /* lbllength, 0..64                                       */
    int32_t mu_dim;      /* 0..4 (the reference's data: 1, the friction angle)     */
    int32_t hidden;      /* i_dim * scale_mlp, 1..64 (the reference's default: 30)  */
    int32_t siren;       /* 1: sin(omega_0 x) and clip-to-[-1, 1]; 0: ELU, standardise */
    float omega_0;
    int32_t pad0;
} MpmStressDecoder; /* 32 bytes */

/* Number of floats of the packed parameter blob (negative: bad dimensions). */
int64_t mpm_decoder_param_count(const MpmStressDecoder *d);

/* NetDec.forward (CROMnet_secondary.py:288-291) on n device rows of
 * label_dim + 3 + mu_dim floats -> out (n, 6). */
int mpm_decoder_forward(const MpmStressDecoder *d, const float *rows, float *out, int64_t n, void *stream);

/* The decoder as the stress source of the next substep (the reduced-order loop
 * feeds it through load_uvstress_from_tensor, mpm_solver_warp.py:253-266):
 * every particle's row is (label, its x_initial, its mu row), label one
 * frame's label_dim floats and mu (n, mu_dim) in user order (NULL when
 * mu_dim = 0); the decoded components are written as the symmetric stress
 * [q0 q1 q2; q1 q3 q4; q2 q4 q5] of the particle, read by the next mpm_p2g2p. */
int mpm_decoder_stress(MpmBuffers *b, const MpmStressDecoder *d, const float *label, const float *mu,
                       void *stream);

/* ---- element kernels on plain arrays --------------------------------- */

/* Batched 3x3 SVD, A (n,9) row-major -> U (n,9), s (n,3), V (n,9):
 * U, V rotations, |s| descending, sign(det A) on s[2].  Replaces wp.svd3
 * (called at engine_stress/mpm_utils.py:64, :92, :297). */
int mpm_svd3(const float *A, float *U, float *s, float *V, int64_t n, void *stream);

/* Batched return mapping + Kirchhoff stress of one scene's material:
 * F_trial (n,9) -> F (n,9), stress (n,9); yield (n) read and, with
 * hardening, updated (may be NULL unless the material is metal).
 * Replaces von_mises_return_mapping / sand_return_mapping and the stress
 * functions (engine_stress/mpm_utils.py:29-112, :284-306). */
int mpm_return_map(const MpmScene *scene, const float *F_trial, float *yield, float *F,
                   float *stress, int64_t n, void *stream);

/* ---- stress-surrogate network (12 -> 128 -> 128 -> 128 -> 6, SiLU) ---
 * No counterpart in the reference's solver; the nearest relative is the
 * stress decoder CROMnet_secondary.NetDec (CROMnet_secondary.py:203-301),
 * whose 6-component output is stored as [xx, xy, xz, yy, yz, zz]
 * (engine_stress/mpm_solver_warp.py:383).  BF16 weights and activations,
 * FP32 accumulation on the tensor cores.  The parameter blob (device,
 * mpm_mlp_param_bytes() bytes) holds bf16 weights W1 [128][16] (inputs
 * 12..15 zero), W2, W3 [128][128], W4 [16][128] (outputs 6..15 zero),
 * then fp32 biases b1, b2, b3 [128], b4 [16].  Gradients and the Adam
 * master copy use the same order in fp32: MPM_MLP_PARAMS floats. */
#define MPM_MLP_IN 12
#define MPM_MLP_OUT 6
#define MPM_MLP_HIDDEN 128
#define MPM_MLP_PARAMS 37264 /* 36864 weights + 400 biases */
int64_t mpm_mlp_param_bytes(void);

/* y (n,6) = net(x (n,12)).  With target (n,6) != NULL also writes the
 * loss gradient dy (n,16 bf16) = grad_scale * (y - target), the
 * pre-activations zsave (3,n,128 bf16) for the backward pass, and adds
 * the summed squared error to *loss (device float).  y may be NULL. */
int mpm_mlp_forward(const void *params, const float *x, float *y, const float *target, void *zsave,
                    void *dy, float *loss, float grad_scale, int64_t n, void *stream);
/* The same forward on the tcgen05 tensor cores (accumulators in tensor
 * memory, one 128-row tile per CTA step).  err: one device int32 the
 * kernel ORs 1 into if a tensor-core completion wait ran out (results then
 * incomplete); the caller zeroes it. */
int mpm_mlp_forward_tc(const void *params, const float *x, float *y, const float *target, void *zsave,
                       void *dy, float *loss, float grad_scale, int64_t n, int32_t *err, void *stream);
/* Adds the parameter gradient of the forward's loss into grad (fp32,
 * MPM_MLP_PARAMS).  work: 2*n*128 bf16 scratch. */
int mpm_mlp_backward(const void *params, const float *x, const void *zsave, const void *dy, void *work,
                     float *grad, int64_t n, void *stream);
/* The same backward on the tcgen05 tensor cores: one persistent CTA per SM
 * holds the four weight gradients in tensor memory over all of its 128-row
 * tiles and adds them, with the bias sums, into grad once at the end (no
 * scratch).  err: one device int32 the kernel ORs 1 into if a tensor-core
 * completion wait ran out (grad then incomplete); the caller zeroes it. */
int mpm_mlp_backward_tc(const void *params, const float *x, const void *zsave, const void *dy, float *grad,
                        int64_t n, int32_t *err, void *stream);
/* One Adam step (torch.optim.Adam semantics, step >= 1) on the fp32
 * master parameters; rewrites the bf16/fp32 blob params from them. */
int mpm_mlp_adam(float *master, float *m, float *v, const float *grad, void *params, float lr,
                 float beta1, float beta2, float eps, int32_t step, void *stream);

/* ---- surrogate stress step ------------------------------------------
 * A substep whose Drucker-Prager return map + Kirchhoff stress
 * (engine_stress/mpm_utils.py:45-52, :87-112, called from
 * g2p_apic_and_stress :284-306) comes from the network instead of the SVD.
 * Network input (12): the 9 entries of Bhat = (F F^T - I) / rho with
 * rho = ||F F^T - I||_F, then (log10 rho + 2.5) / 1.5, (nu - 0.3) / 0.1 and
 * (friction angle in degrees - 30) / 10, nu and the angle recovered from
 * the scene's lam, mu and alpha.  Output (6): tau / (mu rho) as
 * [xx, xy, xz, yy, yz, zz].  The network's stress is corrected to the exact
 * mean stress and deviatoric norm (closed-form eigenvalues of F F^T, no
 * SVD); a particle falls back to the SVD return map when it leaves the
 * training domain, reaches the cone apex, takes a plastic increment above
 * dgamma_max, or when its error estimate (max of the correction size, the
 * non-coaxiality of the deviator with F F^T and its Lode-angle mismatch)
 * exceeds tol.  Non-sand scenes always take the SVD path. */
typedef struct MpmSurrogateConfig {
    float tol;                /* gate on the relative error estimate (1e-2)          */
    float rho_min, rho_max;   /* domain of ||F F^T - I||_F                           */
    float nu_min, nu_max;     /* domain of Poisson's ratio                           */
    float phi_min, phi_max;   /* domain of the friction angle, degrees               */
    float dgamma_max;         /* larger plastic increments fall back                 */
} MpmSurrogateConfig;

/* stats[] slots (int32, device): per-particle outcome counts, accumulated
 * across calls (the caller zeroes them), and the fallback count of the
 * last call (reset by each call). */
#define MPM_SUR_ELASTIC 0    /* accepted, elastic (F = F_trial)                  */
#define MPM_SUR_PLASTIC 1    /* accepted, on the cone (F = exp(-dgamma N) F_trial) */
#define MPM_SUR_FB_DOMAIN 2  /* fallback: outside the training domain           */
#define MPM_SUR_FB_APEX 3    /* fallback: projection to the cone apex            */
#define MPM_SUR_FB_STEP 4    /* fallback: plastic increment above dgamma_max     */
#define MPM_SUR_FB_GATE 5    /* fallback: error estimate above tol               */
#define MPM_SUR_FB_MATERIAL 6 /* fallback: material other than sand             */
#define MPM_SUR_LAST_FALLBACKS 7
#define MPM_SUR_STATS 8

/* Training tuples from F_trial (n,9), the scene's material and the plain
 * return map's stress (n,9) (mpm_return_map): x (n,12) network inputs,
 * y (n,6) targets tau / (mu rho).  stress may be NULL (then y is not
 * written). */
int mpm_surrogate_features(const MpmScene *scene, const float *F, const float *stress, float *x,
                           float *y, int64_t n, void *stream);

/* The surrogate on plain arrays of one scene: F_trial (n,9) -> F (n,9),
 * stress (n,9) and the outcome code (n, MPM_SUR_*) of each row; rows the
 * gate rejects are computed by the SVD return map (as mpm_return_map). */
int mpm_surrogate_apply(const MpmScene *scene, const void *mlp_params, const MpmSurrogateConfig *cfg,
                        const float *F_trial, float *F, float *stress, int32_t *codes, int64_t n,
                        void *stream);

/* G2P with the surrogate stress stage (replaces mpm_g2p in a substep).
 * fallback: device scratch of 2 * n_particles int32.  stats: MPM_SUR_STATS
 * device int32.  mlp_params: the network blob (mpm_mlp_param_bytes). */
int mpm_g2p_surrogate(MpmBuffers *b, const void *mlp_params, const MpmSurrogateConfig *cfg,
                      void *fallback, int32_t *stats, float dt, void *stream);
/* mpm_p2g2p with mpm_g2p_surrogate in place of mpm_g2p. */
int mpm_p2g2p_surrogate(MpmBuffers *b, const void *mlp_params, const MpmSurrogateConfig *cfg,
                        void *fallback, int32_t *stats, float time, float dt, void *stream);

/* ---- reverse mode (sand) ---------------------------------------------
 * No counterpart in the reference (it has no wp.Tape or gradient code):
 * the adjoint of one substep, the latest substep first.  Call it with the
 * live state holding the state BEFORE the substep, after mpm_sort, mpm_p2g
 * and mpm_grid_update have run on that state with the substep's time and
 * dt (the grid of the substep is then in the workspace).  adj_out is the
 * adjoint of the state after the substep, adj_in receives the adjoint of
 * the state before it; both hold MPM_ADJ_WORDS floats per particle in user
 * order: x 0-2, v 3-5, C 6-14, F 15-23, stress 24-32 (matrices row-major).
 * grid_adj: device scratch of plan.total_blocks * 64 * 16 bytes.
 * theta_bar: 3 device doubles, the adjoints of (mu, lam, alpha), added to.
 * Scenes must be sand.  Particles outside the grid pass their adjoint
 * through unchanged (the forward carries them over). */
#define MPM_ADJ_WORDS 36
int mpm_adjoint_substep(MpmBuffers *b, const float *adj_out, float *adj_in, void *grid_adj,
                        double *theta_bar, float time, float dt, void *stream);

/* Saved grids for the reverse pass (checkpointing with recompute).  The
 * reverse pass of a substep and the substep's G2P read its sorted order, its
 * active-block list, its G2P chunk list and those blocks' grid momentum +
 * mass and velocity.  mpm_save_substep_grid copies them (active blocks
 * only) into a device blob of mpm_substep_grid_bytes(plan) bytes (256-byte
 * aligned) right after the substep's mpm_grid_update; mpm_load_substep_grid
 * puts them back, after which mpm_adjoint_substep -- or mpm_g2p, to rebuild
 * the state after the substep from the state before it -- needs no new
 * sort, P2G or grid update.  Loading leaves grid blocks of other substeps in
 * the accumulator: mpm_clear_grid empties it (call it before stepping
 * forward again). */
int64_t mpm_substep_grid_bytes(const MpmPlan *plan);
int mpm_save_substep_grid(MpmBuffers *b, void *dst, void *stream);
int mpm_load_substep_grid(MpmBuffers *b, const void *src, void *stream);
int mpm_clear_grid(MpmBuffers *b, void *stream);

/* Element form of the return-map adjoint (sand): F_trial (n,9) and the
 * adjoints of the returned F and of the stress (n,9 each) -> the adjoint of
 * F_trial (n,9, written) and of (mu, lam, alpha) (3 device doubles, added
 * to).  The return map it differentiates is mpm_return_map's. */
int mpm_return_map_vjp(const MpmScene *scene, const float *F_trial, const float *F_bar,
                       const float *stress_bar, float *F_trial_bar, double *theta_bar, int64_t n,
                       void *stream);

/* ---- misc ------------------------------------------------------------ */
int mpm_abi_version(void);
/* sizeof of the ABI structs, for binding checks: out[0..5] =
 * MpmCollider, MpmScene, MpmPlan, MpmBuffers, MpmReducedGrid, MpmStressDecoder. */
void mpm_struct_sizes(int64_t *out);
const char *mpm_error_string(int code);
/* Last CUDA error text seen by the library on this host thread ("" if none). */
const char *mpm_last_cuda_error(void);

#ifdef __cplusplus
}
#endif
#endif /* MPM_GB300_H */
