/* A complete C caller of the substep: a 4,096-particle sand
 * column on a 32^3 grid with a sticky floor and the box, 20 substeps, u read
 * back to the host.  tests/test_capi_cpu.py compiles and links it (no GPU
 * needed for that); run on a GPU machine it prints the column's mean
 * displacement and the status word. */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "mpm_gb300.h"

#define CHECK(x)                                                            \
    do {                                                                    \
        int r_ = (x);                                                       \
        if (r_ != MPM_OK) {                                                 \
            fprintf(stderr, "%s: %s %s\n", #x, mpm_error_string(r_), mpm_last_cuda_error()); \
            return 1;                                                       \
        }                                                                   \
    } while (0)

int main(void) {
    const int n = 4096, n_grid = 32;
    const float dt = 1e-4f, E = 2e5f, nu = 0.3f, rho = 2200.0f, phi = 30.0f;
    MpmScene scene = {0};
    scene.n_grid = n_grid;
    scene.dx = 1.0f / n_grid;
    scene.inv_dx = (float)n_grid;
    scene.material = MPM_SAND;
    scene.mu = E / 2.0f / (1.0f + nu);                            /* mpm_solver_warp.py:41 */
    scene.lam = E * nu / (1.0f + nu) / (1.0f - 2.0f * nu);        /* :42 */
    const float s = sinf(phi / 180.0f * 3.14159265f);
    scene.alpha = sqrtf(2.0f / 3.0f) * 2.0f * s / (3.0f - s);    /* :113-116 */
    scene.gravity[2] = -9.8f;
    scene.n_colliders = 2;
    scene.colliders[0].kind = MPM_COLLIDER_SURFACE;               /* sticky floor at z = 0.15 */
    scene.colliders[0].point[2] = 0.15f;
    scene.colliders[0].normal[2] = 1.0f;
    scene.colliders[0].end_time = 999.0f;
    scene.colliders[1].kind = MPM_COLLIDER_BOX;
    scene.colliders[1].end_time = 999.0f;
    scene.particle_begin = 0;
    scene.particle_count = n;
    MpmPlan plan;
    CHECK(mpm_plan(&scene, 1, n, 0, &plan));

    float *x0 = (float *)malloc(sizeof(float) * 3 * n), *vol = (float *)malloc(sizeof(float) * n);
    float *mass = (float *)malloc(sizeof(float) * n), *u = (float *)malloc(sizeof(float) * 3 * n);
    srand(0);
    for (int i = 0; i < n; ++i) {
        x0[3 * i + 0] = 0.35f + 0.3f * rand() / (float)RAND_MAX;
        x0[3 * i + 1] = 0.35f + 0.3f * rand() / (float)RAND_MAX;
        x0[3 * i + 2] = 0.15f + 0.6f * rand() / (float)RAND_MAX;
        vol[i] = 0.3f * 0.3f * 0.6f / n;
        mass[i] = rho * vol[i];
    }

    MpmBuffers b = {0};
    if (cudaMalloc(&b.state[0], plan.state_bytes) != cudaSuccess ||
        cudaMalloc(&b.state[1], plan.state_bytes) != cudaSuccess ||
        cudaMalloc(&b.workspace, plan.workspace_bytes) != cudaSuccess ||
        cudaMalloc(&b.scenes, sizeof(MpmScene)) != cudaSuccess ||
        cudaMalloc((void **)&b.status, sizeof(int32_t)) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc failed\n");
        return 1;
    }
    b.plan = plan;
    cudaStream_t stream;
    cudaStreamCreate(&stream);
    CHECK(mpm_init(&b, stream));
    CHECK(mpm_upload_scenes(&b, &scene, 1, stream));
    CHECK(mpm_load(&b, MPM_FIELD_X_INITIAL, x0, 1, stream));
    CHECK(mpm_load(&b, MPM_FIELD_VOL, vol, 1, stream));
    CHECK(mpm_load(&b, MPM_FIELD_MASS, mass, 1, stream));
    for (int k = 0; k < 20; ++k) CHECK(mpm_p2g2p(&b, (float)(k * dt), dt, stream));
    CHECK(mpm_export(&b, MPM_FIELD_U, u, 1, stream));
    int32_t status = 0;
    cudaMemcpyAsync(&status, b.status, sizeof(status), cudaMemcpyDeviceToHost, stream);
    cudaStreamSynchronize(stream);
    double uz = 0.0;
    for (int i = 0; i < n; ++i) uz += u[3 * i + 2];
    printf("mean u_z %.6e status %d\n", uz / n, status);
    cudaFree(b.state[0]);
    cudaFree(b.state[1]);
    cudaFree(b.workspace);
    cudaFree(b.scenes);
    cudaFree(b.status);
    cudaStreamDestroy(stream);
    free(x0);
    free(vol);
    free(mass);
    free(u);
    return status != 0;
}
