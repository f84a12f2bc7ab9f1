/* A plain-C caller of the library's host-side entry points (no GPU needed):
 * plans the buffers of one 1,024-particle sand scene on a 32^3 grid and
 * prints the ABI version, the struct sizes and the plan.  Built and run by
 * tests/test_capi_cpu.py::test_plain_c_caller. */
#include <stdio.h>

#include "mpm_gb300.h"

int main(void) {
    MpmScene scene = {0};
    scene.n_grid = 32;
    scene.dx = 1.0f / 32.0f;
    scene.inv_dx = 32.0f;
    scene.material = MPM_SAND;
    scene.particle_begin = 0;
    scene.particle_count = 1024;
    MpmPlan plan;
    int r = mpm_plan(&scene, 1, 1024, 0, &plan);
    if (r != MPM_OK) {
        printf("mpm_plan: %s\n", mpm_error_string(r));
        return 1;
    }
    int64_t sizes[6];
    mpm_struct_sizes(sizes);
    printf("abi %d sizes %lld %lld %lld %lld %lld %lld\n", mpm_abi_version(), (long long)sizes[0],
           (long long)sizes[1], (long long)sizes[2], (long long)sizes[3], (long long)sizes[4], (long long)sizes[5]);
    printf("plan %lld %lld %lld %lld %d\n", (long long)plan.state_bytes, (long long)plan.workspace_bytes,
           (long long)plan.total_blocks, (long long)plan.particle_stride, plan.chunk_size);
    scene.dx = 0.0f; /* a bad scene is refused */
    printf("bad %d\n", mpm_plan(&scene, 1, 1024, 0, &plan));
    return 0;
}
