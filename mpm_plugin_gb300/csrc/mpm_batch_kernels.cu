// The batched substep: the substep kernels of mpm_substep_kernels.cuh over a device table of scenes, one
// launch per kernel for all scenes of a batch.
#include <cuda_runtime.h>

#include "mpm_internal.h"
#include "mpm_substep_kernels.cuh"

namespace mpm {

void launch_batch_substep(cudaStream_t st, const BatchLaunch& b) {
    const SceneTable sc{b.scenes, b.cta_scene, b.cta_first, b.n_scenes};
    const unsigned int list_ctas = b.shape.list_ctas;
    k_step_begin<<<1, 128, 0, st>>>(sc);
    k_clear_blocks<<<list_ctas, 256, 0, st>>>(sc);
    if (b.particle_ctas > 0) k_p2g_scatter<<<b.particle_ctas, 256, 0, st>>>(sc);
    k_grid_update<<<list_ctas, 256, 0, st>>>(sc);
    if (b.any_colliders) k_grid_colliders<<<list_ctas, 128, 0, st>>>(sc);
    if (b.particle_ctas > 0) {
        if (b.shape.g2p_variant == 1)
            k_g2p<SceneTable, 1><<<b.particle_ctas, 256, 0, st>>>(sc);
        else
            k_g2p<SceneTable, 3><<<b.particle_ctas, 256, 0, st>>>(sc);
    }
    if (b.any_colliders) k_project_particles<<<list_ctas, 128, 0, st>>>(sc);
}

int batch_substep_kernel_count(const BatchLaunch& b) {
    return 3 + (b.particle_ctas > 0 ? 2 : 0) + (b.any_colliders ? 2 : 0);
}

}  // namespace mpm
