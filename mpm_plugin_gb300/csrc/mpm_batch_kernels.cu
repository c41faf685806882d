// The batched substep: the substep kernels of mpm_substep_kernels.cuh over a device table of scenes, one
// launch per kernel for all scenes of a batch.
#include <cuda_runtime.h>

#include <algorithm>

#include "mpm_internal.h"
#include "mpm_substep_kernels.cuh"

namespace mpm {

void launch_batch_substep(cudaStream_t st, const BatchLaunch& b) {
    const SceneTable sc{b.scenes, b.cta_scene, b.cta_first, b.n_scenes};
    const unsigned int list_ctas = b.shape.list_ctas ? b.shape.list_ctas : sm_count() * kCtasPerSm;
    const bool pdl = b.shape.pdl != 0;
    // P2G and G2P walk the (scene, chunk) list of the running scenes: enough CTAs for every chunk of every
    // scene, at most eight per SM
    const unsigned int walk_ctas = std::min<unsigned int>(b.particle_ctas, sm_count() * 8u);
    launch_step_kernel(k_step_begin<SceneTable>, 1, 128, st, pdl, sc);
    launch_step_kernel(k_clear_blocks<SceneTable>, list_ctas, 256, st, pdl, sc);
    if (b.particle_ctas > 0) {  // a deterministic scene takes the warp-segment path inside k_p2g_tile
        const bool merge = b.shape.p2g_merge != 0;
        if (b.shape.p2g_tile)
            launch_step_kernel_smem(k_p2g_tile<SceneTable>, b.particle_ctas, 256, kP2gTileBytes, st, pdl, sc);
        else
            launch_step_kernel(b.any_fixed ? k_p2g_scatter<SceneTable>  // (the fixed-point path does not merge)
                                           : (merge ? k_p2g_scatter<SceneTable, false, false, 2, true>
                                                    : k_p2g_scatter<SceneTable, false, false>),
                               walk_ctas, 256, st, pdl, sc);
    }
    launch_step_kernel(k_grid_update<SceneTable>, list_ctas, 256, st, pdl, sc);
    if (b.any_colliders) launch_step_kernel(k_grid_colliders<SceneTable>, list_ctas, 128, st, pdl, sc);
    if (b.particle_ctas > 0) {
        if (b.any_fp64_clamp)
            launch_step_kernel(k_g2p<SceneTable, 2, true>, walk_ctas, 256, st, pdl, sc);
        else if (b.shape.g2p_variant == 1)
            launch_step_kernel(k_g2p<SceneTable, 1>, walk_ctas, 256, st, pdl, sc);
        else
            launch_step_kernel(k_g2p<SceneTable, 3>, walk_ctas, 256, st, pdl, sc);
    }
    if (b.any_colliders) launch_step_kernel(k_project_particles<SceneTable>, list_ctas, 128, st, pdl, sc);
}

cudaError_t prepare_batch_kernels() {
    return cudaFuncSetAttribute(k_p2g_tile<SceneTable>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP2gTileBytes);
}

int batch_substep_kernel_count(const BatchLaunch& b) {
    return 3 + (b.particle_ctas > 0 ? 2 : 0) + (b.any_colliders ? 2 : 0);
}

}  // namespace mpm
