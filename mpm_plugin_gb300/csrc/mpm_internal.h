// Launchers of the kernels in mpm_kernels.cu, called by the C-ABI host code in mpm_abi.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "mpm_types.h"

namespace mpm {

struct EscapeBounds {  // particles past these planes on open sides are removed (warp/solver.py:222-240)
    int open_lo[3], open_hi[3];
    float lo[3], hi[3];
};

// Records the message mpm_last_error(NULL) returns on this thread.
void set_last_error(const std::string& msg);

void launch_step_begin(cudaStream_t st, StepParams* sp, ColliderDev* cols, int n_col);
void launch_p2g(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                float4* grid, unsigned int* fp64);
void launch_grid_update(cudaStream_t st, const GridDesc& g, float4* grid, const StepParams* sp, const ColliderDev* cols,
                        int n_col, const BvhNode* nodes, const MeshTri* tris);
void launch_g2p(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                const float4* grid, const ColliderDev* cols, int n_col, const BvhNode* nodes, const MeshTri* tris,
                unsigned int* fp64);
void launch_max_speed(cudaStream_t st, const Particles& P, unsigned int* out);
void launch_state_in(cudaStream_t st, const Particles& P, int64_t off, int64_t n, const float* x, const float* v,
                     const float* C, const float* F, const float* Jp, const int32_t* mat, const int32_t* emitter);
void launch_state_out(cudaStream_t st, const Particles& P, float* x, float* v, float* C, float* F, float* Jp,
                      int32_t* mat, int32_t* emitter);
void launch_flag_escaped(cudaStream_t st, const Particles& P, const EscapeBounds& eb, int32_t* keep_phys,
                         int32_t* keep_by_id, unsigned int* removed_per_mat);
void launch_compact(cudaStream_t st, const Particles& src, const Particles& dst, const int32_t* keep_phys,
                    const int32_t* dst_index, const int32_t* new_id);
int64_t scan_tile_count(int64_t n);
void launch_exclusive_scan(cudaStream_t st, const int32_t* in, int64_t n, int32_t* out, int32_t* tile_tmp,
                           int32_t* total);
void launch_scatter_volume(cudaStream_t st, const Particles& P, const GridDesc& g, float* vol);
void launch_grid_unblock(cudaStream_t st, const GridDesc& g, const float4* grid, float4* out);
void launch_query_fill(cudaStream_t st, const GridDesc& g, const float* vol, float cell_vol, int64_t m,
                       const float* pts, uint8_t* out);

}  // namespace mpm
