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

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount, cached per device; 1 if
// the query fails). Grids that stride over device-sized work are sized as a multiple of it.
unsigned int sm_count();
constexpr unsigned int kCtasPerSm = 8;  // default CTAs per SM of the kernels that stride over work lists


void launch_collider_poses(cudaStream_t st, const ColliderDev* cols, int n_col, ColliderPose* poses, int steps,
                           float s_given, float inv_frame_dt);
// One substep: step counters, clear of the previous blocks, P2G, grid update, collider contact, G2P,
// particle projection. With ev (5 events), records ev[0..4] around: clear | P2G | grid | G2P (as event
// nodes when `capturing`).
// Launch choices the autotuner sets: CTAs of the kernels that walk work lists, the G2P build (0: capped
// at 80 registers, 3 CTAs of 256 per SM; 1: uncapped) and P2G's reduction group.
struct LaunchShape {
    unsigned int list_ctas = 0;  // 0: kCtasPerSm per SM of the device (resolved at launch)
    int g2p_variant = 0;
    int p2g_group = 32;  // lanes of the aligned groups P2G sums within (a power of two, 1 .. 32)
    int pdl = 1;         // 1: the substep kernels launch with programmatic dependent launch
    int p2g_tile = 0;    // 1: P2G through shared-memory tiles per CTA (k_p2g_tile); 0: warp segments only
    int block_sweep = 0; // 1: P2G flags blocks with plain stores, k_list_blocks lists them (one grid only)
    int ppt = 1;         // particles per thread of the plain P2G and G2P (grid = ceil(chunks / ppt) CTAs)
    int p2g_merge = 1;   // 1: P2G merges its leaders' sums along z before the reductions
};

// Launch of a substep kernel: with shape.pdl the launch carries the programmatic-stream-serialization
// attribute (the kernel's launch may overlap the previous kernel's tail; the kernel waits for it itself).
template <typename... KArgs, typename... Args>
inline void launch_step_kernel_smem(void (*kernel)(KArgs...), unsigned int grid, unsigned int block, size_t smem,
                                    cudaStream_t st, bool pdl, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}
template <typename... KArgs, typename... Args>
inline void launch_step_kernel(void (*kernel)(KArgs...), unsigned int grid, unsigned int block, cudaStream_t st,
                               bool pdl, Args... args) {
    launch_step_kernel_smem(kernel, grid, block, 0, st, pdl, args...);
}
// Function attributes the substep kernels need (the tiled P2G's dynamic shared memory above 48 KB); called
// once per solver and batch, outside stream capture.
cudaError_t prepare_substep_kernels();
cudaError_t prepare_batch_kernels();
void launch_substep(cudaStream_t st, const SubstepArgs& a, const LaunchShape& shape, cudaEvent_t* ev, bool capturing);
// reps substeps of one scene in one cooperative launch (k_substeps_coop); bar: 3 device words (barrier and
// error flag), zeroed here. Grid: the particle chunks of 256, at most the CTAs resident at once.
cudaError_t launch_substeps_coop(cudaStream_t st, const SubstepArgs& a, int reps, unsigned int* bar);
// One grid barrier on 2 CTAs (cooperative); with stall no CTA completes it and both give up after the spin
// limit. *timed_out (host) receives the error flag; synchronises the stream.
cudaError_t barrier_selftest(cudaStream_t st, bool stall, unsigned int* bar, unsigned int* timed_out);
int substep_kernel_count(const SubstepArgs& a);

// One batched substep over a device table of scenes (mpm_batch_kernels.cu). The particle kernels run
// particle_ctas CTAs of 256 threads; CTA b works on scene cta_scene[b], particles
// (b - cta_first[scene]) * 256 + thread.
struct BatchLaunch {
    const SubstepArgs* scenes;
    const int32_t* cta_scene;
    const int32_t* cta_first;
    int n_scenes;
    unsigned int particle_ctas;
    bool any_colliders;
    bool any_fp64_clamp;  // some scene redoes the plastic clamp in FP64 (the G2P build with the redo)
    bool any_fixed;       // some scene is in deterministic mode (the P2G build with the fixed-point path)
    LaunchShape shape;
};
void launch_batch_substep(cudaStream_t st, const BatchLaunch& b);
int batch_substep_kernel_count(const BatchLaunch& b);
// Occupancy in deterministic mode: the volume splat as fixed-point integers (unsigned per node, 2^-20
// particle volumes per unit) and the query against 0.5 cell_vol in those units.
void launch_scatter_volume_fixed(cudaStream_t st, const Particles& P, const GridDesc& g, unsigned int* vol);
void launch_query_fill_fixed(cudaStream_t st, const GridDesc& g, const unsigned int* vol, double cell_vol, int64_t m,
                             const float* pts, uint8_t* out);
// FP64 totals: mass, momentum xyz, mass-weighted position xyz, kinetic energy, non-finite particles.
void launch_conservation(cudaStream_t st, const Particles& P, const Material* mats, double* out);
// Counting sort of the particles by the grid node of their stencil base: fills ss.order (scan_tmp: scan
// scratch of scan_cap + 2 entries, at least scan_tile_count(n_nodes + 1) + 1).
void launch_sort(cudaStream_t st, const Particles& P, const GridDesc& g, const SortScratch& ss, int64_t n_nodes,
                 int32_t* scan_tmp, int64_t scan_cap);
// Kirchhoff stress of the particles [off, off + n) from their F and Jp.
void launch_particle_stress(cudaStream_t st, const Particles& P, int64_t off, int64_t n, const Material* mats,
                            unsigned int* fp64);
// dst[i] = src[order[i]] for every field of a particle arena (kParticleFields planes of cap words each).
void launch_permute(cudaStream_t st, const void* src_arena, void* dst_arena, int64_t cap, int64_t n,
                    const int32_t* order);

constexpr int kSdfMaxCandidates = 128;
// Narrow-band voxel grid of one collider: classify every voxel (cells[v].y: candidate count, kSdfFar or
// kSdfUseBvh; counts[v]: the count, 0 otherwise), then, with starts = exclusive scan of counts plus the
// collider's base, write the candidate lists (cells[v].x: first candidate).
void launch_sdf_classify(cudaStream_t st, const ColliderDev& col, const BvhNode* nodes, const MeshTri* tris,
                         int64_t n_vox, int max_cand, int2* cells, int32_t* counts);
void launch_sdf_fill(cudaStream_t st, const ColliderDev& col, const BvhNode* nodes, const MeshTri* tris, int64_t n_vox,
                     int max_cand, int2* cells, const int32_t* starts, int32_t* cand);
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
