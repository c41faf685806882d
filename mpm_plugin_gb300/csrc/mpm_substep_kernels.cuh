// The kernels of one substep, written once for two ways of naming the scenes they work on:
//   OneScene    - a single scene whose arguments are kernel parameters (the plain solver);
//   SceneTable  - a device table of scenes (a batch). Particle kernels take one scene per CTA (a per-CTA
//                 scene index), the kernels over work lists walk every scene's list in turn, and a scene
//                 whose advance is done (StepParams::active == 0) is skipped by all of them.
// One substep = step_begin -> clear -> P2G -> grid update -> collider contact -> G2P -> particle projection
// (warp/solver.py:187-212 for the order).
#pragma once

#include "mpm_substep.cuh"

namespace mpm {

struct OneScene {
    SubstepArgs a;
    __device__ __forceinline__ int count() const { return 1; }
    __device__ __forceinline__ SubstepArgs get(int) const { return a; }
    __device__ __forceinline__ int scene_of_cta(unsigned int) const { return 0; }
    __device__ __forceinline__ unsigned int first_cta(int) const { return 0; }
    __device__ __forceinline__ bool active(const SubstepArgs&) const { return true; }
};

struct SceneTable {
    const SubstepArgs* __restrict__ scenes;
    const int32_t* __restrict__ cta_scene;  // particle kernels: the scene of each CTA
    const int32_t* __restrict__ cta_first;  // per scene: its first CTA in the particle kernels
    int n;
    __device__ __forceinline__ int count() const { return n; }
    __device__ __forceinline__ SubstepArgs get(int s) const { return scenes[s]; }
    __device__ __forceinline__ int scene_of_cta(unsigned int b) const { return __ldg(&cta_scene[b]); }
    __device__ __forceinline__ unsigned int first_cta(int s) const { return (unsigned int)__ldg(&cta_first[s]); }
    __device__ __forceinline__ bool active(const SubstepArgs& a) const { return a.sp->active != 0; }
};

// Warp-aggregated append: one atomic per warp.
__device__ __forceinline__ void warp_append(int32_t* __restrict__ list, unsigned int* __restrict__ count, int32_t v) {
    const unsigned int mask = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    list[base + __popc(mask & ((1u << lane) - 1u))] = v;
}

// ------------------------------------------------------------------------------------------------------
// Start of a substep: counters, substep fraction s = (k + 1) / steps (warp/solver.py:218-219), pose offset;
// the work lists of this substep start empty. A scene that has run all `steps` substeps of its advance
// goes idle (active = 0) and keeps its counters, so its next advance continues where it stopped.
// ------------------------------------------------------------------------------------------------------
__device__ __forceinline__ void step_begin(StepParams* sp, unsigned int* counts, int n_col) {
    StepParams p = *sp;
    if (p.steps > 0 && p.k + 1 >= p.steps) {
        sp->active = 0;
        return;
    }
    p.active = 1;
    p.seq += 1;
    if (p.steps > 0) {
        p.k += 1;
        p.s = (float)((double)(p.k + 1) / (double)p.steps);
        p.pose_base = p.k * n_col;
    } else {
        p.pose_base = 0;
    }
    *sp = p;
    counts[p.seq & 1u] = 0u;
    counts[2] = 0u;
    counts[3] = 0u;
}

template <class Scenes>
__global__ void k_step_begin(Scenes sc) {
    for (int s = threadIdx.x; s < sc.count(); s += blockDim.x) {
        const SubstepArgs a = sc.get(s);
        step_begin(a.sp, a.wl.counts, a.cd.n_col);
    }
}

// Zeroes the grid blocks the previous substep used (and their flags), so the whole grid is zero again.
template <class Scenes>
__global__ void __launch_bounds__(256) k_clear_blocks(Scenes sc) {
    for (int s = 0; s < sc.count(); ++s) {
        const SubstepArgs a = sc.get(s);
        if (!sc.active(a)) continue;
        const unsigned int prev = (a.sp->seq - 1u) & 1u;
        const unsigned int n = a.wl.counts[prev];
        const int32_t* __restrict__ list = active_blocks(a.wl, prev);
        for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += gridDim.x * 4u) {
            const int64_t b = list[i];
            a.grid[b * 64 + (threadIdx.x & 63)] = make_float4(0.f, 0.f, 0.f, 0.f);
            if ((threadIdx.x & 63) == 0) a.wl.block_flag[b] = 0u;
        }
    }
}

// P2G with warp-level aggregation: lanes whose stencils start at the same grid node (neighbours in the
// particle order after the reorder by grid node) form a segment; each of the 27 x 4 contributions is summed
// over the segment with shuffles (after round r a lane holds the sum of the next 2^r lanes of its segment)
// and only the segment's first lane issues the 16-byte reduction, so a cell of ~8 particles costs one
// reduction per node instead of eight. Lanes past the end or with a stencil outside the grid are
// single-lane segments that add nothing. The segment's first lane also lists the grid blocks it touches.
template <class Scenes>
__global__ void __launch_bounds__(256) k_p2g_scatter(Scenes sc) {
    const int s = sc.scene_of_cta(blockIdx.x);
    const SubstepArgs a = sc.get(s);
    if (!sc.active(a)) return;
    const int64_t first = (int64_t)(blockIdx.x - sc.first_cta(s)) * blockDim.x;
    const int64_t p = first + threadIdx.x;
    const int lane = (int)(threadIdx.x & 31u);
    if (first + (threadIdx.x & ~31u) >= a.n) return;  // whole warp past the end
    const GridDesc& g = a.g;
    const Particles P = particles_of(a);
    P2gTerms t;
    const bool valid = p < a.n && p2g_terms(P, p, a.mats, g, a.sp->dt, t);
    const int64_t key = valid ? node_index(g, t.base[0], t.base[1], t.base[2]) : -1 - (int64_t)lane;
    const int64_t key_prev = __shfl_up_sync(0xffffffffu, key, 1);
    const int64_t key_next = __shfl_down_sync(0xffffffffu, key, 1);
    const bool seg_first = lane == 0 || key_prev != key;
    const bool seg_last = lane == 31 || key_next != key;
    const unsigned int ends = __ballot_sync(0xffffffffu, seg_last);
    const int tail = __ffs(ends >> lane) - 1;  // lanes after this one in its segment
    const int span = (int)__reduce_max_sync(0xffffffffu, (unsigned int)tail);
    const bool leader = valid && seg_first;
    if (leader) {
        const unsigned int cur = a.sp->seq & 1u;
        mark_stencil_blocks(g, t.base, a.wl.block_flag, active_blocks(a.wl, cur), &a.wl.counts[cur]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float val[4] = {0.f, 0.f, 0.f, 0.f};
                if (valid) p2g_node(t, g, i, j, k, val);
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    if (d <= span) {  // warp-uniform
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float o = __shfl_down_sync(0xffffffffu, val[c], d);
                            if (d <= tail) val[c] += o;
                        }
                    }
                }
                if (leader)
                    grid_add(&a.grid[node_index(g, t.base[0] + i, t.base[1] + j, t.base[2] + k)], val[0], val[1],
                             val[2], val[3]);
            }
}

// Grid update (normalise, gravity, walls) over the active blocks, four 4x4x4 blocks per 256-thread CTA;
// nodes with mass inside some collider's margin box are listed for k_grid_colliders.
template <class Scenes>
__global__ void __launch_bounds__(256) k_grid_update(Scenes sc) {
    for (int s = 0; s < sc.count(); ++s) {
        const SubstepArgs a = sc.get(s);
        if (!sc.active(a)) continue;
        const GridDesc& g = a.g;
        const unsigned int cur = a.sp->seq & 1u;
        const unsigned int n = a.wl.counts[cur];
        const float dt = a.sp->dt;
        ColliderData cd = a.cd;
        cd.poses += a.sp->pose_base;
        const int l = threadIdx.x & 63;
        for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += gridDim.x * 4u) {
            const int64_t b = active_blocks(a.wl, cur)[i];
            const int bk = (int)(b % g.nb[2]);
            const int bj = (int)((b / g.nb[2]) % g.nb[1]);
            const int bi = (int)(b / ((int64_t)g.nb[2] * g.nb[1]));
            const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
            bool has_mass = grid_node_walls(g, &a.grid[b * 64 + l], idx, dt);
            if (has_mass && cd.n_col > 0) {
                float pos[3];
                node_position(g, idx, pos);
                if (near_any_collider(pos, cd)) warp_append(a.wl.node_cand, &a.wl.counts[2], (int32_t)(b * 64 + l));
            }
        }
    }
}

// Mesh-collider contact of the listed nodes (full warps of candidates; voxel grid, then BVH queries).
template <class Scenes>
__global__ void __launch_bounds__(128) k_grid_colliders(Scenes sc) {
    for (int s = 0; s < sc.count(); ++s) {
        const SubstepArgs a = sc.get(s);
        if (!sc.active(a) || a.cd.n_col == 0) continue;
        const GridDesc& g = a.g;
        const unsigned int n = a.wl.counts[2];
        ColliderData cd = a.cd;
        cd.poses += a.sp->pose_base;
        for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const int64_t q = a.wl.node_cand[i];
            const int64_t b = q >> 6;
            const int l = (int)(q & 63);
            const int bk = (int)(b % g.nb[2]);
            const int bj = (int)((b / g.nb[2]) % g.nb[1]);
            const int bi = (int)(b / ((int64_t)g.nb[2] * g.nb[1]));
            const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
            grid_node_colliders(g, &a.grid[q], idx, cd);
        }
    }
}

// G2P; particles that end inside a collider's margin box are listed for k_project_particles. Capped at 80
// registers (3 CTAs of 256 per SM): the kernel is bound by instruction latency, and the extra resident warps
// outweigh the few spilled values (measured 10 % faster than the uncapped 120 registers).
template <class Scenes>
__global__ void __launch_bounds__(256, 3) k_g2p(Scenes sc) {
    const int s = sc.scene_of_cta(blockIdx.x);
    const SubstepArgs a = sc.get(s);
    if (!sc.active(a)) return;
    const int64_t p = (int64_t)(blockIdx.x - sc.first_cta(s)) * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    float nx[3];
    g2p_particle(particles_of(a), p, a.mats, a.g, a.sp->dt, a.grid, a.fp64, nx);
    if (a.cd.n_col > 0) {
        ColliderData cd = a.cd;
        cd.poses += a.sp->pose_base;
        if (near_any_collider(nx, cd)) warp_append(a.wl.part_cand, &a.wl.counts[3], (int32_t)p);
    }
}

template <class Scenes>
__global__ void __launch_bounds__(128) k_project_particles(Scenes sc) {
    for (int s = 0; s < sc.count(); ++s) {
        const SubstepArgs a = sc.get(s);
        if (!sc.active(a) || a.cd.n_col == 0) continue;
        const unsigned int n = a.wl.counts[3];
        ColliderData cd = a.cd;
        cd.poses += a.sp->pose_base;
        const Particles P = particles_of(a);
        for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            project_particle(P, a.wl.part_cand[i], a.g, cd);
    }
}

}  // namespace mpm
