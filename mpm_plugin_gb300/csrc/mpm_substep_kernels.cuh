// The kernels of one substep, written once for two ways of naming the scenes they work on:
//   OneScene    - a single scene whose arguments are kernel parameters (the plain solver);
//   SceneTable  - a device table of scenes (a batch). Particle kernels take one scene per CTA (a per-CTA
//                 scene index), the kernels over work lists share out the flattened (scene, item) list of
//                 all scenes, and a scene whose advance is done (StepParams::active == 0) is skipped by all.
// One substep = step_begin -> clear -> P2G -> grid update -> collider contact -> G2P -> particle projection
// (warp/solver.py:187-212 for the order).
//
// Two-grid mode (SubstepArgs::grid2 set; one scene, not in deterministic mode): substep seq uses grid
// grid_of(seq & 1) and active list seq & 1. Within an advance (or between explicit substeps with the same dt)
// the G2P of substep seq also scatters every particle it has just updated into the grid of substep seq + 1,
// and the projection kernel scatters the particles it projected, so the P2G kernel of seq + 1 has nothing
// left to do (StepParams::p2g_skip). The bookkeeping that makes this hold:
//   clear(seq)        zeroes the blocks of list (seq - 1) & 1 in grid (seq - 1) & 1 = the grid G2P(seq) fills;
//   grid update(seq)  empties list (seq + 1) & 1 (cleared above, read by nobody after the clear) and takes the
//                     block flags of list seq & 1 down, so G2P(seq) can list the blocks it scatters into;
//   step begin(seq)   empties list seq & 1 only when P2G(seq) will fill it.
// The host discards a scatter made for a substep that does not follow (zero grids, flags and lists).
#pragma once

#include <climits>

#include "mpm_substep.cuh"

namespace mpm {

struct OneScene {
    static constexpr bool kTable = false;
    SubstepArgs a;
    __device__ __forceinline__ int count() const { return 1; }
    __device__ __forceinline__ SubstepArgs get(int) const { return a; }
    __device__ __forceinline__ int scene_of_cta(unsigned int) const { return 0; }
    __device__ __forceinline__ unsigned int first_cta(int) const { return 0; }
    __device__ __forceinline__ bool active(const SubstepArgs&) const { return true; }
};

struct SceneTable {
    static constexpr bool kTable = true;
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

// Programmatic dependent launch: every substep kernel first lets the next kernel of the sequence start
// launching (its CTAs are placed once all CTAs of this one have begun), then waits until the kernel before
// it has completed and its writes are visible. Launch latency overlaps the previous kernel's tail; without
// the launch attribute both instructions do nothing. The wait ends when a grid that is already running
// completes, so it cannot hang.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

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
// (scene, item) work lists of a batch: every CTA loads the item count of each scene (0 for an idle scene)
// into shared memory and scans it, so that the flattened items 0 .. total-1 are shared out over all CTAs and
// item q belongs to the scene s with off[s] <= q < off[s + 1] (binary search). One warp scans, 32 scenes per
// round. count(a) returns the scene's item count.
// ------------------------------------------------------------------------------------------------------
template <class Scenes, class Count>
__device__ __forceinline__ unsigned int scene_offsets(const Scenes& sc, Count count, unsigned int* off) {
    const int S = sc.count();
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
        const SubstepArgs a = sc.get(s);
        off[s + 1] = sc.active(a) ? count(a) : 0u;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned int carry = 0;
        for (int base = 0; base < S; base += 32) {
            const int s = base + (int)threadIdx.x;
            unsigned int v = s < S ? off[s + 1] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, v, o);
                if ((int)threadIdx.x >= o) v += y;
            }
            if (s < S) off[s + 1] = carry + v;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
        if (threadIdx.x == 0) off[0] = 0u;
    }
    __syncthreads();
    return off[S];
}

// The scene of flattened item q: the last s with off[s] <= q.
__device__ __forceinline__ int scene_of_item(const unsigned int* off, int S, unsigned int q) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------------------------------------------------
// Start of a substep: counters, substep fraction s = (k + 1) / steps (warp/solver.py:218-219), pose offset;
// the work lists of this substep start empty. A scene that has run all `steps` substeps of its advance
// goes idle (active = 0) and keeps its counters, so its next advance continues where it stopped.
// ------------------------------------------------------------------------------------------------------
// two: two-grid mode (the substep's G2P may scatter for the next substep, see the top of this file).
__device__ __forceinline__ void step_begin(StepParams* sp, unsigned int* counts, int n_col, bool two) {
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
    // within an advance the next substep has the same dt; an explicit substep scatters on the host's word
    p.p2g_skip = two && (p.steps > 0 ? p.k > 0 : p.skip_first != 0);
    p.scatter = two && (p.steps > 0 ? p.k + 1 < p.steps : p.speculate != 0);
    *sp = p;
    if (!p.p2g_skip) counts[p.seq & 1u] = 0u;
    counts[2] = 0u;
    counts[3] = 0u;
}

template <class Scenes>
__global__ void k_step_begin(Scenes sc) {
    pdl_begin();
    for (int s = threadIdx.x; s < sc.count(); s += blockDim.x) {
        const SubstepArgs a = sc.get(s);
        step_begin(a.sp, a.wl.counts, a.cd.n_col, a.grid2 != nullptr);
    }
}

// Zeroes the grid blocks the previous substep used (and their flags), so the whole grid is zero again.
// Four blocks per 256-thread CTA. prev: the previous substep's parity.
__device__ __forceinline__ void clear_block(const SubstepArgs& a, unsigned int prev, unsigned int i) {
    const int64_t b = active_blocks(a.wl, prev)[i];
    const int64_t q = b * 64 + (threadIdx.x & 63);
    grid_of(a, prev)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.fixed) {
        reinterpret_cast<ulonglong2*>(a.fixed)[2 * q] = make_ulonglong2(0ull, 0ull);
        reinterpret_cast<ulonglong2*>(a.fixed)[2 * q + 1] = make_ulonglong2(0ull, 0ull);
        a.poison[q] = 0u;
    }
    if ((threadIdx.x & 63) == 0) a.wl.block_flag[b] = 0u;
}

// Where a segment's leader adds its sums when the warp's segments are merged along z (p2g_column_sums):
// src1 / src2 the lanes of the previous two leaders, d1 the z distance to the previous leader when it shares
// the leader's x and y base (1 or 2, else 0), ok2 whether the one before that sits at z distance 2 (with
// d1 = 1), ws the z distance to the next leader when it shares x and y (1 or 2, else 0).
struct ColumnMerge {
    int src1, src2, d1, ws;
    bool ok2;
};

// The merge bookkeeping of one lane (meaningful for leaders; a lane with no earlier or later leader names
// itself and merges nothing).
__device__ __forceinline__ ColumnMerge column_merge_of(const P2gTerms& t, bool valid, bool leader, int lane) {
    const unsigned int leaders = __ballot_sync(0xffffffffu, leader);
    const unsigned int below = leaders & ((1u << lane) - 1u);
    const int p1 = below ? 31 - __clz(below) : lane;
    const unsigned int below2 = below & ((1u << p1) - 1u);
    const int p2 = below2 ? 31 - __clz(below2) : lane;
    const unsigned int above = lane == 31 ? 0u : leaders & ~((2u << lane) - 1u);
    const int s1 = above ? __ffs(above) - 1 : lane;
    const int xy = valid ? t.base[0] * 65536 + t.base[1] : -1 - lane;  // x, y base (grid dims < 65536)
    const int z = t.base[2];
    const int xy1 = __shfl_sync(0xffffffffu, xy, p1), z1 = __shfl_sync(0xffffffffu, z, p1);
    const int xy2 = __shfl_sync(0xffffffffu, xy, p2), z2 = __shfl_sync(0xffffffffu, z, p2);
    const int xys = __shfl_sync(0xffffffffu, xy, s1), zs = __shfl_sync(0xffffffffu, z, s1);
    ColumnMerge m;
    m.src1 = p1;
    m.src2 = p2;
    m.d1 = (p1 != lane && xy1 == xy && (z - z1 == 1 || z - z1 == 2)) ? z - z1 : 0;
    m.ok2 = m.d1 == 1 && p2 != p1 && xy2 == xy && z - z2 == 2;
    m.ws = (s1 != lane && xys == xy && (zs - z == 1 || zs - z == 2)) ? zs - z : 0;
    return m;
}

// Deterministic-mode P2G of one warp (k_p2g_scatter's arguments): every contribution becomes a 64-bit
// fixed-point integer (the float times 2^fixed_exp, exact, then rounded to an integer) before it is summed,
// so the warp sums and the global atomics are exact integer additions and the node totals do not depend on
// particle order or atomic timing. A non-finite or out-of-range contribution poisons its node instead (the
// grid update then makes that node NaN, as a float sum would). (Merging the leaders' sums along z here, as
// the float path does, kept the totals bit-identical but spilled the 64-bit values: P2G 94.6 against 80.0 us
// in the deterministic profiling case, measured, so this path does not merge.)
__device__ __forceinline__ void p2g_fixed_warp(const SubstepArgs& a, const P2gTerms& t, bool valid, bool leader,
                                               int tail, int span) {
    const GridDesc& g = a.g;
    const float scale = __int_as_float((127 + a.fixed_exp) << 23);  // 2^fixed_exp
#pragma unroll
    for (int n = 0; n < 27; ++n) {
        const int i = n / 9, j = (n / 3) % 3, k = n % 3;
        float val[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid) p2g_node(t, i, j, k, val);
        long long q[4];
        bool bad = false;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float x = val[c] * scale;
            const bool ok = fabsf(x) < 4.0e18f;  // false for NaN and inf too
            bad |= !ok;
            q[c] = ok ? __float2ll_rn(x) : 0ll;
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            if (d <= span) {  // warp-uniform
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const long long o = __shfl_down_sync(0xffffffffu, q[c], d);
                    if (d <= tail) q[c] += o;
                }
            }
        }
        const int64_t node = valid ? node_index(g, t.base[0] + i, t.base[1] + j, t.base[2] + k) : 0;
        if (valid && bad) atomicOr(&a.poison[node], 1u);
        if (leader) {
            unsigned long long* f = a.fixed + node * 4;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (q[c] != 0) atomicAdd(&f[c], (unsigned long long)q[c]);
        }
    }
}

// Runs after k_step_begin: seq has advanced, so the substep before has parity (seq - 1) & 1.
template <class Scenes>
__global__ void __launch_bounds__(256) k_clear_blocks(Scenes sc) {
    pdl_begin();
    if constexpr (!Scenes::kTable) {
        const SubstepArgs a = sc.get(0);
        const unsigned int prev = (a.sp->seq - 1u) & 1u;
        const unsigned int n = a.wl.counts[prev];
        for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += gridDim.x * 4u) clear_block(a, prev, i);
    } else {
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total = scene_offsets(sc, [](const SubstepArgs& a) {
            return a.wl.counts[(a.sp->seq - 1u) & 1u];
        }, off);
        for (unsigned int q = blockIdx.x * 4u + (threadIdx.x >> 6); q < total; q += gridDim.x * 4u) {
            const int s = scene_of_item(off, sc.count(), q);
            const SubstepArgs a = sc.get(s);
            clear_block(a, (a.sp->seq - 1u) & 1u, q - off[s]);
        }
    }
}

// The 27 x 4 contributions of each lane summed over its segment in kRounds shuffle rounds (after round r a
// lane holds the sum of the next 2^r lanes of its segment); the segment's first lane adds each node's sums to
// the grid. kRounds is fixed per warp, so the rounds carry no per-node branches.
template <int kRounds>
__device__ __forceinline__ void p2g_segment_sums(float4* grid, const P2gTerms& t, bool valid, bool leader, int tail,
                                                 const StencilIndex& at) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float val[4] = {0.f, 0.f, 0.f, 0.f};
                if (valid) p2g_node(t, i, j, k, val);
#pragma unroll
                for (int r = 0; r < kRounds; ++r) {
                    const int d = 1 << r;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float o = __shfl_down_sync(0xffffffffu, val[c], d);
                        if (d <= tail) val[c] += o;
                    }
                }
                if (leader) grid_add(&grid[at(i, j, k)], val[0], val[1], val[2], val[3]);
            }
}


// The segment sums of p2g_segment_sums, then merged along z between the leaders of one x-y column: stencils
// whose bases differ by one or two nodes in z share nodes, and each shared node is added to the grid once,
// by the leader with the larger base, which takes the earlier leaders' sums for it by shuffles (three
// values per (i, j) node column instead of one reduction per node and leader). In the particle orders used
// here (the sampler's z-ascending columns, the reorder's z-fastest node order) runs of consecutive
// particles climb in z, so most of a warp's leaders chain this way. A leader writes node (i, j, k) unless
// the next leader's base is within k (that leader covers it); it adds the previous leader's sum for
// (i, j, k + d1) and, when the one before sits at distance 2, its sum for (i, j, 2) to node k = 0.
template <int kRounds>
__device__ __forceinline__ void p2g_column_sums(float4* grid, const P2gTerms& t, bool valid, bool leader, int tail,
                                                const StencilIndex& at, const ColumnMerge& m) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float v[3][4];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
#pragma unroll
                for (int c = 0; c < 4; ++c) v[k][c] = 0.f;
                if (valid) p2g_node(t, i, j, k, v[k]);
#pragma unroll
                for (int r = 0; r < kRounds; ++r) {
                    const int d = 1 << r;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float o = __shfl_down_sync(0xffffffffu, v[k][c], d);
                        if (d <= tail) v[k][c] += o;
                    }
                }
            }
            float o0[4], o1[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float a1 = __shfl_sync(0xffffffffu, v[1][c], m.src1);  // previous leader, k = 1
                const float a2 = __shfl_sync(0xffffffffu, v[2][c], m.src1);  // previous leader, k = 2
                const float b2 = __shfl_sync(0xffffffffu, v[2][c], m.src2);  // the one before, k = 2
                o0[c] = v[0][c] + (m.d1 == 1 ? a1 : (m.d1 == 2 ? a2 : 0.f)) + (m.ok2 ? b2 : 0.f);
                o1[c] = v[1][c] + (m.d1 == 1 ? a2 : 0.f);
            }
            if (leader) {
                grid_add(&grid[at(i, j, 0)], o0[0], o0[1], o0[2], o0[3]);
                if (m.ws != 1) grid_add(&grid[at(i, j, 1)], o1[0], o1[1], o1[2], o1[3]);
                if (m.ws == 0) grid_add(&grid[at(i, j, 2)], v[2][0], v[2][1], v[2][2], v[2][3]);
            }
        }
}

// P2G with warp-level aggregation: lanes whose stencils start at the same grid node (neighbours in the
// particle order after the reorder by grid node) form a segment; each of the 27 x 4 contributions is summed
// over the segment with shuffles (after round r a lane holds the sum of the next 2^r lanes of its segment)
// and only the segment's first lane issues the 16-byte reduction, so a cell of ~8 particles costs one
// reduction per node instead of eight. Runs are also cut at aligned groups of p2g_group lanes: fewer shuffle
// rounds for more reductions (the autotuner picks the group). Lanes past the end or with a stencil outside
// the grid are single-lane segments that add nothing. The segment's first lane lists the blocks it touches.
// grid / parity: the grid and the active list scattered into. All 32 lanes of the warp take part.
// kMaybeFixed = false: a build for scenes outside deterministic mode, without the fixed-point path (in line,
// though not taken, it cost the float path registers: 328 against 112 bytes of spill loads). kSweep: 0 the
// leaders list the blocks (no block-sweep code), 1 they only flag them (a.block_sweep set), 2 either, by
// a.block_sweep (the block-sweep branch in line cost another 112 -> 36 bytes of spill loads). kMerge: the
// float sums merged along z between leaders (p2g_column_sums).
template <bool kMaybeFixed = true, int kSweep = 2, bool kMerge = false>
__device__ __forceinline__ void p2g_warp_segments(const SubstepArgs& a, float4* grid, unsigned int parity,
                                                  const P2gTerms& t, bool valid) {
    const int lane = (int)(threadIdx.x & 31u);
    const GridDesc& g = a.g;
    const int64_t key = valid ? node_index(g, t.base[0], t.base[1], t.base[2]) : -1 - (int64_t)lane;
    const int64_t key_prev = __shfl_up_sync(0xffffffffu, key, 1);
    const int64_t key_next = __shfl_down_sync(0xffffffffu, key, 1);
    const int gmask = a.p2g_group - 1;  // runs are also cut at group boundaries
    const bool seg_first = (lane & gmask) == 0 || key_prev != key;
    const bool seg_last = (lane & gmask) == gmask || key_next != key;
    const unsigned int ends = __ballot_sync(0xffffffffu, seg_last);
    const int tail = __ffs(ends >> lane) - 1;  // lanes after this one in its segment
    const int span = (int)__reduce_max_sync(0xffffffffu, (unsigned int)tail);
    const bool leader = valid && seg_first;
    if (leader) {
        if (kSweep == 1 || (kSweep == 2 && a.block_sweep))
            flag_stencil_blocks(g, t.base, a.wl.block_flag);
        else
            mark_stencil_blocks(g, t.base, a.wl.block_flag, active_blocks(a.wl, parity), &a.wl.counts[parity]);
    }
    if constexpr (kMaybeFixed) {
        if (a.fixed) {
            p2g_fixed_warp(a, t, valid, leader, tail, span);
            return;
        }
    }
    const StencilIndex at = stencil_index(g, t.base);
    // shuffle rounds needed by the longest segment of the warp: 0, 1, 2, 3 or 5 (4 takes 5)
    const int rounds = span == 0 ? 0 : 32 - __clz(span);
    if constexpr (kMerge) {
        const ColumnMerge m = column_merge_of(t, valid, leader, lane);
        if (rounds == 0)
            p2g_column_sums<0>(grid, t, valid, leader, tail, at, m);
        else if (rounds == 1)
            p2g_column_sums<1>(grid, t, valid, leader, tail, at, m);
        else if (rounds == 2)
            p2g_column_sums<2>(grid, t, valid, leader, tail, at, m);
        else if (rounds == 3)
            p2g_column_sums<3>(grid, t, valid, leader, tail, at, m);
        else
            p2g_column_sums<5>(grid, t, valid, leader, tail, at, m);
        return;
    }
    if (rounds == 0)
        p2g_segment_sums<0>(grid, t, valid, leader, tail, at);
    else if (rounds == 1)
        p2g_segment_sums<1>(grid, t, valid, leader, tail, at);
    else if (rounds == 2)
        p2g_segment_sums<2>(grid, t, valid, leader, tail, at);
    else if (rounds == 3)
        p2g_segment_sums<3>(grid, t, valid, leader, tail, at);
    else
        p2g_segment_sums<5>(grid, t, valid, leader, tail, at);
}

// P2G of the 256 particles from `first` (one CTA's share; the warps past the end return).
template <bool kMaybeFixed = true, int kSweep = 2, bool kMerge = false>
__device__ __forceinline__ void p2g_cta(const SubstepArgs& a, int64_t first) {
    const int64_t p = first + threadIdx.x;
    if (first + (threadIdx.x & ~31u) >= a.n) return;  // whole warp past the end
    const Particles P = particles_of(a);
    P2gTerms t;
    const bool valid = p < a.n && p2g_terms(P, p, a.mats, a.g, a.sp->dt, t);
    const unsigned int cur = a.sp->seq & 1u;
    p2g_warp_segments<kMaybeFixed, kSweep, kMerge>(a, grid_of(a, cur), cur, t, valid);
}

// Chunks of 256 particles of a scene (the work items of the batched particle kernels).
__device__ __forceinline__ unsigned int particle_chunks(const SubstepArgs& a) {
    return (unsigned int)((a.n + 255) / 256);
}

// A batch's particle kernels walk the flattened (scene, chunk) list of the scenes that run this substep
// (scene_offsets over the chunk counts), grid-stride, so a scene that has finished its substeps for the
// frame costs no CTAs. One scene: one CTA per chunk, or with kWalk (the particles-per-thread launch choice)
// fewer CTAs that walk the chunks grid-stride. The walk is its own build: its loop costs the single-chunk
// kernels registers (G2P's spills grew from 152 to 252 bytes with it). kMaybeFixed = false: the build for a
// scene outside deterministic mode (a batch keeps the check per scene); kSweep, kMerge as in
// p2g_warp_segments.
// Four CTAs of 256 per SM (64 registers, no spills): with the z-merge's live values, five CTAs at 48
// registers spilled (488 bytes of loads) and ran P2G at 33.4-34.6 against 31.8 us (same box, alternating;
// substep 4.35-4.38e9 against 4.50e9). (Five CTAs had won by 2-3 % before the cold paths left the kernel.)
template <class Scenes, bool kWalk = false, bool kMaybeFixed = true, int kSweep = 2, bool kMerge = false>
__global__ void __launch_bounds__(256, 4) k_p2g_scatter(Scenes sc) {
    pdl_begin();
    if constexpr (!Scenes::kTable) {
        const SubstepArgs a = sc.get(0);
        if (a.sp->p2g_skip) return;
        if constexpr (kWalk) {
            const unsigned int chunks = particle_chunks(a);
#pragma unroll 1
            for (unsigned int q = blockIdx.x; q < chunks; q += gridDim.x)
                p2g_cta<kMaybeFixed, kSweep, kMerge>(a, (int64_t)q * blockDim.x);
        } else {
            p2g_cta<kMaybeFixed, kSweep, kMerge>(a, (int64_t)blockIdx.x * blockDim.x);
        }
    } else {
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total = scene_offsets(sc, [](const SubstepArgs& a) {
            return a.sp->p2g_skip ? 0u : particle_chunks(a);
        }, off);
#pragma unroll 1
        for (unsigned int q = blockIdx.x; q < total; q += gridDim.x) {
            const int s = scene_of_item(off, sc.count(), q);
            p2g_cta(sc.scenes[s], (int64_t)(q - off[s]) * blockDim.x);  // the table entry in place
        }
    }
}

// P2G through shared-memory tiles. The CTA's 256 particles (a contiguous range of the particle order) are
// taken with a stride of 8 inside the range (lane l of warp w takes particle 8 l + w), so the lanes of a warp
// sit in different cells whether the order is by cell (about 8 particles per cell) or the sampler's lattice
// order. The CTA's stencils are bounded by a box of nodes; when it holds at most kP2gTileNodes nodes, each
// warp adds its lanes' contributions into its own copy of the box with plain shared-memory read-add-writes
// (no atomics): at one stencil offset, lanes with different stencil bases write different nodes, and lanes
// that share a base take turns (rounds by their rank among the lanes with that base), with __syncwarp
// ordering each step. The warps' copies are then summed per node and every node that received anything is
// added to the grid with one 16-byte reduction (its grid block listed): a few reductions per box node
// instead of ~4.7 per particle, and no shuffle sums. A CTA whose box is larger (scattered particles) or a
// deterministic-mode scene takes the warp-segment path.
constexpr int kP2gTileNodes = 432;  // per warp: 8 copies x 432 nodes x 16 B = 55,296 B of shared memory
constexpr size_t kP2gTileBytes = (size_t)8 * kP2gTileNodes * sizeof(float4);

template <class Scenes>
__global__ void __launch_bounds__(256) k_p2g_tile(Scenes sc) {
    pdl_begin();
    extern __shared__ float4 tiles[];  // 8 warp copies of the box, node-major, `nodes` apart
    __shared__ int box[6];             // min x, y, z and max x, y, z of the stencil bases
    const int s = sc.scene_of_cta(blockIdx.x);
    const SubstepArgs a = sc.get(s);
    if (!sc.active(a) || a.sp->p2g_skip) return;
    const int64_t first = (int64_t)(blockIdx.x - sc.first_cta(s)) * blockDim.x;
    if (first >= a.n) return;  // CTA-uniform
    const int tid = (int)threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t p = first + lane * 8 + warp;
    const GridDesc& g = a.g;
    const Particles P = particles_of(a);
    P2gTerms t;
    const bool valid = p < a.n && p2g_terms(P, p, a.mats, g, a.sp->dt, t);
    if (tid < 6) box[tid] = tid < 3 ? INT_MAX : INT_MIN;
    __syncthreads();
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int lo = __reduce_min_sync(0xffffffffu, valid ? t.base[d] : INT_MAX);
        const int hi = __reduce_max_sync(0xffffffffu, valid ? t.base[d] : INT_MIN);
        if (lane == 0 && lo <= hi) {
            atomicMin(&box[d], lo);
            atomicMax(&box[3 + d], hi);
        }
    }
    __syncthreads();
    const int lo0 = box[0], lo1 = box[1], lo2 = box[2];
    if (lo0 > box[3]) return;  // no particle of the CTA scatters (CTA-uniform)
    const int e1 = box[4] - lo1 + 3, e2 = box[5] - lo2 + 3;
    const int nodes = (box[3] - lo0 + 3) * e1 * e2;
    const unsigned int cur = a.sp->seq & 1u;
    float4* grid = grid_of(a, cur);
    if (a.fixed || nodes > kP2gTileNodes) {  // CTA-uniform
        p2g_warp_segments(a, grid, cur, t, valid);
        return;
    }
    for (int q = tid; q < 8 * nodes; q += 256) tiles[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int o = valid ? ((t.base[0] - lo0) * e1 + (t.base[1] - lo1)) * e2 + (t.base[2] - lo2) : 0;
    const unsigned int peers = __match_any_sync(0xffffffffu, valid ? o : -1 - lane);
    const int rank = __popc(peers & ((1u << lane) - 1u));  // lanes before this one with the same base
    const int rounds = (int)__reduce_max_sync(0xffffffffu, (unsigned int)rank) + 1;
    float4* mine = tiles + warp * nodes;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float val[4] = {0.f, 0.f, 0.f, 0.f};
                if (valid) p2g_node(t, i, j, k, val);
                float4* cell = mine + o + (i * e1 + j) * e2 + k;
                for (int r = 0; r < rounds; ++r) {  // warp-uniform; one round unless lanes share a base
                    if (valid && rank == r) {
                        float4 c = *cell;
                        c.x += val[0];
                        c.y += val[1];
                        c.z += val[2];
                        c.w += val[3];
                        *cell = c;
                    }
                    __syncwarp();
                }
            }
    __syncthreads();
    for (int q = tid; q < nodes; q += 256) {
        float4 v = tiles[q];
#pragma unroll
        for (int w = 1; w < 8; ++w) {
            const float4 u = tiles[w * nodes + q];
            v.x += u.x;
            v.y += u.y;
            v.z += u.z;
            v.w += u.w;
        }
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {  // true for NaN too
            const int qk = q % e2, qij = q / e2;
            const int64_t node = node_index(g, lo0 + qij / e1, lo1 + qij % e1, lo2 + qk);
            grid_add(&grid[node], v.x, v.y, v.z, v.w);
            mark_block(node >> 6, a.wl.block_flag, active_blocks(a.wl, cur), &a.wl.counts[cur]);
        }
    }
}

// The active-block list of this substep from the block flags P2G set with plain stores (one scene, one grid,
// SubstepArgs::block_sweep): a sweep over every block's flag, one warp-aggregated append per warp.
template <class Scenes>
__global__ void __launch_bounds__(256) k_list_blocks(Scenes sc) {
    pdl_begin();
    const SubstepArgs a = sc.get(0);
    const unsigned int cur = a.sp->seq & 1u;
    const int64_t nblk = (int64_t)a.g.nb[0] * a.g.nb[1] * a.g.nb[2];
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk; b += (int64_t)gridDim.x * blockDim.x)
        if (a.wl.block_flag[b]) warp_append(active_blocks(a.wl, cur), &a.wl.counts[cur], (int32_t)b);
}

// Grid update (normalise, gravity, walls) over the active blocks, four 4x4x4 blocks per 256-thread CTA;
// nodes with mass inside some collider's margin box are listed for k_grid_colliders.
__device__ __forceinline__ void grid_update_block(const SubstepArgs& a, unsigned int i) {
    const GridDesc& g = a.g;
    const unsigned int cur = a.sp->seq & 1u;
    const int l = threadIdx.x & 63;
    const int64_t b = active_blocks(a.wl, cur)[i];
    const int bk = (int)(b % g.nb[2]);
    const int bj = (int)((b / g.nb[2]) % g.nb[1]);
    const int bi = (int)(b / ((int64_t)g.nb[2] * g.nb[1]));
    const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
    float4* grid = grid_of(a, cur);
    if (a.grid2 && l == 0) a.wl.block_flag[b] = 0u;  // two-grid mode: this substep's G2P lists blocks anew
    if (a.fixed) {  // deterministic mode: the node's fixed-point sums become its float momentum and mass
        const int64_t q = b * 64 + l;
        const ulonglong2 f01 = reinterpret_cast<const ulonglong2*>(a.fixed)[2 * q];
        const ulonglong2 f23 = reinterpret_cast<const ulonglong2*>(a.fixed)[2 * q + 1];
        const double inv = ldexp(1.0, -a.fixed_exp);
        float4 v = make_float4((float)((double)(long long)f01.x * inv), (float)((double)(long long)f01.y * inv),
                               (float)((double)(long long)f23.x * inv), (float)((double)(long long)f23.y * inv));
        if (a.poison[q]) v = make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                         __int_as_float(0x7fc00000), v.w);
        grid[q] = v;
    }
    bool has_mass = grid_node_walls(g, &grid[b * 64 + l], idx, a.sp->dt);
    if (has_mass && a.cd.n_col > 0) {
        ColliderData cd = a.cd;
        cd.poses += a.sp->pose_base;
        float pos[3];
        node_position(g, idx, pos);
        if (near_any_collider(pos, cd)) warp_append(a.wl.node_cand, &a.wl.counts[2], (int32_t)(b * 64 + l));
    }
}

template <class Scenes>
__global__ void __launch_bounds__(256) k_grid_update(Scenes sc) {
    pdl_begin();
    if constexpr (!Scenes::kTable) {
        const SubstepArgs a = sc.get(0);
        const unsigned int n = a.wl.counts[a.sp->seq & 1u];
        // two-grid mode: the list G2P fills (its blocks were cleared by this substep's clear kernel)
        if (a.grid2 && blockIdx.x == 0 && threadIdx.x == 0) a.wl.counts[(a.sp->seq + 1u) & 1u] = 0u;
        for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += gridDim.x * 4u)
            grid_update_block(a, i);
    } else {  // (a batch runs its scenes in one-grid mode)
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total =
            scene_offsets(sc, [](const SubstepArgs& a) { return a.wl.counts[a.sp->seq & 1u]; }, off);
        for (unsigned int q = blockIdx.x * 4u + (threadIdx.x >> 6); q < total; q += gridDim.x * 4u) {
            const int s = scene_of_item(off, sc.count(), q);
            grid_update_block(sc.get(s), q - off[s]);
        }
    }
}

// Contact work lists run in one of two shapes, chosen per launch from the list's length (identical
// results): up to warp_shape_items() items, one warp per item, whose lanes share the item's mesh queries
// (32 candidate triangles at a time), so a few slow queries do not hold up the kernel; beyond that, one
// thread per item, for throughput when contact is widespread. The bound is 128 items per SM of the device,
// not a share of the launch: tied to the launch, a tuned 16 work-list CTAs per SM kept the 256^3 pour's
// widespread contact in the warp shape (grid slot 0.15 -> 0.37 ms per substep, measured).
__device__ __forceinline__ unsigned int warp_shape_items() {
    unsigned int sms;
    asm("mov.u32 %0, %%nsmid;" : "=r"(sms));
    return 128u * sms;
}

// Rank of this warp among the launch's warps for the one-warp-per-item shape, CTA-major: warp 0 of every
// CTA first, then warp 1, ... A short list (a few hundred items) then lands one query warp per CTA, spread
// over all SMs, instead of four to a CTA on the first SMs, where the queries' FP64 evaluations of the winning
// face shared an SM's FP64 pipe (1/64 of the FP32 rate) and made the slowest SM the kernel's length.
__device__ __forceinline__ unsigned int contact_warp_rank() {
    return (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
}

// Mesh-collider contact of one listed node.
template <bool kWarp>
__device__ __forceinline__ void grid_collider_node(const SubstepArgs& a, unsigned int i) {
    const GridDesc& g = a.g;
    ColliderData cd = a.cd;
    cd.poses += a.sp->pose_base;
    const int64_t q = a.wl.node_cand[i];
    const int64_t b = q >> 6;
    const int l = (int)(q & 63);
    const int bk = (int)(b % g.nb[2]);
    const int bj = (int)((b / g.nb[2]) % g.nb[1]);
    const int bi = (int)(b / ((int64_t)g.nb[2] * g.nb[1]));
    const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
    grid_node_colliders<kWarp>(g, &grid_of(a, a.sp->seq & 1u)[q], idx, cd);
}

template <class Scenes>
__global__ void __launch_bounds__(128) k_grid_colliders(Scenes sc) {
    pdl_begin();
    const unsigned int tid = blockIdx.x * blockDim.x + threadIdx.x, threads = gridDim.x * blockDim.x;
    const unsigned int warp = contact_warp_rank(), warps = threads >> 5;
    if constexpr (!Scenes::kTable) {
        const SubstepArgs a = sc.get(0);
        const unsigned int n = a.wl.counts[2];
        if (n <= warp_shape_items()) {
            for (unsigned int i = warp; i < n; i += warps) grid_collider_node<true>(a, i);
        } else {
            for (unsigned int i = tid; i < n; i += threads) grid_collider_node<false>(a, i);
        }
    } else {
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total = scene_offsets(sc, [](const SubstepArgs& a) {
            return a.cd.n_col > 0 ? a.wl.counts[2] : 0u;
        }, off);
        if (total <= warp_shape_items()) {
            for (unsigned int q = warp; q < total; q += warps) {
                const int s = scene_of_item(off, sc.count(), q);
                grid_collider_node<true>(sc.get(s), q - off[s]);
            }
        } else {
            for (unsigned int q = tid; q < total; q += threads) {
                const int s = scene_of_item(off, sc.count(), q);
                grid_collider_node<false>(sc.get(s), q - off[s]);
            }
        }
    }
}

// G2P; particles that end inside a collider's margin box are listed for k_project_particles. kMinCtas = 4
// caps it at 64 registers (4 CTAs of 256 per SM): the kernel is bound by instruction latency, and the extra
// resident warps outweigh the spilled values (112 bytes) on the mixed workload (substep 1.2 % faster than at
// 80 registers, 3 CTAs; kernel 5 % faster under ncu; measured on a GB300). While the FP64 SVD fallback was
// in line, 80 registers was the best cap (10 % faster than kMinCtas = 1; 64 and 128 slower). The 80- and
// uncapped builds are kept; the autotuner picks one per workload. kFp64Clamp: the build with the FP64 redo at the
// Drucker-Prager and snow clamp (MPM_OPT_FP64_CLAMP), launched only when a scene has the option set.
// kScatter: the two-grid build. Where the substep scatters (StepParams::scatter), each warp then adds its
// particles to the next substep's grid, as k_p2g_scatter would at the start of that substep, from the
// values just computed (x, v and C read back from L2, the stress from registers): P2G without reading the
// particle state from memory again. Particles listed for the projection kernel are left to it (it scatters
// them once projected).
template <bool kFp64Clamp = false, class Source = GlobalSource, bool kScatter = false>
__device__ __forceinline__ void g2p_cta(const SubstepArgs& a, int64_t first) {
    const int64_t p = first + threadIdx.x;
    const unsigned int cur = a.sp->seq & 1u;
    if constexpr (!kScatter) {
        if (p >= a.n) return;
        float nx[3];
        g2p_particle<kFp64Clamp, Source>(particles_of(a), p, a.mats, a.g, a.sp->dt, grid_of(a, cur), a.fp64, nx,
                                         a.fp64_clamp, nullptr, a.fp64_redo);
        if (a.cd.n_col > 0) {
            ColliderData cd = a.cd;
            cd.poses += a.sp->pose_base;
            if (near_any_collider(nx, cd)) warp_append(a.wl.part_cand, &a.wl.counts[3], (int32_t)p);
        }
    } else {
        if (first + (threadIdx.x & ~31u) >= a.n) return;  // whole warp past the end; the others stay whole
        const Particles P = particles_of(a);
        const bool live = p < a.n;
        float nx[3], tau[6];
        bool listed = false;
        if (live) {
            g2p_particle<kFp64Clamp, Source>(P, p, a.mats, a.g, a.sp->dt, grid_of(a, cur), a.fp64, nx,
                                             a.fp64_clamp, tau, a.fp64_redo);
            if (a.cd.n_col > 0) {
                ColliderData cd = a.cd;
                cd.poses += a.sp->pose_base;
                listed = near_any_collider(nx, cd);
                if (listed) warp_append(a.wl.part_cand, &a.wl.counts[3], (int32_t)p);
            }
        }
        if (a.sp->scatter) {  // the same for the whole scene
            P2gTerms t;
            const bool valid = live && !listed && p2g_terms_of(ScatterFields{P, p, tau}, a.mats, a.g, a.sp->dt, t);
            const unsigned int next = cur ^ 1u;
            p2g_warp_segments<false, 0>(a, grid_of(a, next), next, t, valid);  // two grids: no fixed point, no sweep
        }
    }
}

template <class Scenes, int kMinCtas, bool kFp64Clamp = false, bool kScatter = false, bool kWalk = false>
__global__ void __launch_bounds__(256, kMinCtas) k_g2p(Scenes sc) {
    pdl_begin();
    if constexpr (!Scenes::kTable) {
        if constexpr (kWalk) {  // the chunks grid-stride, as in k_p2g_scatter
            const unsigned int chunks = particle_chunks(sc.a);
#pragma unroll 1
            for (unsigned int q = blockIdx.x; q < chunks; q += gridDim.x)
                g2p_cta<kFp64Clamp, GlobalSource, kScatter>(sc.get(0), (int64_t)q * blockDim.x);
        } else {
            g2p_cta<kFp64Clamp, GlobalSource, kScatter>(sc.get(0), (int64_t)blockIdx.x * blockDim.x);
        }
    } else {  // (scene, chunk) list of the running scenes, as in k_p2g_scatter
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total = scene_offsets(sc, [](const SubstepArgs& a) { return particle_chunks(a); }, off);
#pragma unroll 1
        for (unsigned int q = blockIdx.x; q < total; q += gridDim.x) {
            const int s = scene_of_item(off, sc.count(), q);
            // the scene's entry is read in place from the table (a copy of the whole record would be spilled)
            g2p_cta<kFp64Clamp, GlobalSource, kScatter>(sc.scenes[s], (int64_t)(q - off[s]) * blockDim.x);
        }
    }
}

// Projection of one listed particle (the same two shapes as for the nodes); where the substep scatters for
// the next one (two-grid mode), the lane that stored the particle then adds it to the next substep's grid.
template <bool kWarp>
__device__ __forceinline__ void project_candidate(const SubstepArgs& a, unsigned int i) {
    ColliderData cd = a.cd;
    cd.poses += a.sp->pose_base;
    const Particles P = particles_of(a);
    const int64_t p = a.wl.part_cand[i];
    project_particle<kWarp>(P, p, a.g, cd);
    if (a.sp->scatter && stores_result<kWarp>()) {
        const unsigned int next = (a.sp->seq + 1u) & 1u;
        p2g_particle(P, p, a.mats, a.g, a.sp->dt, grid_of(a, next), a.wl.block_flag, active_blocks(a.wl, next),
                     &a.wl.counts[next]);
    }
}

template <class Scenes>
__global__ void __launch_bounds__(128) k_project_particles(Scenes sc) {
    pdl_begin();
    const unsigned int tid = blockIdx.x * blockDim.x + threadIdx.x, threads = gridDim.x * blockDim.x;
    const unsigned int warp = contact_warp_rank(), warps = threads >> 5;
    if constexpr (!Scenes::kTable) {
        const SubstepArgs a = sc.get(0);
        const unsigned int n = a.wl.counts[3];
        if (n <= warp_shape_items()) {
            for (unsigned int i = warp; i < n; i += warps) project_candidate<true>(a, i);
        } else {
            for (unsigned int i = tid; i < n; i += threads) project_candidate<false>(a, i);
        }
    } else {
        __shared__ unsigned int off[kMaxBatchScenes + 1];
        const unsigned int total = scene_offsets(sc, [](const SubstepArgs& a) {
            return a.cd.n_col > 0 ? a.wl.counts[3] : 0u;
        }, off);
        if (total <= warp_shape_items()) {
            for (unsigned int q = warp; q < total; q += warps) {
                const int s = scene_of_item(off, sc.count(), q);
                project_candidate<true>(sc.get(s), q - off[s]);
            }
        } else {
            for (unsigned int q = tid; q < total; q += threads) {
                const int s = scene_of_item(off, sc.count(), q);
                project_candidate<false>(sc.get(s), q - off[s]);
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------------
// Several substeps of one scene in one cooperative launch: the phases of the kernels above, each over all
// CTAs of the grid, separated by grid-wide barriers. A small scene's substep is then one barrier per phase
// instead of one kernel launch per phase. Each CTA takes the same particle chunks in every phase; data
// written by other CTAs is read after a barrier (whose fences order it) through coherent loads: the G2P
// gather reads the grid from L2, never through the read-only path.
// ------------------------------------------------------------------------------------------------------
constexpr unsigned int kBarrierSpins = 1u << 22;  // polls of an L2 word: about a second

// Grid-wide barrier (bar[0] arrivals, bar[1] generation). A CTA that waits longer than kBarrierSpins sets
// *err and goes on; every CTA then leaves the kernel at its next barrier. Returns false once *err is set.
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, unsigned int* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vb = bar;
        const unsigned int gen = vb[1];
        __threadfence();
        if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            unsigned int spins = 0;
            while (vb[1] == gen) {
                if (++spins > kBarrierSpins) {
                    atomicOr(err, 1u);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile unsigned int*)err == 0u;
}

// reps substeps; bar: 2 barrier words and the error word, zeroed before the launch.
template <int kMinCtas>
__global__ void __launch_bounds__(256, kMinCtas) k_substeps_coop(OneScene sc, int reps, unsigned int* bar) {
    const SubstepArgs a = sc.get(0);
    unsigned int* err = bar + 2;
    const unsigned int ncta = gridDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x, threads = ncta * blockDim.x;
    const unsigned int warp = tid >> 5, warps = threads >> 5;
    const int64_t pctas = (a.n + 255) / 256;
    for (int r = 0; r < reps; ++r) {
        if (blockIdx.x == 0 && threadIdx.x == 0) step_begin(a.sp, a.wl.counts, a.cd.n_col, false);
        if (!grid_barrier(bar, err)) return;
        {
            const unsigned int prev = (a.sp->seq - 1u) & 1u;
            const unsigned int n = a.wl.counts[prev];
            for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += ncta * 4u)
                clear_block(a, prev, i);
        }
        if (!grid_barrier(bar, err)) return;
        for (int64_t c = blockIdx.x; c < pctas; c += ncta) p2g_cta(a, c * 256);
        if (!grid_barrier(bar, err)) return;
        {
            const unsigned int n = a.wl.counts[a.sp->seq & 1u];
            for (unsigned int i = blockIdx.x * 4u + (threadIdx.x >> 6); i < n; i += ncta * 4u)
                grid_update_block(a, i);
        }
        if (!grid_barrier(bar, err)) return;
        if (a.cd.n_col > 0) {
            const unsigned int n = a.wl.counts[2];
            if (n <= warp_shape_items()) {
                for (unsigned int i = warp; i < n; i += warps) grid_collider_node<true>(a, i);
            } else {
                for (unsigned int i = tid; i < n; i += threads) grid_collider_node<false>(a, i);
            }
            if (!grid_barrier(bar, err)) return;
        }
        for (int64_t c = blockIdx.x; c < pctas; c += ncta) g2p_cta<false, CoherentSource>(a, c * 256);
        if (!grid_barrier(bar, err)) return;
        if (a.cd.n_col > 0) {
            const unsigned int n = a.wl.counts[3];
            if (n <= warp_shape_items()) {
                for (unsigned int i = warp; i < n; i += warps) project_candidate<true>(a, i);
            } else {
                for (unsigned int i = tid; i < n; i += threads) project_candidate<false>(a, i);
            }
            if (!grid_barrier(bar, err)) return;
        }
    }
}

}  // namespace mpm
