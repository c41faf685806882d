// Plain structs shared by the host library and the kernels. FP32 device-side copies of the host's float64
// constants (the reference computes them in float64 and converts at launch, warp/solver.py:37-71).
#pragma once

#include <cstdint>

namespace mpm {

constexpr int kBlock = 4;       // grid block edge (nodes); a block is 64 nodes x 16 B = 1 KiB contiguous
constexpr int kPad = 3;         // padding cells around the domain, warp/solver.py:18
constexpr int kMaxMaterials = 64;

// Grid: dense padded node box, stored as 4x4x4 blocks; each node is float4 {momentum|velocity xyz, mass}.
struct GridDesc {
    int dims[3];   // padded node counts, warp/solver.py:40
    int nb[3];     // blocks per axis (dims rounded up to kBlock)
    float origin[3];
    float dx, inv_dx, p_vol;
    float gravity[3];
    int wall_lo_node[3], wall_hi_node[3], lo_on[3], hi_on[3];
    float wall_friction;
    float wall_lo[3], wall_hi[3], clamp_lo[3], clamp_hi[3];
    float thickness, band;  // open-collider thickness 2 dx and contact band dx
};

__host__ __device__ inline int64_t node_index(const GridDesc& g, int i, int j, int k) {
    int64_t b = ((int64_t)(i >> 2) * g.nb[1] + (j >> 2)) * g.nb[2] + (k >> 2);
    return b * 64 + (((i & 3) * 4 + (j & 3)) * 4 + (k & 3));
}

struct Material {
    int model;  // 0 elastic, 1 von Mises, 2 Drucker-Prager, 3 snow (kernels.py:8-13)
    float mu, lam, yield_stress, alpha, hardening, max_hardening;
    float clamp_lo, clamp_hi;  // snow: 1 - critical_compression, 1 + critical_stretch
    float p_mass;              // density * p_vol in FP32 (warp/solver.py:91)
};

// Particle state, structure of arrays; every component is its own array of `cap` entries.
// Words per particle in the arena: x3 v3 C9 F9 Jp tau6 mat emitter id Vq4, one plane of `cap` words each.
constexpr int kParticleFields = 38;

struct Particles {
    float* x[3];
    float* v[3];
    float* C[9];  // row-major APIC affine matrix
    float* F[9];  // row-major deformation gradient
    float* Jp;
    float* tau[6];  // Kirchhoff stress xx yy zz xy xz yz, from F and Jp (set by G2P and when particles enter)
    int32_t* mat;
    int32_t* emitter;
    int32_t* id;  // insertion rank: the reference's particle order, restored on every download
    // The right singular vectors of the particle's last SVD as a unit quaternion (x, y, z, w): the next
    // substep's SVD starts from them (set by G2P and when particles enter; null: every SVD starts cold)
    float* Vq[4];
    int64_t n, cap;
};

struct BvhNode {  // 32 B; internal: children at start, start+1 (count == 0); leaf: count triangles at start
    float lo[3];
    int start;
    float hi[3];
    int count;
};

struct MeshTri {  // 128 B, leaf order
    float a[3], b[3], c[3];
    int face;       // index in the collider's own triangle list (tie-break of equal distances)
    float fn[3];    // unit face normal
    float en[3][3]; // edge pseudonormals ab, bc, ca
    float vn[3][3]; // vertex pseudonormals a, b, c
    float pad[1];
};

// Narrow-band voxel grid of one collider in its local space (see mpm_device.cuh).
struct SdfGridDev {
    float lo[3], h;       // corner and voxel edge, local units
    int dims[3];
    int built;            // 0: not built, queries use the BVH
    int64_t cell_offset;  // first cell of this collider in the shared cell array
    float cutoff;         // local distance beyond which an outside point cannot reach the contact band
    float thick;          // local distance beyond which a point behind an open mesh is outside it
    float margin;         // margin of the bounding box the grid covers
};

// Per collider: static data and the pose pair of the current advance.
struct ColliderDev {
    SdfGridDev sdf;
    float aabb_lo[3], aabb_hi[3];
    float margin, friction;
    float mesh_scale;  // largest |coordinate| of the mesh's local bounding box
    int closed;
    int node_offset, tri_offset, n_tris;
    // pose pair of the current advance: translation, quaternion (x, y, z, w), symmetric stretch
    float t0[3], t1[3], q0[4], q1[4], S0[9], S1[9];
};

// A collider's pose at one substep: world transform, its inverse, and d(transform)/dt for the velocity.
struct ColliderPose {
    float M[3][4], Minv[3][4], dM[3][4];
};

// Everything a collider query needs, as device pointers.
struct ColliderData {
    const ColliderDev* cols;
    const ColliderPose* poses;  // of the current substep (already offset)
    int n_col;
    const BvhNode* nodes;
    const MeshTri* tris;
    const int2* cells;      // narrow-band voxel grids (may be null)
    const int32_t* cand;    // their candidate lists
};

// Values a substep reads from device memory, so one captured graph of a substep replays for all of them.
struct StepParams {
    float dt;
    float s;             // fraction of the advance at the end of this substep, (k + 1) / steps
    float inv_frame_dt;  // 1 / duration of the current advance call
    int k, steps;        // substep index within the advance; steps == 0 for a single explicit substep
    // Two-grid mode, single explicit substeps (set by the host with the fields above):
    int skip_first;      // 1: this substep's grid already holds the scatter of the G2P before it (same dt)
    int speculate;       // 1: this substep's G2P scatters for a next explicit substep with the same dt
    unsigned int seq;    // substeps run so far on this handle (selects the active-block list in use)
    int pose_base;       // first pose of this substep in the pose array
    int active;          // 1 while this scene has a substep to run (a batch idles scenes whose advance is done)
    // Two-grid mode, set per substep by the step-begin kernel:
    int p2g_skip;        // 1: the G2P before this substep scattered into this substep's grid; P2G does nothing
    int scatter;         // 1: this substep's G2P (and projection) scatter into the next substep's grid
};

// Work lists the substep builds on the device. Active blocks are the 4x4x4 grid blocks P2G touched;
// there are two lists, used by alternate substeps, so a substep can clear the blocks of the one before.
struct WorkLists {
    unsigned int* block_flag;   // one per grid block: 1 while the block is in the current list
    int32_t* blocks[2];         // active block ids
    unsigned int* counts;       // [0], [1]: active block counts; [2]: collider node candidates;
                                // [3]: collider particle candidates
    int32_t* node_cand;         // grid nodes (blocked index) inside some collider's margin box
    int32_t* part_cand;         // particles inside some collider's margin box after G2P
};

// The active-block list of parity `cur`, selected without indexing the struct's array (a dynamic index into
// a kernel parameter's array makes the compiler copy the whole struct to local memory).
__host__ __device__ __forceinline__ int32_t* active_blocks(const WorkLists& wl, unsigned int cur) {
    return cur ? wl.blocks[1] : wl.blocks[0];
}

// Periodic reorder of the particle arena by grid node: key = blocked index of the stencil's base node (or
// the node count for stencils outside the grid), a counting sort by key, then a permutation of every field.
struct SortScratch {
    int32_t* key;        // per particle
    int32_t* rank;       // per particle: arrival order within its key
    int32_t* order;      // per particle: the particle that goes to position i
    unsigned int* count; // per key (grid nodes + 1)
    int32_t* start;      // per key: exclusive prefix sum of count
};

// Most scenes a batch holds (the kernels over work lists keep one count per scene in shared memory).
constexpr int kMaxBatchScenes = 1024;

// Everything one substep's kernels read for one scene; the pointers stay fixed while a captured graph is
// replayed (a batch keeps one per scene in a device table).
struct SubstepArgs {
    float* arena;  // kParticleFields planes of cap words (particles_of gives the field pointers)
    int64_t cap, n;
    const Material* mats;
    GridDesc g;
    StepParams* sp;
    float4* grid;
    // Two-grid mode (null: one grid). Substeps alternate between grid (even seq) and grid2 (odd seq), so one
    // substep's G2P can gather from its own grid while it scatters each particle into the next substep's grid
    // (P2G fused into G2P: the particle state is not read again). Never set together with `fixed`.
    float4* grid2;
    unsigned int* fp64;
    WorkLists wl;
    ColliderData cd;  // poses: the start of the pose array; kernels add the substep's pose_base
    // Deterministic mode (null when off): P2G accumulates momentum xyz and mass of every node as 64-bit
    // fixed point in units of 2^-fixed_exp (integer sums are exact, so the result does not depend on the
    // order contributions arrive in); poison marks nodes that received a non-finite or out-of-range value.
    unsigned long long* fixed;
    unsigned int* poison;
    int fixed_exp;
    int p2g_group;  // P2G sums runs of same-base lanes within aligned groups of this many lanes (1 .. 32)
    int fp64_clamp;  // Drucker-Prager / snow return mapping redone in FP64 in G2P: 1 the lanes whose FP32
                     // decision was marginal, 2 every lane whose clamp was active, 0 none
    unsigned int* fp64_redo;  // count of the lanes redone in FP64
    unsigned int* err;  // set to nonzero by a kernel whose bounded wait gave up (the host reports it)
    int block_sweep;    // 1: P2G only flags the blocks it touches; k_list_blocks lists them afterwards
};

// The field pointers of a particle arena: plane f starts at arena + f * cap (x3 v3 C9 F9 Jp tau6 mat
// emitter id Vq4). Computed, not stored, so kernels that take a scene from a table keep two values live
// instead of 34 pointers.
__host__ __device__ __forceinline__ Particles make_particles(float* arena, int64_t cap, int64_t n) {
    Particles P;
    for (int a = 0; a < 3; ++a) P.x[a] = arena + (int64_t)a * cap;
    for (int a = 0; a < 3; ++a) P.v[a] = arena + (int64_t)(3 + a) * cap;
    for (int e = 0; e < 9; ++e) P.C[e] = arena + (int64_t)(6 + e) * cap;
    for (int e = 0; e < 9; ++e) P.F[e] = arena + (int64_t)(15 + e) * cap;
    P.Jp = arena + (int64_t)24 * cap;
    for (int e = 0; e < 6; ++e) P.tau[e] = arena + (int64_t)(25 + e) * cap;
    P.mat = reinterpret_cast<int32_t*>(arena + (int64_t)31 * cap);
    P.emitter = reinterpret_cast<int32_t*>(arena + (int64_t)32 * cap);
    P.id = reinterpret_cast<int32_t*>(arena + (int64_t)33 * cap);
    for (int e = 0; e < 4; ++e) P.Vq[e] = arena + (int64_t)(34 + e) * cap;
    P.n = n;
    P.cap = cap;
    return P;
}

__host__ __device__ __forceinline__ Particles particles_of(const SubstepArgs& a) {
    return make_particles(a.arena, a.cap, a.n);
}

// The grid of the substeps whose seq has this parity (the one grid outside two-grid mode).
__host__ __device__ __forceinline__ float4* grid_of(const SubstepArgs& a, unsigned int parity) {
    return (parity && a.grid2) ? a.grid2 : a.grid;
}

}  // namespace mpm
