// Host side of the C-ABI in include/mpm_gb300.h: device memory, host-side constants, collider BVHs and
// narrow-band voxel grids, the substep launch sequence (captured into CUDA graphs of one or eight substeps
// and replayed), CFL time stepping, the periodic reorder, removal of escaped particles, state I/O
// (synchronous and overlapped), deterministic mode, and batches of scenes.
//
// The host constants follow mpm_core/backends/warp/solver.py:37-71 in float64 and are rounded to FP32
// when stored for the kernels, as the reference's launches do.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpm_gb300.h"
#include "mpm_bvh.h"
#include "mpm_host.h"
#include "mpm_internal.h"

using namespace mpm;

namespace {

constexpr double kCFL = 0.4;  // warp/solver.py:19
constexpr int kFields = kParticleFields;    // x3 v3 C9 F9 Jp tau6 mat emitter id Vq4

thread_local std::string g_last_error;

struct Status {
    int code = MPM_OK;
    std::string msg;
};

// Instantiated substep graphs keyed by what the kernels' arguments depend on (and how many substeps one
// graph holds); four entries, so the two particle arenas the reorder alternates between, each with its
// many-substep and one-substep graph, all keep theirs.
struct GraphCache {
    static constexpr int kKey = 8, kSlots = 4;
    cudaGraphExec_t exec[kSlots] = {};
    int64_t key[kSlots][kKey] = {};
    int64_t used[kSlots] = {};
    int64_t tick = 0;
    cudaGraphExec_t find(const int64_t* k) {
        for (int i = 0; i < kSlots; ++i)
            if (exec[i] && std::memcmp(key[i], k, sizeof(int64_t) * kKey) == 0) {
                used[i] = ++tick;
                return exec[i];
            }
        return nullptr;
    }
    int victim() const {
        int v = 0;
        for (int i = 0; i < kSlots; ++i) {
            if (!exec[i]) return i;
            if (used[i] < used[v]) v = i;
        }
        return v;
    }
    void put(int i, const int64_t* k, cudaGraphExec_t g) {
        if (exec[i]) cudaGraphExecDestroy(exec[i]);
        exec[i] = g;
        std::memcpy(key[i], k, sizeof(int64_t) * kKey);
        used[i] = ++tick;
    }
    void clear() {
        for (auto& e : exec) {
            if (e) cudaGraphExecDestroy(e);
            e = nullptr;
        }
    }
};

struct Batch;

struct Handle {
    int device = 0;
    cudaStream_t stream = nullptr;      // the stream all work runs on: own_stream, or the batch's
    cudaStream_t own_stream = nullptr;
    Batch* batch = nullptr;             // the batch this scene belongs to, if any
    MpmDomainDesc dom{};
    HostDomain hd{};
    double dx = 0, inv_dx = 0, p_vol = 0;
    double origin[3] = {0, 0, 0};
    int dims[3] = {0, 0, 0};
    GridDesc g{};
    int ppc = 8;
    std::vector<MpmMaterialDesc> mat_desc;
    std::vector<double> wave;          // P-wave speed per material incl. worst-case snow hardening
    std::vector<int64_t> mat_count;    // particles per material ("present" materials)
    Material* d_mats = nullptr;

    Particles P{}, spare{};
    void* arena = nullptr;
    void* spare_arena = nullptr;

    float4* grid = nullptr;
    int64_t grid_nodes = 0;
    // Two-grid mode (MPM_OPT_FUSED_P2G): the second grid, and the state of the grids on the device
    float4* grid2 = nullptr;
    bool fused_p2g = false;    // the option
    bool two_live = false;     // the substeps so far ran in two-grid mode (lists and flags refer to both grids)
    bool pending = false;      // the last explicit substep scattered into the next one's grid, for dt pending_dt
    float pending_dt = 0.f;
    float* vol = nullptr;              // occupancy scratch, one float per node

    StepParams* d_sp = nullptr;
    unsigned int* d_counters = nullptr;  // [0] vmax bits, [1] fp64 lanes, [2..] removed per material
    unsigned int* h_counters = nullptr;  // pinned

    int n_col = 0;
    std::vector<ColliderDev> cols;
    ColliderDev* d_cols = nullptr;
    ColliderPose* d_poses = nullptr;  // poses of every substep of the current advance
    int64_t pose_cap = 0;
    // What d_poses holds: the (steps, s, 1 / frame_dt) of its last computation while pose_valid; cleared
    // when the colliders or their transforms change. A call with the same key reuses the poses.
    bool pose_valid = false;
    int pose_steps = 0;
    float pose_s = 0.f, pose_inv_fdt = 0.f;
    WorkLists wl{};                   // active blocks and collider candidates, sized for the grid / particles
    int64_t part_cand_cap = 0;
    int2* d_sdf_cells = nullptr;      // narrow-band voxel grids of all colliders
    int32_t* d_sdf_cand = nullptr;
    size_t sdf_bytes = 0, collider_bytes = 0;
    bool sdf_dirty = true;
    BvhNode* d_nodes = nullptr;
    MeshTri* d_tris = nullptr;
    double frame_dt = 1.0;

    // removal scratch
    int32_t* d_keep = nullptr;  // keep_phys | keep_by_id | dst_index | new_id, each cap entries
    int32_t* d_scan_tmp = nullptr;
    int64_t keep_cap = 0, scan_cap = 0;

    void* stage = nullptr;  // device staging for host-order arrays
    size_t stage_bytes = 0;

    // asynchronous read-back (mpm_read_begin / mpm_read_wait)
    void* rb_dev = nullptr;
    size_t rb_bytes = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t rb_ready = nullptr, rb_done = nullptr;
    bool rb_pending = false;

    int64_t launches = 0;       // kernels of this library launched so far (graph replays count their kernels)
    int64_t graph_kernels = 0;  // kernels in the captured substep graph

    SortScratch ss{};            // counting sort of the particles by grid node
    int64_t ss_cap = 0;          // particle capacity the per-particle sort arrays were sized for
    int32_t* ss_scan = nullptr;  // scan scratch over the grid's node counts
    int64_t ss_scan_cap = 0;
    int sort_interval = 4;       // reorder the particles by grid node after every this many substeps (0: never)
    int64_t since_sort = 0;

    LaunchShape shape;                      // autotuned launch choices
    int fp64_clamp = 0;                     // Drucker-Prager / snow return mapping redone in FP64 (0, 1, 2)
    bool deterministic = false;
    unsigned long long* d_fixed = nullptr;  // deterministic mode: fixed-point node sums (4 per node)
    unsigned int* d_poison = nullptr;       // deterministic mode: non-finite marks (1 per node)
    int fixed_exp = 0;

    bool use_graph = true;
    GraphCache graphs;           // the substep graph, one per particle arena (the reorder alternates two)
    int coop = 0;                // several substeps per cooperative launch: 0 never, 1 always, 2 small scenes
    unsigned int* d_coop = nullptr;  // its barrier words and error flag
    bool coop_used = false;      // a cooperative launch ran since the last check of its error flag

    int timing = 0;              // 1: events between the kernel groups; 2: events around each substep only
    cudaEvent_t tev[5] = {};     // event nodes of the timed graph
    GraphCache tgraphs;          // the substep graph with timing events
    GraphCache bgraphs;          // the substep graph with events at its two ends
    cudaEvent_t perm_ev[2] = {};
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::vector<cudaEvent_t>> ev_pending;  // per substep: 4 events around p2g / grid / g2p
    double t_ms[5] = {0, 0, 0, 0, 0};  // p2g, grid, g2p, other; [4]: whole substeps (timing 2)
    int64_t t_launches[5] = {0, 0, 0, 0, 0};

    std::string err;
};

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return Status{MPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

#define TRY(expr)                            \
    do {                                     \
        Status s_ = (expr);                  \
        if (s_.code != MPM_OK) return s_;    \
    } while (0)

int finish(Handle* h, Status s) {
    if (s.code != MPM_OK) {
        if (h) h->err = s.msg;
        g_last_error = s.msg;
    }
    return s.code;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur;
        if (cudaGetDevice(&cur) == cudaSuccess && prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// ---- particles -------------------------------------------------------------------------------------

Particles bind_arena(void* base, int64_t cap, int64_t n) {
    return make_particles(static_cast<float*>(base), cap, n);
}

void invalidate_graph(Handle* h) {
    h->graphs.clear();
    h->tgraphs.clear();
    h->bgraphs.clear();
}

Status ensure_capacity(Handle* h, int64_t need) {
    if (need <= h->P.cap) return {};
    // a multiple of 256 entries: every plane starts 1 KB-aligned
    int64_t cap = (std::max<int64_t>({need, 2 * h->P.cap, 4096}) + 255) / 256 * 256;
    void* fresh = nullptr;
    if (cudaMalloc(&fresh, (size_t)cap * kFields * 4) != cudaSuccess) {
        cudaGetLastError();
        return {MPM_ERR_MEMORY, "device allocation of particle storage failed"};
    }
    Particles np = bind_arena(fresh, cap, h->P.n);
    if (h->P.n > 0) {  // keep the live particles: copy each field's first n entries
        const float* src = static_cast<const float*>(h->arena);
        float* dst = static_cast<float*>(fresh);
        for (int f = 0; f < kFields; ++f)
            CK(cudaMemcpyAsync(dst + (int64_t)f * cap, src + (int64_t)f * h->P.cap, (size_t)h->P.n * 4,
                               cudaMemcpyDeviceToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    if (h->arena) cudaFree(h->arena);
    if (h->spare_arena) cudaFree(h->spare_arena);
    h->spare_arena = nullptr;
    h->arena = fresh;
    h->P = np;
    h->spare = Particles{};
    invalidate_graph(h);
    return {};
}

Status ensure_stage(Handle* h, size_t bytes) {
    if (bytes <= h->stage_bytes) return {};
    CK(cudaStreamSynchronize(h->stream));
    if (h->stage) cudaFree(h->stage);
    h->stage = nullptr;
    size_t b = std::max(bytes, h->stage_bytes * 2);
    if (cudaMalloc(&h->stage, b) != cudaSuccess) {
        cudaGetLastError();
        h->stage_bytes = 0;
        return {MPM_ERR_MEMORY, "device allocation of the staging buffer failed"};
    }
    h->stage_bytes = b;
    return {};
}

// Deterministic mode: fixed-point accumulators for every node, zeroed (the active-block clear keeps them
// zero afterwards), and the fixed-point exponent: 2^-e = 2^-40 of the heaviest particle's mass, so a node
// (at most 27 x 8 particles) stays far below 2^63 while one particle's contribution keeps ~40 bits.
Status set_deterministic(Handle* h, bool on) {
    if (on == h->deterministic) return {};
    CK(cudaStreamSynchronize(h->stream));
    invalidate_graph(h);
    if (on && !h->d_fixed) {
        if (cudaMalloc(&h->d_fixed, sizeof(unsigned long long) * 4 * (size_t)h->grid_nodes) != cudaSuccess ||
            cudaMalloc(&h->d_poison, sizeof(unsigned int) * (size_t)h->grid_nodes) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(h->d_fixed);
            h->d_fixed = nullptr;
            return {MPM_ERR_MEMORY, "device allocation of the deterministic-mode accumulators failed"};
        }
    }
    if (on) {
        CK(cudaMemsetAsync(h->d_fixed, 0, sizeof(unsigned long long) * 4 * (size_t)h->grid_nodes, h->stream));
        CK(cudaMemsetAsync(h->d_poison, 0, sizeof(unsigned int) * (size_t)h->grid_nodes, h->stream));
        double pm = 0.0;
        for (const auto& m : h->mat_desc) pm = std::max(pm, (double)(float)(m.density * h->p_vol));
        h->fixed_exp = std::clamp(40 - (int)std::ceil(std::log2(std::max(pm, 1e-30))), -60, 100);
        // the grid must start zero, as the float path leaves it: clear whatever the last substep touched
        CK(cudaMemsetAsync(h->grid, 0, (size_t)h->grid_nodes * sizeof(float4), h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    h->deterministic = on;
    return {};
}

Status prepare_grids(Handle* h, bool two, bool keep_pending);

// MPM_OPT_FUSED_P2G: the second grid is allocated on the way in and freed on the way out; the grids are
// brought into the new mode before the next substep (prepare_grids).
Status set_fused_p2g(Handle* h, bool on) {
    if (on == h->fused_p2g) return {};
    CK(cudaStreamSynchronize(h->stream));
    invalidate_graph(h);  // the second grid is a kernel argument of the captured graphs
    if (on && !h->grid2) {
        if (cudaMalloc(&h->grid2, (size_t)h->grid_nodes * sizeof(float4)) != cudaSuccess) {
            cudaGetLastError();
            h->grid2 = nullptr;
            return {MPM_ERR_MEMORY, "device allocation of the second grid failed"};
        }
        CK(cudaMemset(h->grid2, 0, (size_t)h->grid_nodes * sizeof(float4)));
    }
    h->fused_p2g = on;
    if (!on) {
        TRY(prepare_grids(h, false, false));  // before the second grid goes: nothing may refer to it
        CK(cudaStreamSynchronize(h->stream));
        cudaFree(h->grid2);
        h->grid2 = nullptr;
    }
    return {};
}

// Device memory the handle holds now (the allocations it made, by their sizes).
int64_t handle_device_bytes(const Handle* h) {
    const int64_t nblk = (int64_t)h->g.nb[0] * h->g.nb[1] * h->g.nb[2];
    int64_t b = (int64_t)h->P.cap * kFields * 4 * (h->spare_arena ? 2 : 1);
    b += h->grid_nodes * (h->grid2 ? 32 : 16) + (h->vol ? h->grid_nodes * 4 : 0) + (h->d_fixed ? h->grid_nodes * 36 : 0);
    b += nblk * 12 + h->grid_nodes * 4 + h->part_cand_cap * 4 + 16;                      // work lists
    b += h->ss_cap * 12 + (h->grid_nodes + 1) * 8 + (h->ss_scan_cap + 2) * 4;           // sort
    b += h->keep_cap * 16 + (h->scan_cap + 2) * 4;                                       // removal
    b += h->pose_cap * (int64_t)sizeof(ColliderPose) + (int64_t)h->collider_bytes + (int64_t)h->sdf_bytes;
    b += (int64_t)h->stage_bytes + (int64_t)sizeof(StepParams) + 4 * (2 + kMaxMaterials);
    b += (int64_t)sizeof(Material) * (int64_t)std::max<size_t>(1, h->mat_desc.size());
    return b;
}

// ---- substep sequence ---------------------------------------------------------------------------------

void free_colliders(Handle* h) {
    h->pose_valid = false;
    if (h->d_cols) cudaFree(h->d_cols);
    if (h->d_nodes) cudaFree(h->d_nodes);
    if (h->d_tris) cudaFree(h->d_tris);
    h->d_cols = nullptr;
    h->d_nodes = nullptr;
    h->d_tris = nullptr;
    h->collider_bytes = 0;
}

cudaEvent_t take_event(Handle* h) {
    if (!h->ev_pool.empty()) {
        cudaEvent_t e = h->ev_pool.back();
        h->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// Two-grid mode for this handle's next substeps: the option, and neither deterministic mode (fixed-point
// node sums) nor the FP64 clamp build (a G2P build of its own).
bool two_grids(const Handle* h) {
    return h->fused_p2g && h->grid2 && !h->deterministic && !h->fp64_clamp;
}

// Puts the grids into the state the next substeps expect. Nothing changes while the mode stays and a pending
// scatter is kept; otherwise both grids, the block flags and the active lists start empty (a scatter made
// for a substep that does not follow is dropped). Stream-ordered: no synchronisation.
Status prepare_grids(Handle* h, bool two, bool keep_pending) {
    if (two == h->two_live && (!h->pending || keep_pending)) return {};
    const int64_t nblk = (int64_t)h->g.nb[0] * h->g.nb[1] * h->g.nb[2];
    CK(cudaMemsetAsync(h->grid, 0, (size_t)h->grid_nodes * sizeof(float4), h->stream));
    if (h->grid2) CK(cudaMemsetAsync(h->grid2, 0, (size_t)h->grid_nodes * sizeof(float4), h->stream));
    CK(cudaMemsetAsync(h->wl.block_flag, 0, sizeof(unsigned int) * (size_t)nblk, h->stream));
    CK(cudaMemsetAsync(h->wl.counts, 0, sizeof(unsigned int) * 2, h->stream));
    h->two_live = two;
    h->pending = false;
    return {};
}

// Drops a scatter made for an explicit substep that may not follow (the particles are about to change).
// The kept scatter is valid only while the particle state, the materials and dt are what the previous
// explicit substep left: every entry point that changes particle state or materials (today add_particles and
// load_state; advance and run_substeps start from fresh grids through prepare_grids) must call this before
// the change, and so must any such entry point added later.
Status drop_pending(Handle* h) {
    return h->pending ? prepare_grids(h, h->two_live, false) : Status{};
}

SubstepArgs substep_args(Handle* h) {
    SubstepArgs a{};
    a.arena = static_cast<float*>(h->arena);
    a.cap = h->P.cap;
    a.n = h->P.n;
    a.mats = h->d_mats;
    a.g = h->g;
    a.sp = h->d_sp;
    a.grid = h->grid;
    a.grid2 = two_grids(h) ? h->grid2 : nullptr;
    a.fp64 = h->d_counters + 1;
    a.wl = h->wl;
    a.cd.cols = h->d_cols;
    a.cd.poses = h->d_poses;
    a.cd.n_col = h->n_col;
    a.cd.nodes = h->d_nodes;
    a.cd.tris = h->d_tris;
    a.cd.cells = h->d_sdf_cells;
    a.cd.cand = h->d_sdf_cand;
    a.fixed = h->deterministic ? h->d_fixed : nullptr;
    a.poison = h->deterministic ? h->d_poison : nullptr;
    a.fixed_exp = h->fixed_exp;
    a.p2g_group = h->shape.p2g_group;
    a.fp64_clamp = h->fp64_clamp;
    a.fp64_redo = h->d_counters + 2 + kMaxMaterials;
    a.err = h->d_coop + 3;
    a.block_sweep = h->shape.block_sweep && !two_grids(h) && !h->shape.p2g_tile ? 1 : 0;
    return a;
}

Status ensure_part_cand(Handle* h) {
    if (h->part_cand_cap >= h->P.cap) return {};
    CK(cudaStreamSynchronize(h->stream));
    if (h->wl.part_cand) cudaFree(h->wl.part_cand);
    h->wl.part_cand = nullptr;
    if (cudaMalloc(&h->wl.part_cand, sizeof(int32_t) * (size_t)h->P.cap) != cudaSuccess) {
        cudaGetLastError();
        h->part_cand_cap = 0;
        return {MPM_ERR_MEMORY, "device allocation of the collider candidate list failed"};
    }
    h->part_cand_cap = h->P.cap;
    invalidate_graph(h);
    return {};
}

// Per-particle sort arrays (key, rank, order), sized for the particle capacity.
Status ensure_sort_scratch(Handle* h) {
    if (h->ss_cap >= h->P.cap) return {};
    CK(cudaStreamSynchronize(h->stream));
    cudaFree(h->ss.key);
    h->ss.key = h->ss.rank = h->ss.order = nullptr;
    h->ss_cap = 0;
    const int64_t cap = h->P.cap;
    if (cudaMalloc(&h->ss.key, sizeof(int32_t) * 3 * (size_t)cap) != cudaSuccess) {
        cudaGetLastError();
        h->ss.key = nullptr;
        return {MPM_ERR_MEMORY, "device allocation of the particle sort arrays failed"};
    }
    h->ss.rank = h->ss.key + cap;
    h->ss.order = h->ss.key + 2 * cap;
    h->ss_cap = cap;
    return {};
}

// Reorders the particle arena by the grid node of each particle's stencil base (counting sort, then
// dst[i] = src[order[i]] for every field), so that neighbouring threads of the next substeps' P2G and G2P
// touch neighbouring grid nodes. Particle ids travel with the particles, so host order is unchanged.
Status reorder_particles(Handle* h) {
    if (h->P.n == 0) return {};
    TRY(ensure_sort_scratch(h));
    if (!h->spare_arena) {
        if (cudaMalloc(&h->spare_arena, (size_t)h->P.cap * kFields * 4) != cudaSuccess) {
            cudaGetLastError();
            h->spare_arena = nullptr;
            return {MPM_ERR_MEMORY, "device allocation of particle storage failed"};
        }
    }
    Particles dst = bind_arena(h->spare_arena, h->P.cap, h->P.n);
    if (h->timing) {
        if (!h->perm_ev[0])
            for (auto& e : h->perm_ev) CK(cudaEventCreate(&e));
        CK(cudaEventRecord(h->perm_ev[0], h->stream));
    }
    launch_sort(h->stream, h->P, h->g, h->ss, h->grid_nodes, h->ss_scan, h->ss_scan_cap);
    launch_permute(h->stream, h->arena, h->spare_arena, h->P.cap, h->P.n, h->ss.order);
    CK(cudaGetLastError());
    h->launches += 6;  // keys, three-pass scan, order, permutation
    if (h->timing) {
        CK(cudaEventRecord(h->perm_ev[1], h->stream));
        CK(cudaEventSynchronize(h->perm_ev[1]));
        float t = 0;
        cudaEventElapsedTime(&t, h->perm_ev[0], h->perm_ev[1]);
        h->t_ms[h->timing == 2 ? 4 : 3] += t;
    }
    std::swap(h->arena, h->spare_arena);
    h->P = dst;
    return {};
}

void accumulate_times(Handle* h, const cudaEvent_t* ev) {  // ev: | clear | P2G | grid + colliders | G2P + projection |
    const int slot_of[4] = {3, 0, 1, 2};
    for (int k = 0; k < 4; ++k) {
        float t = 0;
        cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
        h->t_ms[slot_of[k]] += t;
        h->t_launches[slot_of[k]] += 1;
    }
}

// reps substeps in one graph (the launch cost of one graph per reps substeps); events only with reps == 1.
Status capture_graph(Handle* h, const SubstepArgs& a, cudaEvent_t* ev, cudaGraphExec_t* out, int reps = 1) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int r = 0; r < reps; ++r) launch_substep(h->stream, a, h->shape, reps == 1 ? ev : nullptr, true);
    cudaError_t e0 = cudaGetLastError();
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    CK(e0);
    CK(e);
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    CK(e);
    return {};
}

// reps substeps (reps > 1 only with graphs and without kernel timing).
Status run_substep(Handle* h, int reps = 1) {
    TRY(ensure_part_cand(h));
    SubstepArgs a = substep_args(h);
    const int kernels = substep_kernel_count(a);
    h->launches += (int64_t)kernels * reps;
    int64_t key[GraphCache::kKey] = {h->P.n, h->P.cap, h->n_col, (int64_t)(intptr_t)h->arena,
                                     (int64_t)(intptr_t)h->d_poses, (int64_t)(intptr_t)h->wl.part_cand,
                                     (int64_t)h->shape.list_ctas,
                                     (((((((((int64_t)h->shape.g2p_variant * 64 + h->shape.p2g_group) * 2 + h->shape.pdl) *
                                                2 + (h->fp64_clamp ? 1 : 0)) * 2 + h->shape.p2g_tile) * 2 +
                                              (a.grid2 ? 1 : 0)) * 2 + a.block_sweep) * 16 + h->shape.ppt) * 2 +
                                            h->shape.p2g_merge) * 64 + reps};
    if (!h->use_graph) {
        if (h->timing) {
            std::vector<cudaEvent_t> ev(5);
            for (auto& e : ev) e = take_event(h);
            launch_substep(h->stream, a, h->shape, ev.data(), false);
            h->ev_pending.push_back(ev);
        } else {
            launch_substep(h->stream, a, h->shape, nullptr, false);
        }
        CK(cudaGetLastError());
        return {};
    }
    if (h->timing == 2) {  // events at the substep graph's two ends: the substep's device time, with the
                           // kernels inside chained as in the untimed graph
        if (!h->tev[0])
            for (auto& e : h->tev) CK(cudaEventCreate(&e));
        cudaGraphExec_t g = h->bgraphs.find(key);
        if (!g) {
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            cudaEventRecordWithFlags(h->tev[0], h->stream, cudaEventRecordExternal);
            launch_substep(h->stream, a, h->shape, nullptr, true);
            cudaEventRecordWithFlags(h->tev[4], h->stream, cudaEventRecordExternal);
            cudaError_t e0 = cudaGetLastError();
            cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
            CK(e0);
            CK(e);
            e = cudaGraphInstantiate(&g, graph, 0);
            cudaGraphDestroy(graph);
            CK(e);
            h->bgraphs.put(h->bgraphs.victim(), key, g);
        }
        CK(cudaGraphLaunch(g, h->stream));
        CK(cudaEventSynchronize(h->tev[4]));
        float t = 0;
        cudaEventElapsedTime(&t, h->tev[0], h->tev[4]);
        h->t_ms[4] += t;
        h->t_launches[4] += 1;
        return {};
    }
    if (h->timing) {  // the same graph with event nodes; read them before the next replay overwrites them
        if (!h->tev[0])
            for (auto& e : h->tev) CK(cudaEventCreate(&e));
        cudaGraphExec_t g = h->tgraphs.find(key);
        if (!g) {
            TRY(capture_graph(h, a, h->tev, &g));
            h->tgraphs.put(h->tgraphs.victim(), key, g);
        }
        CK(cudaGraphLaunch(g, h->stream));
        CK(cudaEventSynchronize(h->tev[4]));
        accumulate_times(h, h->tev);
        return {};
    }
    cudaGraphExec_t g = h->graphs.find(key);
    if (!g) {
        TRY(capture_graph(h, a, nullptr, &g, reps));
        h->graphs.put(h->graphs.victim(), key, g);
    }
    CK(cudaGraphLaunch(g, h->stream));
    return {};
}

// One substep, then the reorder into bin order when it is due.
Status substep_and_sort(Handle* h) {
    TRY(run_substep(h));
    if (h->sort_interval > 0 && ++h->since_sort >= h->sort_interval) {
        TRY(reorder_particles(h));
        h->since_sort = 0;
    }
    return {};
}

// count substeps, kGraphReps per graph launch where they fit between reorders (one launch per substep
// costs more host time than a small scene's substep takes on the GPU).
constexpr int kGraphReps = 8;

// Scenes up to this many particles take the cooperative launch in the automatic mode. Measured on a GB300,
// the cooperative launch is slower than the graph of separate kernels at every size tried (32k particles:
// 70 us against 30 us per substep; 295k: 187 against 67), so neither mode is the default.
constexpr int64_t kCoopAutoMaxParticles = 131072;
constexpr int kCoopMaxReps = 64;  // substeps per cooperative launch (a launch stays in the milliseconds)

bool coop_eligible(const Handle* h, int count) {
    if (h->coop == 0 || count < 2 || h->timing || !h->use_graph || h->fp64_clamp || h->shape.p2g_tile ||
        two_grids(h))
        return false;
    return h->coop == 1 || h->P.n <= kCoopAutoMaxParticles;
}

// reps substeps in one cooperative launch.
Status run_coop(Handle* h, int reps) {
    TRY(ensure_part_cand(h));
    SubstepArgs a = substep_args(h);
    a.grid2 = nullptr;  // one grid (coop_eligible excludes two-grid mode)
    a.block_sweep = 0;  // the cooperative kernel's P2G lists the blocks itself
    CK(launch_substeps_coop(h->stream, a, reps, h->d_coop));
    h->launches += 1;
    h->coop_used = true;
    return {};
}

// After a synchronisation: fails if a grid barrier of a cooperative launch gave up waiting.
Status check_coop(Handle* h) {
    unsigned int err[2] = {0u, 0u};
    if (!h->coop_used && h->shape.g2p_variant != 2) return {};
    CK(cudaMemcpy(err, h->d_coop + 2, sizeof(err), cudaMemcpyDeviceToHost));
    if (err[0] && h->coop_used) {
        h->coop_used = false;
        return {MPM_ERR_CUDA, "cooperative substeps: a grid barrier timed out"};
    }
    h->coop_used = false;
    if (err[1]) {
        CK(cudaMemset(h->d_coop + 3, 0, sizeof(unsigned int)));
        return {MPM_ERR_CUDA, "tile G2P: a wait for its TMA copies timed out"};
    }
    return {};
}

Status substeps_and_sort(Handle* h, int count) {
    while (count > 0) {
        if (coop_eligible(h, count)) {
            int reps = std::min(count, kCoopMaxReps);
            if (h->sort_interval > 0) reps = (int)std::min<int64_t>(reps, h->sort_interval - h->since_sort);
            reps = std::max(reps, 1);
            TRY(run_coop(h, reps));
            count -= reps;
            h->since_sort += reps;
            if (h->sort_interval > 0 && h->since_sort >= h->sort_interval) {
                TRY(reorder_particles(h));
                h->since_sort = 0;
            }
            continue;
        }
        int reps = 1;
        if (h->use_graph && !h->timing && count >= kGraphReps) {
            reps = kGraphReps;
            if (h->sort_interval > 0) reps = (int)std::min<int64_t>(reps, h->sort_interval - h->since_sort);
            reps = std::max(reps, 1);
        }
        TRY(run_substep(h, reps));
        count -= reps;
        h->since_sort += reps;
        if (h->sort_interval > 0 && h->since_sort >= h->sort_interval) {
            TRY(reorder_particles(h));
            h->since_sort = 0;
        }
    }
    return {};
}

// (Re)builds the colliders' narrow-band voxel grids when a mesh or the scale of its pose changed enough.
Status ensure_sdf(Handle* h) {
    if (!h->sdf_dirty || h->n_col == 0) return {};
    CK(cudaStreamSynchronize(h->stream));
    int64_t total = 0;
    std::vector<int64_t> nvox(h->n_col);
    for (int c = 0; c < h->n_col; ++c) {
        ColliderDev& col = h->cols[c];
        sdf_grid_params(col, total);
        nvox[c] = (int64_t)col.sdf.dims[0] * col.sdf.dims[1] * col.sdf.dims[2];
        total += col.n_tris > 0 ? nvox[c] : 0;
    }
    if (h->d_sdf_cells) cudaFree(h->d_sdf_cells);
    if (h->d_sdf_cand) cudaFree(h->d_sdf_cand);
    h->d_sdf_cells = nullptr;
    h->d_sdf_cand = nullptr;
    h->sdf_bytes = 0;
    invalidate_graph(h);
    if (total == 0) {
        h->sdf_dirty = false;
        return {};
    }
    int32_t *counts = nullptr, *starts = nullptr, *tmp = nullptr;
    const int64_t tiles = scan_tile_count(total) + 2;
    h->sdf_bytes = sizeof(int2) * (size_t)total;
    bool ok = cudaMalloc(&h->d_sdf_cells, sizeof(int2) * (size_t)total) == cudaSuccess &&
              cudaMalloc(&counts, sizeof(int32_t) * (size_t)total) == cudaSuccess &&
              cudaMalloc(&starts, sizeof(int32_t) * (size_t)total) == cudaSuccess &&
              cudaMalloc(&tmp, sizeof(int32_t) * (size_t)(tiles + 1)) == cudaSuccess;
    auto release = [&]() { cudaFree(counts); cudaFree(starts); cudaFree(tmp); };
    if (!ok) {
        cudaGetLastError();
        release();
        return {MPM_ERR_MEMORY, "device allocation of the collider voxel grids failed"};
    }
    for (int c = 0; c < h->n_col; ++c) {
        const ColliderDev& col = h->cols[c];
        if (col.n_tris == 0) continue;
        launch_sdf_classify(h->stream, col, h->d_nodes + col.node_offset, h->d_tris + col.tri_offset, nvox[c],
                            kSdfMaxCandidates, h->d_sdf_cells + col.sdf.cell_offset, counts + col.sdf.cell_offset);
        h->launches += 1;
    }
    launch_exclusive_scan(h->stream, counts, total, starts, tmp, tmp + tiles);
    h->launches += 3;
    int32_t n_cand = 0;
    cudaError_t e = cudaMemcpyAsync(&n_cand, tmp + tiles, sizeof n_cand, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    h->sdf_bytes += sizeof(int32_t) * (size_t)std::max(n_cand, 1);
    if (e == cudaSuccess && cudaMalloc(&h->d_sdf_cand, sizeof(int32_t) * (size_t)std::max(n_cand, 1)) != cudaSuccess)
        e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
        for (int c = 0; c < h->n_col; ++c) {
            const ColliderDev& col = h->cols[c];
            if (col.n_tris == 0) continue;
            launch_sdf_fill(h->stream, col, h->d_nodes + col.node_offset, h->d_tris + col.tri_offset, nvox[c],
                            kSdfMaxCandidates, h->d_sdf_cells + col.sdf.cell_offset, starts + col.sdf.cell_offset,
                            h->d_sdf_cand);
            h->launches += 1;
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    release();
    if (e != cudaSuccess) return {MPM_ERR_CUDA, std::string("collider voxel grid build: ") + cudaGetErrorString(e)};
    for (auto& col : h->cols) col.sdf.built = col.n_tris > 0 ? 1 : 0;
    CK(cudaMemcpyAsync(h->d_cols, h->cols.data(), sizeof(ColliderDev) * h->n_col, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->sdf_dirty = false;
    return {};
}

// Poses of the colliders for `steps` substeps (steps == 0: one substep ending at s). The pose kernel is one
// thread per pose running about 1,500 dependent FP64 operations (three slerped matrices and an FP64
// inverse, about 20 us on a GB300), so a call whose poses are already in place (explicit substeps at the
// same s with unchanged transforms, a static collider) launches nothing.
Status prepare_poses(Handle* h, int steps, double s, double frame_dt) {
    if (h->n_col == 0) return {};
    const float s_f = steps > 0 ? 0.f : (float)s, inv_fdt = (float)(1.0 / frame_dt);
    if (h->pose_valid && h->d_poses && h->pose_steps == steps && h->pose_s == s_f && h->pose_inv_fdt == inv_fdt)
        return {};
    h->pose_valid = false;
    int64_t need = (int64_t)std::max(steps, 1) * h->n_col;
    if (need > h->pose_cap) {
        CK(cudaStreamSynchronize(h->stream));
        if (h->d_poses) cudaFree(h->d_poses);
        h->d_poses = nullptr;
        int64_t cap = std::max<int64_t>(need, 2 * h->pose_cap);
        if (cudaMalloc(&h->d_poses, sizeof(ColliderPose) * (size_t)cap) != cudaSuccess) {
            cudaGetLastError();
            h->pose_cap = 0;
            return {MPM_ERR_MEMORY, "device allocation of collider poses failed"};
        }
        h->pose_cap = cap;
        invalidate_graph(h);
    }
    launch_collider_poses(h->stream, h->d_cols, h->n_col, h->d_poses, steps, (float)s, inv_fdt);
    CK(cudaGetLastError());
    h->launches += 1;
    h->pose_valid = true;
    h->pose_steps = steps;
    h->pose_s = s_f;
    h->pose_inv_fdt = inv_fdt;
    return {};
}

// skip_first / speculate: StepParams (two-grid mode, explicit substeps).
Status set_step(Handle* h, double dt, double s, double frame_dt, int steps, bool skip_first = false,
                bool speculate = false) {
    StepParams sp{};
    sp.dt = (float)dt;
    sp.s = (float)s;
    sp.inv_frame_dt = (float)(1.0 / frame_dt);
    sp.k = -1;
    sp.steps = steps;
    sp.skip_first = skip_first ? 1 : 0;
    sp.speculate = speculate ? 1 : 0;
    // only the fields before `seq`: the substep counter keeps running across calls. A pageable source is
    // staged by the driver before this call returns, so `sp` may go out of scope.
    CK(cudaMemcpyAsync(h->d_sp, &sp, offsetof(StepParams, seq), cudaMemcpyHostToDevice, h->stream));
    return {};
}

Status remove_escaped(Handle* h, int32_t* removed_out) {
    *removed_out = 0;
    EscapeBounds eb{};
    bool any = false;
    for (int a = 0; a < 3; ++a) {
        eb.open_lo[a] = !h->dom.wall_lo[a];
        eb.open_hi[a] = !h->dom.wall_hi[a];
        eb.lo[a] = (float)(h->dom.min[a] - h->dx);
        eb.hi[a] = (float)(h->dom.max[a] + h->dx);
        any = any || eb.open_lo[a] || eb.open_hi[a];
    }
    if (!any || h->P.n == 0) return {};
    const int64_t n = h->P.n;
    if (h->keep_cap < n) {
        if (h->d_keep) cudaFree(h->d_keep);
        h->d_keep = nullptr;
        h->keep_cap = std::max<int64_t>(n, h->P.cap);
        if (cudaMalloc(&h->d_keep, (size_t)h->keep_cap * 4 * sizeof(int32_t)) != cudaSuccess) {
            cudaGetLastError();
            h->keep_cap = 0;
            return {MPM_ERR_MEMORY, "device allocation of removal scratch failed"};
        }
    }
    int64_t tiles = scan_tile_count(n) + 1;
    if (h->scan_cap < tiles) {
        if (h->d_scan_tmp) cudaFree(h->d_scan_tmp);
        h->scan_cap = std::max<int64_t>(tiles, 1024);
        if (cudaMalloc(&h->d_scan_tmp, (size_t)(h->scan_cap + 2) * sizeof(int32_t)) != cudaSuccess) {
            cudaGetLastError();
            h->scan_cap = 0;
            return {MPM_ERR_MEMORY, "device allocation of scan scratch failed"};
        }
    }
    int32_t* keep_phys = h->d_keep;
    int32_t* keep_by_id = h->d_keep + h->keep_cap;
    int32_t* dst_index = h->d_keep + 2 * h->keep_cap;
    int32_t* new_id = h->d_keep + 3 * h->keep_cap;
    const int nm = (int)h->mat_desc.size();
    CK(cudaMemsetAsync(h->d_counters + 2, 0, sizeof(unsigned int) * nm, h->stream));
    launch_flag_escaped(h->stream, h->P, eb, keep_phys, keep_by_id, h->d_counters + 2);
    h->launches += 1;
    CK(cudaMemcpyAsync(h->h_counters + 2, h->d_counters + 2, sizeof(unsigned int) * nm, cudaMemcpyDeviceToHost,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int64_t removed = 0;
    for (int m = 0; m < nm; ++m) removed += h->h_counters[2 + m];
    if (removed == 0) return {};
    launch_exclusive_scan(h->stream, keep_phys, n, dst_index, h->d_scan_tmp, h->d_scan_tmp + h->scan_cap);
    launch_exclusive_scan(h->stream, keep_by_id, n, new_id, h->d_scan_tmp, h->d_scan_tmp + h->scan_cap);
    if (!h->spare_arena) {
        if (cudaMalloc(&h->spare_arena, (size_t)h->P.cap * kFields * 4) != cudaSuccess) {
            cudaGetLastError();
            h->spare_arena = nullptr;
            return {MPM_ERR_MEMORY, "device allocation of particle storage failed"};
        }
    }
    Particles dst = bind_arena(h->spare_arena, h->P.cap, n - removed);
    launch_compact(h->stream, h->P, dst, keep_phys, dst_index, new_id);
    h->launches += 7;  // two three-pass scans and the compaction
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    std::swap(h->arena, h->spare_arena);
    h->P = dst;
    for (int m = 0; m < nm; ++m) h->mat_count[m] -= h->h_counters[2 + m];
    invalidate_graph(h);
    *removed_out = (int32_t)removed;
    return {};
}

// CFL step from the bits of max |v| (warp/solver.py:176-185): dt = min(0.4 dx / (c_max + vmax), frame_dt)
// over the materials present, then the frame split into equal substeps.
void choose_dt(const Handle* h, unsigned int vmax_bits, double frame_dt, double* dt_out, int* steps_out) {
    float vmax_f;
    std::memcpy(&vmax_f, &vmax_bits, 4);
    double vmax = std::isfinite(vmax_f) ? (double)vmax_f : 0.0;
    double c = 0.0;
    for (size_t m = 0; m < h->wave.size(); ++m)
        if (h->mat_count[m] > 0) c = std::max(c, h->wave[m]);
    double dt = std::min(kCFL * h->dx / (c + vmax), frame_dt);
    int steps = (int)std::ceil(frame_dt / dt - 1e-9);
    *dt_out = frame_dt / steps;
    *steps_out = steps;
}

Status do_advance(Handle* h, double frame_dt, MpmAdvanceStats* stats) {
    if (h->P.n == 0) {
        *stats = MpmAdvanceStats{0, frame_dt, 0};
        return {};
    }
    h->frame_dt = frame_dt;
    // CFL time step (warp/solver.py:176-185): max |v| on the device, one 4-byte read back
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned int), h->stream));
    launch_max_speed(h->stream, h->P, h->d_counters);
    h->launches += 1;
    CK(cudaMemcpyAsync(h->h_counters, h->d_counters, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int steps = 0;
    double dt = 0.0;
    choose_dt(h, h->h_counters[0], frame_dt, &dt, &steps);
    TRY(prepare_grids(h, two_grids(h), false));
    TRY(set_step(h, dt, 0.0, frame_dt, steps));
    TRY(ensure_sdf(h));
    TRY(prepare_poses(h, steps, 0.0, frame_dt));
    TRY(substeps_and_sort(h, steps));
    int32_t removed = 0;
    TRY(remove_escaped(h, &removed));
    CK(cudaStreamSynchronize(h->stream));
    TRY(check_coop(h));
    *stats = MpmAdvanceStats{steps, dt, removed};
    return {};
}

Status check_mats(Handle* h, int64_t n, const int32_t* mat) {
    const int nm = (int)h->mat_desc.size();
    for (int64_t i = 0; i < n; ++i)
        if (mat[i] < 0 || mat[i] >= nm) return {MPM_ERR_VALUE, "material id out of range"};
    return {};
}

Status upload_particles(Handle* h, int64_t off, int64_t n, const float* x, const float* v, const float* C,
                        const float* F, const float* Jp, const int32_t* mat, const int32_t* emitter) {
    size_t per = (3 + 3 + (C ? 9 : 0) + (F ? 9 : 0) + (Jp ? 1 : 0) + 2) * 4;
    TRY(ensure_stage(h, per * (size_t)n));
    char* s = static_cast<char*>(h->stage);
    auto put = [&](const void* src, size_t bytes) -> void* {
        void* dst = s;
        cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream);
        s += bytes;
        return dst;
    };
    const float* dx_ = (const float*)put(x, (size_t)n * 12);
    const float* dv = (const float*)put(v, (size_t)n * 12);
    const float* dC = C ? (const float*)put(C, (size_t)n * 36) : nullptr;
    const float* dF = F ? (const float*)put(F, (size_t)n * 36) : nullptr;
    const float* dJ = Jp ? (const float*)put(Jp, (size_t)n * 4) : nullptr;
    const int32_t* dm = (const int32_t*)put(mat, (size_t)n * 4);
    const int32_t* de = (const int32_t*)put(emitter, (size_t)n * 4);
    CK(cudaGetLastError());
    launch_state_in(h->stream, h->P, off, n, dx_, dv, dC, dF, dJ, dm, de);
    launch_particle_stress(h->stream, h->P, off, n, h->d_mats, h->d_counters + 1);
    h->launches += 2;
    CK(cudaGetLastError());
    return {};
}

Status download_particles(Handle* h, float* x, float* v, float* C, float* F, float* Jp, int32_t* mat,
                          int32_t* emitter) {
    const int64_t n = h->P.n;
    if (n == 0) return {};
    size_t per = ((x ? 3 : 0) + (v ? 3 : 0) + (C ? 9 : 0) + (F ? 9 : 0) + (Jp ? 1 : 0) + (mat ? 1 : 0) + (emitter ? 1 : 0)) * 4;
    TRY(ensure_stage(h, per * (size_t)n));
    char* s = static_cast<char*>(h->stage);
    auto slot = [&](const void* host, size_t bytes) -> void* {
        if (!host) return nullptr;
        void* d = s;
        s += bytes;
        return d;
    };
    float* dx_ = (float*)slot(x, (size_t)n * 12);
    float* dv = (float*)slot(v, (size_t)n * 12);
    float* dC = (float*)slot(C, (size_t)n * 36);
    float* dF = (float*)slot(F, (size_t)n * 36);
    float* dJ = (float*)slot(Jp, (size_t)n * 4);
    int32_t* dm = (int32_t*)slot(mat, (size_t)n * 4);
    int32_t* de = (int32_t*)slot(emitter, (size_t)n * 4);
    launch_state_out(h->stream, h->P, dx_, dv, dC, dF, dJ, dm, de);
    h->launches += 1;
    CK(cudaGetLastError());
    auto get = [&](void* host, const void* dev, size_t bytes) -> cudaError_t {
        return host ? cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, h->stream) : cudaSuccess;
    };
    CK(get(x, dx_, (size_t)n * 12));
    CK(get(v, dv, (size_t)n * 12));
    CK(get(C, dC, (size_t)n * 36));
    CK(get(F, dF, (size_t)n * 36));
    CK(get(Jp, dJ, (size_t)n * 4));
    CK(get(mat, dm, (size_t)n * 4));
    CK(get(emitter, de, (size_t)n * 4));
    CK(cudaStreamSynchronize(h->stream));
    TRY(check_coop(h));  // a kernel that gave up a bounded wait since the last check
    return {};
}

Status read_wait(Handle* h) {
    if (!h->rb_pending) return {};
    h->rb_pending = false;
    CK(cudaEventSynchronize(h->rb_done));
    return {};
}

// Gathers the requested arrays into the handle's read-back storage on its stream (host order), then copies
// them to the host buffers on a copy stream, so the caller's next launches overlap the transfer.
Status read_begin(Handle* h, float* x, float* v, float* C, float* F, float* Jp, int32_t* mat, int32_t* emitter) {
    TRY(read_wait(h));
    const int64_t n = h->P.n;
    if (n == 0) return {};
    const size_t per = ((x ? 3 : 0) + (v ? 3 : 0) + (C ? 9 : 0) + (F ? 9 : 0) + (Jp ? 1 : 0) + (mat ? 1 : 0) +
                        (emitter ? 1 : 0)) * 4;
    if (per * (size_t)n > h->rb_bytes) {
        CK(cudaStreamSynchronize(h->stream));
        cudaFree(h->rb_dev);
        h->rb_dev = nullptr;
        h->rb_bytes = 0;
        const size_t b = std::max(per * (size_t)n, h->rb_bytes * 2);
        if (cudaMalloc(&h->rb_dev, b) != cudaSuccess) {
            cudaGetLastError();
            h->rb_dev = nullptr;
            return {MPM_ERR_MEMORY, "device allocation of the read-back storage failed"};
        }
        h->rb_bytes = b;
    }
    if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    if (!h->rb_ready) CK(cudaEventCreateWithFlags(&h->rb_ready, cudaEventDisableTiming));
    if (!h->rb_done) CK(cudaEventCreateWithFlags(&h->rb_done, cudaEventDisableTiming));
    char* s = static_cast<char*>(h->rb_dev);
    auto slot = [&](const void* host, size_t bytes) -> void* {
        if (!host) return nullptr;
        void* d = s;
        s += bytes;
        return d;
    };
    float* dx_ = (float*)slot(x, (size_t)n * 12);
    float* dv = (float*)slot(v, (size_t)n * 12);
    float* dC = (float*)slot(C, (size_t)n * 36);
    float* dF = (float*)slot(F, (size_t)n * 36);
    float* dJ = (float*)slot(Jp, (size_t)n * 4);
    int32_t* dm = (int32_t*)slot(mat, (size_t)n * 4);
    int32_t* de = (int32_t*)slot(emitter, (size_t)n * 4);
    launch_state_out(h->stream, h->P, dx_, dv, dC, dF, dJ, dm, de);
    h->launches += 1;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->rb_ready, h->stream));
    CK(cudaStreamWaitEvent(h->copy_stream, h->rb_ready, 0));
    auto get = [&](void* host, const void* dev, size_t bytes) -> cudaError_t {
        return host ? cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, h->copy_stream) : cudaSuccess;
    };
    CK(get(x, dx_, (size_t)n * 12));
    CK(get(v, dv, (size_t)n * 12));
    CK(get(C, dC, (size_t)n * 36));
    CK(get(F, dF, (size_t)n * 36));
    CK(get(Jp, dJ, (size_t)n * 4));
    CK(get(mat, dm, (size_t)n * 4));
    CK(get(emitter, de, (size_t)n * 4));
    CK(cudaEventRecord(h->rb_done, h->copy_stream));
    h->rb_pending = true;
    return {};
}

Status create(const MpmDomainDesc* dom, const MpmMaterialDesc* mats, int32_t n_mat, const double gravity[3], int32_t ppc,
              int32_t device, Handle** out) {
    if (!dom || !gravity || !out || (n_mat > 0 && !mats)) return {MPM_ERR_ARGUMENT, "null argument"};
    if (n_mat > kMaxMaterials) return {MPM_ERR_VALUE, "too many materials"};
    if (ppc <= 0) return {MPM_ERR_VALUE, "particles_per_cell must be positive"};
    if (const char* why = domain_problem(*dom)) return {MPM_ERR_VALUE, why};
    for (int m = 0; m < n_mat; ++m) {
        const MpmMaterialDesc& md = mats[m];
        if (md.model < 0 || md.model > 3)
            return {MPM_ERR_NOT_IMPLEMENTED, "material model is not supported by the gb300 backend"};
        // the ranges MaterialParams enforces (mpm_core/materials.py:38-46), checked again here because a raw
        // descriptor can reach this boundary without passing through that record
        if (!(md.youngs_modulus > 0)) return {MPM_ERR_VALUE, "youngs_modulus must be > 0"};
        if (!(md.poisson_ratio >= 0 && md.poisson_ratio < 0.5)) return {MPM_ERR_VALUE, "poisson_ratio must be in [0, 0.5)"};
        if (!(md.density > 0)) return {MPM_ERR_VALUE, "density must be > 0"};
    }
    Handle* h = new Handle();
    *out = h;
    h->device = device;
    DeviceGuard guard(device);
    CK(prepare_substep_kernels());
    CK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;
    h->dom = *dom;
    h->ppc = ppc;
    h->g = make_grid(*dom, gravity, ppc, &h->hd);
    h->dx = h->hd.dx;
    h->inv_dx = h->hd.inv_dx;
    h->p_vol = h->hd.p_vol;
    for (int a = 0; a < 3; ++a) {
        h->origin[a] = h->hd.origin[a];
        h->dims[a] = h->hd.dims[a];
    }
    GridDesc& g = h->g;
    std::vector<Material> table(std::max(1, (int)n_mat));
    h->mat_desc.assign(mats, mats + n_mat);
    h->mat_count.assign(n_mat, 0);
    for (int m = 0; m < n_mat; ++m) {
        double wave;
        table[m] = make_material(mats[m], h->p_vol, &wave);
        h->wave.push_back(wave);
    }
    CK(cudaMalloc(&h->d_mats, sizeof(Material) * table.size()));
    CK(cudaMemcpy(h->d_mats, table.data(), sizeof(Material) * table.size(), cudaMemcpyHostToDevice));
    h->grid_nodes = (int64_t)g.nb[0] * g.nb[1] * g.nb[2] * 64;
    if (cudaMalloc(&h->grid, (size_t)h->grid_nodes * sizeof(float4)) != cudaSuccess) {
        cudaGetLastError();
        return {MPM_ERR_MEMORY, "device allocation of the grid failed"};
    }
    CK(cudaMemset(h->grid, 0, (size_t)h->grid_nodes * sizeof(float4)));
    CK(cudaMalloc(&h->d_sp, sizeof(StepParams)));
    CK(cudaMemset(h->d_sp, 0, sizeof(StepParams)));
    {  // work lists: one flag and two list slots per grid block, one candidate slot per grid node
        const int64_t nblk = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
        CK(cudaMalloc(&h->wl.block_flag, sizeof(unsigned int) * (size_t)nblk));
        CK(cudaMemset(h->wl.block_flag, 0, sizeof(unsigned int) * (size_t)nblk));
        CK(cudaMalloc(&h->wl.blocks[0], sizeof(int32_t) * (size_t)nblk));
        CK(cudaMalloc(&h->wl.blocks[1], sizeof(int32_t) * (size_t)nblk));
        CK(cudaMalloc(&h->wl.counts, sizeof(unsigned int) * 4));
        CK(cudaMemset(h->wl.counts, 0, sizeof(unsigned int) * 4));
        CK(cudaMalloc(&h->wl.node_cand, sizeof(int32_t) * (size_t)h->grid_nodes));
        // sort by grid node: one count and start per node, plus the key of stencils outside the grid
        CK(cudaMalloc(&h->ss.count, sizeof(unsigned int) * (size_t)(h->grid_nodes + 1)));
        CK(cudaMalloc(&h->ss.start, sizeof(int32_t) * (size_t)(h->grid_nodes + 1)));
        h->ss_scan_cap = scan_tile_count(h->grid_nodes + 1) + 1;
        CK(cudaMalloc(&h->ss_scan, sizeof(int32_t) * (size_t)(h->ss_scan_cap + 2)));
    }
    CK(cudaMalloc(&h->d_counters, sizeof(unsigned int) * (3 + kMaxMaterials)));
    CK(cudaMemset(h->d_counters, 0, sizeof(unsigned int) * (3 + kMaxMaterials)));
    CK(cudaMalloc(&h->d_coop, sizeof(unsigned int) * 4));
    CK(cudaMemset(h->d_coop, 0, sizeof(unsigned int) * 4));
    CK(cudaMallocHost(&h->h_counters, sizeof(unsigned int) * (2 + kMaxMaterials)));
    TRY(ensure_capacity(h, 4096));
    return {};
}

Status batch_remove(Batch* b, Handle* h);

void destroy(Handle* h) {
    if (!h) return;
    DeviceGuard guard(h->device);
    read_wait(h);
    if (h->batch) batch_remove(h->batch, h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    invalidate_graph(h);
    for (auto& v : h->ev_pending)
        for (auto e : v) cudaEventDestroy(e);
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    for (auto e : h->tev)
        if (e) cudaEventDestroy(e);
    for (auto e : h->perm_ev)
        if (e) cudaEventDestroy(e);
    free_colliders(h);
    cudaFree(h->arena);
    cudaFree(h->spare_arena);
    cudaFree(h->grid);
    cudaFree(h->grid2);
    cudaFree(h->vol);
    cudaFree(h->d_mats);
    cudaFree(h->d_sp);
    cudaFree(h->d_counters);
    cudaFree(h->d_coop);
    cudaFree(h->d_keep);
    cudaFree(h->d_scan_tmp);
    cudaFree(h->d_poses);
    cudaFree(h->d_sdf_cells);
    cudaFree(h->d_sdf_cand);
    cudaFree(h->wl.block_flag);
    cudaFree(h->wl.blocks[0]);
    cudaFree(h->wl.blocks[1]);
    cudaFree(h->wl.counts);
    cudaFree(h->wl.node_cand);
    cudaFree(h->wl.part_cand);
    cudaFree(h->d_fixed);
    cudaFree(h->d_poison);
    cudaFree(h->ss.key);
    cudaFree(h->ss.count);
    cudaFree(h->ss.start);
    cudaFree(h->ss_scan);
    cudaFree(h->stage);
    cudaFree(h->rb_dev);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->rb_ready) cudaEventDestroy(h->rb_ready);
    if (h->rb_done) cudaEventDestroy(h->rb_done);
    if (h->h_counters) cudaFreeHost(h->h_counters);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
}

Status set_transforms(Handle* h, int32_t n, const float* start16, const float* end16) {
    if (n != h->n_col) return {MPM_ERR_VALUE, "expected " + std::to_string(h->n_col) + " collider transforms"};
    if (n == 0) return {};
    if (!start16 || !end16) return {MPM_ERR_ARGUMENT, "null transform array"};
    h->pose_valid = false;
    for (int c = 0; c < n; ++c) {
        collider_set_pose(h->cols[c], start16 + 16 * c, end16 + 16 * c, h->dx);
        const SdfGridDev& g = h->cols[c].sdf;
        if (!g.built || h->cols[c].margin > g.margin || h->cols[c].margin / 3.0f > g.cutoff) h->sdf_dirty = true;
    }
    CK(cudaMemcpyAsync(h->d_cols, h->cols.data(), sizeof(ColliderDev) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return {};
}

Status set_colliders(Handle* h, int32_t n, const MpmColliderDesc* cs) {
    if (n < 0 || (n > 0 && !cs)) return {MPM_ERR_ARGUMENT, "bad collider list"};
    CK(cudaStreamSynchronize(h->stream));
    free_colliders(h);
    invalidate_graph(h);
    h->sdf_dirty = true;
    h->cols.assign(n, ColliderDev{});
    h->n_col = n;
    std::vector<BvhNode> all_nodes;
    std::vector<MeshTri> all_tris;
    for (int c = 0; c < n; ++c) {
        const MpmColliderDesc& d = cs[c];
        if (d.n_tris < 0 || d.n_verts < 0 || (d.n_tris > 0 && (!d.tris || !d.verts)))
            return {MPM_ERR_VALUE, "bad collider mesh"};
        for (int i = 0; i < 3 * d.n_tris; ++i)
            if (d.tris[i] < 0 || d.tris[i] >= d.n_verts) return {MPM_ERR_VALUE, "collider triangle index out of range"};
        collider_static(h->cols[c], d, (int)all_nodes.size(), (int)all_tris.size());
        std::vector<BvhNode> nodes;
        std::vector<MeshTri> tris;
        build_mesh(MeshInput{d.n_verts, d.n_tris, d.verts, d.tris}, nodes, tris);
        all_nodes.insert(all_nodes.end(), nodes.begin(), nodes.end());  // child indices stay collider-local
        all_tris.insert(all_tris.end(), tris.begin(), tris.end());
    }
    if (n > 0) {
        h->collider_bytes = sizeof(ColliderDev) * n + sizeof(BvhNode) * std::max<size_t>(1, all_nodes.size()) +
                            sizeof(MeshTri) * std::max<size_t>(1, all_tris.size());
        CK(cudaMalloc(&h->d_cols, sizeof(ColliderDev) * n));
        CK(cudaMalloc(&h->d_nodes, sizeof(BvhNode) * std::max<size_t>(1, all_nodes.size())));
        CK(cudaMalloc(&h->d_tris, sizeof(MeshTri) * std::max<size_t>(1, all_tris.size())));
        CK(cudaMemcpy(h->d_nodes, all_nodes.data(), sizeof(BvhNode) * all_nodes.size(), cudaMemcpyHostToDevice));
        if (!all_tris.empty())
            CK(cudaMemcpy(h->d_tris, all_tris.data(), sizeof(MeshTri) * all_tris.size(), cudaMemcpyHostToDevice));
        std::vector<float> eye(16 * (size_t)n, 0.0f);
        for (int c = 0; c < n; ++c)
            for (int k = 0; k < 4; ++k) eye[16 * c + 5 * k] = 1.0f;
        TRY(set_transforms(h, n, eye.data(), eye.data()));
    }
    return {};
}


// ------------------------------------------------------------------------------------------------------
// Batches: independent scenes (handles on one device) advanced together. Every kernel of a substep is
// launched once for all scenes (mpm_batch_kernels.cu) from a device table of the scenes' SubstepArgs; the
// launch sequence of one batched substep is a captured CUDA graph replayed as many times as the scene with
// the most substeps needs, and scenes whose frame is done idle (StepParams::active). Member handles run
// all their work on the batch's stream.
// ------------------------------------------------------------------------------------------------------
struct Batch {
    int device = -1;
    cudaStream_t stream = nullptr;
    std::vector<Handle*> scenes;             // in the order they were added
    std::vector<Handle*> live;               // scenes with particles in the current advance
    SubstepArgs* d_table = nullptr;
    int table_cap = 0;
    int32_t* d_cta = nullptr;                // cta_scene (particle CTAs) followed by cta_first (per scene)
    int64_t cta_cap = 0;
    unsigned int particle_ctas = 0;
    bool any_colliders = false;
    bool any_fp64_clamp = false;
    bool any_fixed = false;  // some scene in deterministic mode (the P2G build with the fixed-point path)
    std::vector<int64_t> layout;             // what the captured graphs depend on
    cudaGraphExec_t graph = nullptr;         // one batched substep
    cudaGraphExec_t graph_many = nullptr;    // kGraphReps batched substeps
    unsigned int* d_vmax = nullptr;          // per scene: max |v| bits
    unsigned int* h_vmax = nullptr;          // pinned
    int vmax_cap = 0;
    int sort_interval = 4;
    LaunchShape shape;
    int64_t launches = 0;
    std::string err;
};

int finish_batch(Batch* b, Status s) {
    if (s.code != MPM_OK) {
        if (b) b->err = s.msg;
        g_last_error = s.msg;
    }
    return s.code;
}

void batch_invalidate(Batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->graph_many) cudaGraphExecDestroy(b->graph_many);
    b->graph = nullptr;
    b->graph_many = nullptr;
    b->layout.clear();
}

// Table of the live scenes and the CTA layout of the particle kernels (ceil(cap / 256) CTAs per scene, so
// the layout changes only when a capacity does). The table itself is uploaded every time it is called.
Status batch_upload(Batch* b) {
    const int n = (int)b->live.size();
    if (n > b->table_cap) {
        CK(cudaStreamSynchronize(b->stream));
        cudaFree(b->d_table);
        b->d_table = nullptr;
        b->table_cap = 0;
        CK(cudaMalloc(&b->d_table, sizeof(SubstepArgs) * (size_t)std::max(n, 8)));
        b->table_cap = std::max(n, 8);
        batch_invalidate(b);
    }
    std::vector<SubstepArgs> table(n);
    std::vector<int64_t> layout{n};
    int64_t ctas = 0;
    bool cols = false, clamp = false, fixed = false;
    for (int s = 0; s < n; ++s) {
        Handle* h = b->live[s];
        TRY(prepare_grids(h, false, false));  // a batch runs its scenes in one-grid mode
        table[s] = substep_args(h);
        table[s].grid2 = nullptr;
        table[s].block_sweep = 0;  // a batch's P2G lists the blocks itself
        table[s].p2g_group = b->shape.p2g_group;
        layout.push_back(h->P.cap);
        ctas += (h->P.cap + 255) / 256;
        cols = cols || h->n_col > 0;
        clamp = clamp || h->fp64_clamp;
        fixed = fixed || table[s].fixed != nullptr;
    }
    layout.push_back(cols ? 1 : 0);
    layout.push_back(clamp ? 1 : 0);
    layout.push_back(fixed ? 1 : 0);
    if (layout != b->layout) {
        CK(cudaStreamSynchronize(b->stream));
        batch_invalidate(b);
        if (ctas + n > b->cta_cap) {
            cudaFree(b->d_cta);
            b->d_cta = nullptr;
            b->cta_cap = 0;
            CK(cudaMalloc(&b->d_cta, sizeof(int32_t) * (size_t)(ctas + n)));
            b->cta_cap = ctas + n;
        }
        std::vector<int32_t> cta(ctas + n);
        int64_t c = 0;
        for (int s = 0; s < n; ++s) {
            cta[ctas + s] = (int32_t)c;
            const int64_t k = (b->live[s]->P.cap + 255) / 256;
            for (int64_t i = 0; i < k; ++i) cta[c++] = s;
        }
        CK(cudaMemcpyAsync(b->d_cta, cta.data(), sizeof(int32_t) * cta.size(), cudaMemcpyHostToDevice, b->stream));
        b->particle_ctas = (unsigned int)ctas;
        b->any_colliders = cols;
        b->any_fp64_clamp = clamp;
        b->any_fixed = fixed;
        b->layout = layout;
    }
    // a pageable source is staged by the driver before the call returns, so `table` may go out of scope
    CK(cudaMemcpyAsync(b->d_table, table.data(), sizeof(SubstepArgs) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
    return {};
}

// reps (1 or kGraphReps) batched substeps in one graph launch.
Status batch_replay(Batch* b, int reps = 1) {
    BatchLaunch bl{b->d_table, b->d_cta, b->d_cta + b->particle_ctas, (int)b->live.size(), b->particle_ctas,
                   b->any_colliders, b->any_fp64_clamp, b->any_fixed, b->shape};
    cudaGraphExec_t& g = reps == 1 ? b->graph : b->graph_many;
    if (!g) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        for (int r = 0; r < reps; ++r) launch_batch_substep(b->stream, bl);
        cudaError_t e0 = cudaGetLastError();
        cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        CK(e0);
        CK(e);
        e = cudaGraphInstantiate(&g, graph, 0);
        cudaGraphDestroy(graph);
        CK(e);
    }
    CK(cudaGraphLaunch(g, b->stream));
    b->launches += (int64_t)batch_substep_kernel_count(bl) * reps;
    return {};
}

// One frame of every scene: per-scene CFL step (one read-back for all scenes), poses and voxel grids, then
// max(steps) batched substeps with the reorder of every scene still running after each sort_interval of
// them, then removal of escaped particles scene by scene.
Status batch_advance(Batch* b, const double* frame_dt, MpmAdvanceStats* stats) {
    const int S = (int)b->scenes.size();
    if (S > b->vmax_cap) {
        CK(cudaStreamSynchronize(b->stream));
        cudaFree(b->d_vmax);
        cudaFreeHost(b->h_vmax);
        b->d_vmax = nullptr;
        b->h_vmax = nullptr;
        b->vmax_cap = 0;
        CK(cudaMalloc(&b->d_vmax, sizeof(unsigned int) * (size_t)std::max(S, 8)));
        CK(cudaMallocHost(&b->h_vmax, sizeof(unsigned int) * (size_t)std::max(S, 8)));
        b->vmax_cap = std::max(S, 8);
    }
    if (S == 0) return {};
    CK(cudaMemsetAsync(b->d_vmax, 0, sizeof(unsigned int) * (size_t)S, b->stream));
    for (int s = 0; s < S; ++s) {
        Handle* h = b->scenes[s];
        if (h->P.n == 0) continue;
        launch_max_speed(b->stream, h->P, b->d_vmax + s);
        h->launches += 1;
    }
    CK(cudaMemcpyAsync(b->h_vmax, b->d_vmax, sizeof(unsigned int) * (size_t)S, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->live.clear();
    std::vector<int> steps(S, 0);
    int max_steps = 0;
    for (int s = 0; s < S; ++s) {
        Handle* h = b->scenes[s];
        stats[s] = MpmAdvanceStats{0, frame_dt[s], 0};
        if (h->P.n == 0) continue;
        double dt = 0.0;
        choose_dt(h, b->h_vmax[s], frame_dt[s], &dt, &steps[s]);
        stats[s] = MpmAdvanceStats{steps[s], dt, 0};
        h->frame_dt = frame_dt[s];
        TRY(set_step(h, dt, 0.0, frame_dt[s], steps[s]));
        TRY(ensure_sdf(h));
        TRY(prepare_poses(h, steps[s], 0.0, frame_dt[s]));
        TRY(ensure_part_cand(h));
        b->live.push_back(h);
        max_steps = std::max(max_steps, steps[s]);
    }
    if (!b->live.empty()) {
        TRY(batch_upload(b));
        for (int k = 0; k < max_steps;) {
            // as many substeps per graph launch as fit before the next reorder is due
            int reps = max_steps - k >= kGraphReps ? kGraphReps : 1;
            if (b->sort_interval > 0 && reps > 1) {
                const int to_sort = b->sort_interval - k % b->sort_interval;
                if (to_sort < reps) reps = 1;
            }
            TRY(batch_replay(b, reps));
            k += reps;
            if (b->sort_interval > 0 && k % b->sort_interval == 0 && k < max_steps) {
                bool any = false;
                for (int s = 0; s < S; ++s) {
                    Handle* h = b->scenes[s];
                    if (h->P.n == 0 || steps[s] <= k) continue;  // done or empty: no later substep
                    TRY(reorder_particles(h));
                    any = true;
                }
                if (any) TRY(batch_upload(b));
            }
        }
    }
    for (int s = 0; s < S; ++s) {
        Handle* h = b->scenes[s];
        if (h->P.n == 0) continue;
        int32_t removed = 0;
        TRY(remove_escaped(h, &removed));
        stats[s].removed = removed;
    }
    CK(cudaStreamSynchronize(b->stream));
    return {};
}

Status batch_add(Batch* b, Handle* h) {
    if (h->batch) return {MPM_ERR_VALUE, "the scene already belongs to a batch"};
    if ((int)b->scenes.size() >= kMaxBatchScenes)
        return {MPM_ERR_VALUE, "a batch holds at most " + std::to_string(kMaxBatchScenes) + " scenes"};
    if (b->device < 0) b->device = h->device;
    if (h->device != b->device) return {MPM_ERR_VALUE, "the scenes of a batch must be on one device"};
    if (!b->stream) CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaStreamSynchronize(h->own_stream));
    h->stream = b->stream;
    h->batch = b;
    invalidate_graph(h);
    b->scenes.push_back(h);
    batch_invalidate(b);
    return {};
}

Status batch_remove(Batch* b, Handle* h) {
    auto it = std::find(b->scenes.begin(), b->scenes.end(), h);
    if (it == b->scenes.end()) return {MPM_ERR_VALUE, "the scene is not in this batch"};
    CK(cudaStreamSynchronize(b->stream));
    b->scenes.erase(it);
    b->live.clear();
    h->stream = h->own_stream;
    h->batch = nullptr;
    invalidate_graph(h);
    batch_invalidate(b);
    return {};
}

void batch_destroy(Batch* b) {
    if (!b) return;
    if (b->device >= 0) {
        DeviceGuard guard(b->device);
        if (b->stream) cudaStreamSynchronize(b->stream);
        for (Handle* h : b->scenes) {
            h->stream = h->own_stream;
            h->batch = nullptr;
            invalidate_graph(h);
        }
        batch_invalidate(b);
        cudaFree(b->d_table);
        cudaFree(b->d_cta);
        cudaFree(b->d_vmax);
        cudaFreeHost(b->h_vmax);
        if (b->stream) cudaStreamDestroy(b->stream);
    }
    delete b;
}
}  // namespace

void mpm::set_last_error(const std::string& msg) { g_last_error = msg; }

// ============================================================================================================
// C-ABI
// ============================================================================================================
extern "C" {

int mpm_create(const MpmDomainDesc* domain, const MpmMaterialDesc* materials, int32_t n_materials,
               const double gravity[3], int32_t particles_per_cell, int32_t device, void** handle) {
    Handle* h = nullptr;
    Status s = create(domain, materials, n_materials, gravity, particles_per_cell, device, &h);
    if (s.code != MPM_OK) {
        destroy(h);
        if (handle) *handle = nullptr;
        return finish(nullptr, s);
    }
    *handle = h;
    return MPM_OK;
}

int mpm_destroy(void* handle) {
    destroy(static_cast<Handle*>(handle));
    return MPM_OK;
}

const char* mpm_last_error(void* handle) {
    return handle ? static_cast<Handle*>(handle)->err.c_str() : g_last_error.c_str();
}

#define HANDLE_OR_FAIL(hv)                                                                     \
    Handle* h = static_cast<Handle*>(hv);                                                      \
    if (!h) return finish(nullptr, Status{MPM_ERR_ARGUMENT, "null handle"});                   \
    DeviceGuard guard_(h->device)

int mpm_add_particles(void* handle, int64_t n, const float* x, const float* v, const int32_t* material_ids,
                      const int32_t* emitter_ids) {
    HANDLE_OR_FAIL(handle);
    if (n == 0) return MPM_OK;
    if (n < 0 || !x || !v || !material_ids || !emitter_ids) return finish(h, {MPM_ERR_ARGUMENT, "bad particle arrays"});
    auto run = [&]() -> Status {
        TRY(check_mats(h, n, material_ids));
        TRY(drop_pending(h));
        TRY(ensure_capacity(h, h->P.n + n));
        TRY(upload_particles(h, h->P.n, n, x, v, nullptr, nullptr, nullptr, material_ids, emitter_ids));
        CK(cudaStreamSynchronize(h->stream));
        h->P.n += n;
        for (int64_t i = 0; i < n; ++i) h->mat_count[material_ids[i]] += 1;
        invalidate_graph(h);
        return {};
    };
    return finish(h, run());
}

int mpm_set_colliders(void* handle, int32_t n, const MpmColliderDesc* colliders) {
    HANDLE_OR_FAIL(handle);
    return finish(h, set_colliders(h, n, colliders));
}

int mpm_set_collider_transforms(void* handle, int32_t n, const float* start16, const float* end16) {
    HANDLE_OR_FAIL(handle);
    return finish(h, set_transforms(h, n, start16, end16));
}

int mpm_advance(void* handle, double frame_dt, MpmAdvanceStats* stats) {
    HANDLE_OR_FAIL(handle);
    if (!stats) return finish(h, {MPM_ERR_ARGUMENT, "null stats"});
    if (!(frame_dt > 0)) return finish(h, {MPM_ERR_VALUE, "frame_dt must be positive"});
    return finish(h, do_advance(h, frame_dt, stats));
}

int mpm_substep(void* handle, double dt, double s, double frame_dt) {
    HANDLE_OR_FAIL(handle);
    auto run = [&]() -> Status {
        if (h->P.n == 0) return {};
        h->frame_dt = frame_dt;
        // two-grid mode: the previous explicit substep scattered for this one if it had the same dt; this
        // one scatters for the next in turn (dropped if the next call is not a substep with this dt)
        const bool two = two_grids(h);
        const bool keep = two && h->two_live && h->pending && (float)dt == h->pending_dt;
        TRY(prepare_grids(h, two, keep));
        TRY(set_step(h, dt, s, frame_dt, 0, keep, two));
        TRY(ensure_sdf(h));
        TRY(prepare_poses(h, 0, s, frame_dt));
        TRY(substep_and_sort(h));
        h->pending = two;
        h->pending_dt = (float)dt;
        return {};
    };
    return finish(h, run());
}

int mpm_coop_barrier_selftest(void* handle, int32_t stall, int32_t* timed_out) {
    HANDLE_OR_FAIL(handle);
    if (!timed_out) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    unsigned int flag = 0;
    auto run = [&]() -> Status {
        CK(cudaStreamSynchronize(h->stream));
        CK(barrier_selftest(h->stream, stall != 0, h->d_coop, &flag));
        return {};
    };
    const int st = finish(h, run());
    *timed_out = (int32_t)flag;
    return st;
}

int mpm_run_substeps(void* handle, double dt, int32_t count, double frame_dt) {
    HANDLE_OR_FAIL(handle);
    if (!(dt > 0.0) || count < 0 || !(frame_dt > 0.0)) return finish(h, {MPM_ERR_VALUE, "bad dt, count or frame_dt"});
    auto run = [&]() -> Status {
        if (h->P.n == 0 || count == 0) return {};
        h->frame_dt = frame_dt;
        TRY(prepare_grids(h, two_grids(h), false));
        TRY(set_step(h, dt, 0.0, frame_dt, count));
        TRY(ensure_sdf(h));
        TRY(prepare_poses(h, count, 0.0, frame_dt));
        TRY(substeps_and_sort(h, count));
        CK(cudaStreamSynchronize(h->stream));
        TRY(check_coop(h));
        return {};
    };
    return finish(h, run());
}

int mpm_particle_count(void* handle, int64_t* n) {
    HANDLE_OR_FAIL(handle);
    if (!n) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    *n = h->P.n;
    return MPM_OK;
}

int mpm_get_particles(void* handle, float* x, float* v, int32_t* material_ids, int32_t* emitter_ids) {
    HANDLE_OR_FAIL(handle);
    return finish(h, download_particles(h, x, v, nullptr, nullptr, nullptr, material_ids, emitter_ids));
}

int mpm_save_state(void* handle, float* x, float* v, float* C, float* F, float* Jp, int32_t* mat, int32_t* emitter) {
    HANDLE_OR_FAIL(handle);
    return finish(h, download_particles(h, x, v, C, F, Jp, mat, emitter));
}

int mpm_load_state(void* handle, int64_t n, const float* x, const float* v, const float* C, const float* F,
                   const float* Jp, const int32_t* mat, const int32_t* emitter) {
    HANDLE_OR_FAIL(handle);
    if (n < 0 || (n > 0 && (!x || !v || !C || !F || !Jp || !mat || !emitter)))
        return finish(h, {MPM_ERR_ARGUMENT, "bad state arrays"});
    auto run = [&]() -> Status {
        TRY(check_mats(h, n, mat));
        TRY(drop_pending(h));
        CK(cudaStreamSynchronize(h->stream));
        h->P.n = 0;
        TRY(ensure_capacity(h, n));
        if (n > 0) TRY(upload_particles(h, 0, n, x, v, C, F, Jp, mat, emitter));
        CK(cudaStreamSynchronize(h->stream));
        h->P.n = n;
        std::fill(h->mat_count.begin(), h->mat_count.end(), 0);
        for (int64_t i = 0; i < n; ++i) h->mat_count[mat[i]] += 1;
        invalidate_graph(h);
        return {};
    };
    return finish(h, run());
}

int mpm_is_occupied(void* handle, int64_t m, const float* points, uint8_t* out) {
    HANDLE_OR_FAIL(handle);
    if (m == 0) return MPM_OK;
    if (m < 0 || !points || !out) return finish(h, {MPM_ERR_ARGUMENT, "bad query arrays"});
    auto run = [&]() -> Status {
        if (!h->vol) {
            if (cudaMalloc(&h->vol, (size_t)h->grid_nodes * sizeof(float)) != cudaSuccess) {
                cudaGetLastError();
                h->vol = nullptr;
                return {MPM_ERR_MEMORY, "device allocation of the occupancy grid failed"};
            }
        }
        TRY(ensure_stage(h, (size_t)m * 13));
        float* dpts = static_cast<float*>(h->stage);
        uint8_t* dout = reinterpret_cast<uint8_t*>(dpts + 3 * m);
        CK(cudaMemsetAsync(h->vol, 0, (size_t)h->grid_nodes * sizeof(float), h->stream));
        CK(cudaMemcpyAsync(dpts, points, (size_t)m * 12, cudaMemcpyHostToDevice, h->stream));
        if (h->deterministic) {
            unsigned int* vol = reinterpret_cast<unsigned int*>(h->vol);
            launch_scatter_volume_fixed(h->stream, h->P, h->g, vol);
            launch_query_fill_fixed(h->stream, h->g, vol, std::pow(h->dx, 3.0), m, dpts, dout);
        } else {
            launch_scatter_volume(h->stream, h->P, h->g, h->vol);
            launch_query_fill(h->stream, h->g, h->vol, (float)std::pow(h->dx, 3.0), m, dpts, dout);
        }
        h->launches += 2;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(out, dout, (size_t)m, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return {};
    };
    return finish(h, run());
}

int mpm_set_option(void* handle, int32_t option, int64_t value) {
    HANDLE_OR_FAIL(handle);
    switch (option) {
        case MPM_OPT_USE_GRAPH:
            h->use_graph = value != 0;
            if (!h->use_graph) invalidate_graph(h);
            return MPM_OK;
        case MPM_OPT_KERNEL_TIMING:
            if (value < 0 || value > 2) return finish(h, {MPM_ERR_VALUE, "kernel timing must be 0, 1 or 2"});
            h->timing = (int)value;
            return MPM_OK;
        case MPM_OPT_DETERMINISTIC:
            return finish(h, set_deterministic(h, value != 0));
        case MPM_OPT_G2P_VARIANT:
            if (value < 0 || value > 3) return finish(h, {MPM_ERR_VALUE, "G2P variant must be 0, 1, 2 or 3"});
            h->shape.g2p_variant = (int)value;
            return MPM_OK;
        case MPM_OPT_LIST_CTAS:
            if (value < 1 || value > (1 << 20)) return finish(h, {MPM_ERR_VALUE, "work-list CTAs out of range"});
            h->shape.list_ctas = (unsigned int)value;
            return MPM_OK;
        case MPM_OPT_PDL:
            h->shape.pdl = value != 0;
            return MPM_OK;
        case MPM_OPT_P2G_TILE:
            h->shape.p2g_tile = value != 0;
            return MPM_OK;
        case MPM_OPT_BLOCK_SWEEP:
            h->shape.block_sweep = value != 0;
            return MPM_OK;
        case MPM_OPT_P2G_MERGE:
            h->shape.p2g_merge = value != 0;
            return MPM_OK;
        case MPM_OPT_PARTICLES_PER_THREAD:
            if (value != 1 && value != 2 && value != 4 && value != 8)
                return finish(h, {MPM_ERR_VALUE, "particles per thread must be 1, 2, 4 or 8"});
            h->shape.ppt = (int)value;
            return MPM_OK;
        case MPM_OPT_COOP:
            if (value < 0 || value > 2) return finish(h, {MPM_ERR_VALUE, "cooperative mode must be 0, 1 or 2"});
            h->coop = (int)value;
            return MPM_OK;
        case MPM_OPT_FP64_CLAMP:
            if (value < 0 || value > 2) return finish(h, {MPM_ERR_VALUE, "FP64 clamp mode must be 0, 1 or 2"});
            h->fp64_clamp = (int)value;
            invalidate_graph(h);  // the flag is a kernel argument of the captured graphs
            return MPM_OK;
        case MPM_OPT_P2G_GROUP:
            if (value < 1 || value > 32 || (value & (value - 1)))
                return finish(h, {MPM_ERR_VALUE, "P2G group must be a power of two from 1 to 32"});
            h->shape.p2g_group = (int)value;
            return MPM_OK;
        case MPM_OPT_SORT_INTERVAL:
            if (value < 0 || value > (1 << 30)) return finish(h, {MPM_ERR_VALUE, "sort interval out of range"});
            h->sort_interval = (int)value;
            h->since_sort = 0;
            return MPM_OK;
        case MPM_OPT_FUSED_P2G:
            return finish(h, set_fused_p2g(h, value != 0));
        default:
            return finish(h, {MPM_ERR_VALUE, "unknown option"});
    }
}

int mpm_get_stream(void* handle, void** stream) {
    HANDLE_OR_FAIL(handle);
    if (!stream) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    *stream = h->stream;
    return MPM_OK;
}

int mpm_synchronize(void* handle) {
    HANDLE_OR_FAIL(handle);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return finish(h, {MPM_ERR_CUDA, cudaGetErrorString(e)});
    return finish(h, check_coop(h));
}

int mpm_kernel_times(void* handle, int32_t n_slots, float* ms, int64_t* launches, int32_t reset) {
    HANDLE_OR_FAIL(handle);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return finish(h, {MPM_ERR_CUDA, cudaGetErrorString(e)});
    for (auto& ev : h->ev_pending) {
        accumulate_times(h, ev.data());
        for (auto x : ev) h->ev_pool.push_back(x);
    }
    h->ev_pending.clear();
    for (int i = 0; i < n_slots && i < 5; ++i) {
        if (ms) ms[i] = (float)h->t_ms[i];
        if (launches) launches[i] = h->t_launches[i];
    }
    if (reset)
        for (int i = 0; i < 5; ++i) { h->t_ms[i] = 0; h->t_launches[i] = 0; }
    return MPM_OK;
}

int mpm_grid_dims(void* handle, int32_t dims[3]) {
    HANDLE_OR_FAIL(handle);
    if (!dims) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    for (int a = 0; a < 3; ++a) dims[a] = h->dims[a];
    return MPM_OK;
}

int mpm_domain_grid_dims(const MpmDomainDesc* domain, int32_t dims[3]) {
    if (!domain || !dims) return finish(nullptr, {MPM_ERR_ARGUMENT, "null argument"});
    if (const char* why = domain_problem(*domain)) return finish(nullptr, {MPM_ERR_VALUE, why});
    const double gravity[3] = {0.0, 0.0, 0.0};
    HostDomain hd{};
    make_grid(*domain, gravity, 1, &hd);
    for (int a = 0; a < 3; ++a) dims[a] = hd.dims[a];
    return MPM_OK;
}

int mpm_read_grid(void* handle, float* out) {
    HANDLE_OR_FAIL(handle);
    if (!out) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    auto run = [&]() -> Status {
        size_t bytes = (size_t)h->dims[0] * h->dims[1] * h->dims[2] * sizeof(float4);
        TRY(ensure_stage(h, bytes));
        const float4* grid = h->grid;
        if (h->two_live) {  // the grid of the last substep
            StepParams sp;
            CK(cudaMemcpyAsync(&sp, h->d_sp, sizeof sp, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (sp.seq & 1u) grid = h->grid2;
        }
        launch_grid_unblock(h->stream, h->g, grid, static_cast<float4*>(h->stage));
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(out, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return {};
    };
    return finish(h, run());
}

int mpm_read_collider_pose(void* handle, int32_t c, float* M12, float* Minv12, float* dM12) {
    HANDLE_OR_FAIL(handle);
    if (c < 0 || c >= h->n_col) return finish(h, {MPM_ERR_VALUE, "collider index out of range"});
    auto run = [&]() -> Status {
        if (!h->d_poses) return {MPM_ERR_VALUE, "no substep has run since the colliders were set"};
        StepParams sp;
        CK(cudaMemcpyAsync(&sp, h->d_sp, sizeof sp, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        ColliderPose pose;
        CK(cudaMemcpyAsync(&pose, h->d_poses + sp.pose_base + c, sizeof pose, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (M12) std::memcpy(M12, pose.M, sizeof pose.M);
        if (Minv12) std::memcpy(Minv12, pose.Minv, sizeof pose.Minv);
        if (dM12) std::memcpy(dM12, pose.dM, sizeof pose.dM);
        return {};
    };
    return finish(h, run());
}

int mpm_launch_count(void* handle, int64_t* launches) {
    HANDLE_OR_FAIL(handle);
    if (!launches) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    *launches = h->launches;
    return MPM_OK;
}

int mpm_fp64_redo_lanes(void* handle, int64_t* lanes) {
    HANDLE_OR_FAIL(handle);
    unsigned int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, h->d_counters + 2 + kMaxMaterials, sizeof(unsigned int),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return finish(h, {MPM_ERR_CUDA, cudaGetErrorString(e)});
    if (lanes) *lanes = v;
    return MPM_OK;
}

int mpm_fp64_lanes(void* handle, int64_t* lanes) {
    HANDLE_OR_FAIL(handle);
    cudaError_t e = cudaMemcpyAsync(h->h_counters + 1, h->d_counters + 1, sizeof(unsigned int),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return finish(h, {MPM_ERR_CUDA, cudaGetErrorString(e)});
    if (lanes) *lanes = h->h_counters[1];
    return MPM_OK;
}


int mpm_read_begin(void* handle, float* x, float* v, float* C, float* F, float* Jp, int32_t* mat, int32_t* emitter) {
    HANDLE_OR_FAIL(handle);
    return finish(h, read_begin(h, x, v, C, F, Jp, mat, emitter));
}

int mpm_read_wait(void* handle) {
    HANDLE_OR_FAIL(handle);
    return finish(h, read_wait(h));
}

int mpm_host_alloc(int64_t bytes, void** ptr) {
    if (!ptr || bytes < 0) return finish(nullptr, {MPM_ERR_ARGUMENT, "bad arguments"});
    *ptr = nullptr;
    if (bytes == 0) return MPM_OK;
    if (cudaMallocHost(ptr, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return finish(nullptr, {MPM_ERR_MEMORY, "page-locked host allocation failed"});
    }
    return MPM_OK;
}

int mpm_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
    return MPM_OK;
}

int mpm_conservation(void* handle, double* out) {
    HANDLE_OR_FAIL(handle);
    if (!out) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    auto run = [&]() -> Status {
        TRY(ensure_stage(h, sizeof(double) * 9));
        double* d = static_cast<double*>(h->stage);
        launch_conservation(h->stream, h->P, h->d_mats, d);
        h->launches += 1;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(out, d, sizeof(double) * 9, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return {};
    };
    return finish(h, run());
}

int mpm_device_bytes(void* handle, int64_t* bytes) {
    HANDLE_OR_FAIL(handle);
    if (!bytes) return finish(h, {MPM_ERR_ARGUMENT, "null output"});
    *bytes = handle_device_bytes(h);
    return MPM_OK;
}

int mpm_batch_create(void** batch) {
    if (!batch) return finish(nullptr, {MPM_ERR_ARGUMENT, "null output"});
    *batch = new Batch();
    return MPM_OK;
}

int mpm_batch_destroy(void* batch) {
    batch_destroy(static_cast<Batch*>(batch));
    return MPM_OK;
}

const char* mpm_batch_last_error(void* batch) {
    return batch ? static_cast<Batch*>(batch)->err.c_str() : g_last_error.c_str();
}

#define BATCH_OR_FAIL(bv)                                                                      \
    Batch* b = static_cast<Batch*>(bv);                                                        \
    if (!b) return finish(nullptr, Status{MPM_ERR_ARGUMENT, "null batch"})

int mpm_batch_add(void* batch, void* handle) {
    BATCH_OR_FAIL(batch);
    Handle* h = static_cast<Handle*>(handle);
    if (!h) return finish_batch(b, {MPM_ERR_ARGUMENT, "null handle"});
    DeviceGuard guard(h->device);
    if (cudaError_t e = prepare_batch_kernels(); e != cudaSuccess)
        return finish_batch(b, {MPM_ERR_CUDA, cudaGetErrorString(e)});
    return finish_batch(b, batch_add(b, h));
}

int mpm_batch_remove(void* batch, void* handle) {
    BATCH_OR_FAIL(batch);
    Handle* h = static_cast<Handle*>(handle);
    if (!h) return finish_batch(b, {MPM_ERR_ARGUMENT, "null handle"});
    DeviceGuard guard(h->device);
    return finish_batch(b, batch_remove(b, h));
}

int mpm_batch_size(void* batch, int32_t* n) {
    BATCH_OR_FAIL(batch);
    if (!n) return finish_batch(b, {MPM_ERR_ARGUMENT, "null output"});
    *n = (int32_t)b->scenes.size();
    return MPM_OK;
}

int mpm_batch_advance(void* batch, const double* frame_dt, MpmAdvanceStats* stats) {
    BATCH_OR_FAIL(batch);
    if (b->scenes.empty()) return MPM_OK;
    if (!frame_dt || !stats) return finish_batch(b, {MPM_ERR_ARGUMENT, "null frame_dt or stats"});
    for (size_t s = 0; s < b->scenes.size(); ++s)
        if (!(frame_dt[s] > 0.0)) return finish_batch(b, {MPM_ERR_VALUE, "frame_dt must be positive"});
    DeviceGuard guard(b->device);
    return finish_batch(b, batch_advance(b, frame_dt, stats));
}

int mpm_batch_set_option(void* batch, int32_t option, int64_t value) {
    BATCH_OR_FAIL(batch);
    if (option == MPM_OPT_SORT_INTERVAL) {
        if (value < 0 || value > (1 << 30)) return finish_batch(b, {MPM_ERR_VALUE, "sort interval out of range"});
        b->sort_interval = (int)value;
        return MPM_OK;
    }
    if (option == MPM_OPT_G2P_VARIANT) {
        if (value != 0 && value != 1) return finish_batch(b, {MPM_ERR_VALUE, "G2P variant must be 0 or 1"});
        b->shape.g2p_variant = (int)value;
        batch_invalidate(b);
        return MPM_OK;
    }
    if (option == MPM_OPT_PDL) {
        b->shape.pdl = value != 0;
        batch_invalidate(b);
        return MPM_OK;
    }
    if (option == MPM_OPT_P2G_TILE) {
        b->shape.p2g_tile = value != 0;
        batch_invalidate(b);
        return MPM_OK;
    }
    if (option == MPM_OPT_P2G_MERGE) {
        b->shape.p2g_merge = value != 0;
        batch_invalidate(b);
        return MPM_OK;
    }
    if (option == MPM_OPT_P2G_GROUP) {
        if (value < 1 || value > 32 || (value & (value - 1)))
            return finish_batch(b, {MPM_ERR_VALUE, "P2G group must be a power of two from 1 to 32"});
        b->shape.p2g_group = (int)value;
        return MPM_OK;
    }
    if (option == MPM_OPT_LIST_CTAS) {
        if (value < 1 || value > (1 << 20)) return finish_batch(b, {MPM_ERR_VALUE, "work-list CTAs out of range"});
        b->shape.list_ctas = (unsigned int)value;
        batch_invalidate(b);
        return MPM_OK;
    }
    return finish_batch(b, {MPM_ERR_VALUE, "unknown option"});
}

int mpm_batch_get_stream(void* batch, void** stream) {
    BATCH_OR_FAIL(batch);
    if (!stream) return finish_batch(b, {MPM_ERR_ARGUMENT, "null output"});
    *stream = b->stream;
    return MPM_OK;
}

int mpm_batch_launch_count(void* batch, int64_t* launches) {
    BATCH_OR_FAIL(batch);
    if (!launches) return finish_batch(b, {MPM_ERR_ARGUMENT, "null output"});
    int64_t total = b->launches;
    for (Handle* h : b->scenes) total += h->launches;
    *launches = total;
    return MPM_OK;
}
}  // extern "C"
