// sm_103a kernels around the MLS-MPM substep (collider poses, CFL speed, particle-state I/O, removal,
// reorder, scans, occupancy, narrow-band voxel grids) and the launcher of one plain substep, whose kernels
// (mpm_substep_kernels.cuh) read dt and s from a StepParams record in device memory, so a captured graph
// of one substep replays for every substep of an advance.
#include <cuda_runtime.h>

#include <algorithm>

#include "mpm_internal.h"
#include "mpm_substep_kernels.cuh"
#include "mpm_tile.cuh"

namespace mpm {

unsigned int sm_count() {
    static unsigned int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < 64 && cached[dev]) return cached[dev];
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < 64) cached[dev] = (unsigned int)sms;
    return (unsigned int)sms;
}

// ------------------------------------------------------------------------------------------------------
// Collider poses of every substep of an advance, one thread per (substep, collider): substep k ends at
// s = (k + 1) / steps (warp/solver.py:218-219). steps == 0: one pose at the given s.
// ------------------------------------------------------------------------------------------------------
__global__ void k_collider_poses(const ColliderDev* __restrict__ cols, int n_col, ColliderPose* __restrict__ poses,
                                 int steps, float s_given, float inv_frame_dt) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)(steps > 0 ? steps : 1) * n_col;
    if (t >= total) return;
    int k = (int)(t / n_col), c = (int)(t % n_col);
    float s = steps > 0 ? (float)((double)(k + 1) / (double)steps) : s_given;
    collider_pose_at(cols[c], s, inv_frame_dt, poses[t]);
}

// exclusive scan of int32 in three passes: per-CTA sums, one CTA over the sums, per-CTA scan + offset.
// A CTA of kScanThreads threads covers kScanItems consecutive values per thread.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh_warp, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? sh_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh_warp[lane] = s;
    }
    __syncthreads();
    int incl = x + (wid > 0 ? sh_warp[wid - 1] : 0);
    if (total) *total = sh_warp[(blockDim.x >> 5) - 1];
    return incl - v;
}

// ------------------------------------------------------------------------------------------------------
// Periodic reorder by grid node: keys and ranks, (exclusive scan of the counts), order, permutation.
// ------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sort_keys(Particles P, GridDesc g, SortScratch ss, int64_t n_nodes) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int base[3];
    float fx;
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) inside &= stencil_axis((P.x[a][p] - g.origin[a]) * g.inv_dx, g.dims[a], &base[a], &fx);
    const int32_t key = (int32_t)(inside ? node_index(g, base[0], base[1], base[2]) : n_nodes);
    ss.key[p] = key;
    ss.rank[p] = (int32_t)atomicAdd(&ss.count[key], 1u);
}

__global__ void __launch_bounds__(256) k_sort_scatter(int64_t n, SortScratch ss) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    ss.order[ss.start[ss.key[p]] + ss.rank[p]] = (int32_t)p;
}

// dst[i] = src[order[i]] for every field: neighbouring threads of P2G and G2P then touch neighbouring grid
// nodes, so their reductions and gathers hit the same cache lines.
// The arena's fields are kParticleFields planes of `cap` words each, so the permutation is one gather per
// plane; all loads of a thread are issued before its stores, which the compiler could not reorder on its own
// (source and destination planes are plain pointers).

__global__ void __launch_bounds__(256) k_permute(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                                 int64_t cap, int64_t n, const int32_t* __restrict__ order) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t q = order[i];
    uint32_t w[kParticleFields];
#pragma unroll
    for (int f = 0; f < kParticleFields; ++f) w[f] = __ldg(&src[f * cap + q]);
#pragma unroll
    for (int f = 0; f < kParticleFields; ++f) dst[f * cap + i] = w[f];
}

// Stress of the particles [off, off + n) from their F and Jp (particles entering the arena).
__global__ void k_particle_stress(Particles P, int64_t off, int64_t n, const Material* __restrict__ mats,
                                  unsigned int* fp64_lanes) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    particle_stress(P, off + i, mats, fp64_lanes);
}

// ------------------------------------------------------------------------------------------------------
// max |v| (kernels.py:266-269); a NaN never wins, as in the oracle. Non-negative floats order like their bits.
// ------------------------------------------------------------------------------------------------------
__global__ void k_max_speed(Particles P, unsigned int* out) {
    float best = 0.0f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += (int64_t)gridDim.x * blockDim.x) {
        float vx = P.v[0][p], vy = P.v[1][p], vz = P.v[2][p];
        best = fmaxf(best, sqrtf(vx * vx + vy * vy + vz * vz));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(best));
}

// ------------------------------------------------------------------------------------------------------
// Conservation accumulators in FP64: total mass, momentum, mass-weighted position and kinetic energy
// (out[0], out[1..3], out[4..6], out[7]); per-CTA sums in shared memory, then one FP64 atomic per CTA and
// value. Non-finite particles are skipped and counted in out[8].
// ------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_conservation(Particles P, const Material* __restrict__ mats,
                                                      double* __restrict__ out) {
    __shared__ double sh[9][8];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += (int64_t)gridDim.x * blockDim.x) {
        const double m = mats[P.mat[p]].p_mass;
        const double x[3] = {P.x[0][p], P.x[1][p], P.x[2][p]}, v[3] = {P.v[0][p], P.v[1][p], P.v[2][p]};
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) {
            acc[8] += 1.0;
            continue;
        }
        acc[0] += m;
        for (int a = 0; a < 3; ++a) {
            acc[1 + a] += m * v[a];
            acc[4 + a] += m * x[a];
        }
        acc[7] += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < 9; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
        atomicAdd(&out[threadIdx.x], v);
    }
}

// ------------------------------------------------------------------------------------------------------
// Particle-state I/O: host-order arrays (N,3) / (N,3,3) / (N,) <-> SoA, ordered by the insertion id.
// ------------------------------------------------------------------------------------------------------
__global__ void k_state_in(Particles P, int64_t off, int64_t n, const float* __restrict__ x, const float* __restrict__ v,
                           const float* __restrict__ C, const float* __restrict__ F, const float* __restrict__ Jp,
                           const int32_t* __restrict__ mat, const int32_t* __restrict__ emitter) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t p = off + i;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P.x[a][p] = x[i * 3 + a];
        P.v[a][p] = v[i * 3 + a];
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        P.C[e][p] = C ? C[i * 9 + e] : 0.0f;
        P.F[e][p] = F ? F[i * 9 + e] : ((e % 4 == 0) ? 1.0f : 0.0f);
    }
    P.Jp[p] = Jp ? Jp[i] : 1.0f;
    P.mat[p] = mat[i];
    P.emitter[p] = emitter[i];
    P.id[p] = (int32_t)p;
}

__global__ void k_state_out(Particles P, float* __restrict__ x, float* __restrict__ v, float* __restrict__ C,
                            float* __restrict__ F, float* __restrict__ Jp, int32_t* __restrict__ mat,
                            int32_t* __restrict__ emitter) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int64_t d = P.id[p];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (x) x[d * 3 + a] = P.x[a][p];
        if (v) v[d * 3 + a] = P.v[a][p];
    }
    if (C)
#pragma unroll
        for (int e = 0; e < 9; ++e) C[d * 9 + e] = P.C[e][p];
    if (F)
#pragma unroll
        for (int e = 0; e < 9; ++e) F[d * 9 + e] = P.F[e][p];
    if (Jp) Jp[d] = P.Jp[p];
    if (mat) mat[d] = P.mat[p];
    if (emitter) emitter[d] = P.emitter[p];
}

// ------------------------------------------------------------------------------------------------------
// Removal of particles more than one cell past an open side (warp/solver.py:222-240), order preserved.
// ------------------------------------------------------------------------------------------------------
__global__ void k_flag_escaped(Particles P, EscapeBounds eb, int32_t* __restrict__ keep_phys,
                               int32_t* __restrict__ keep_by_id, unsigned int* __restrict__ removed_per_mat) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xa = P.x[a][p];
        if (eb.open_lo[a] && xa < eb.lo[a]) out = true;
        if (eb.open_hi[a] && xa > eb.hi[a]) out = true;
    }
    keep_phys[p] = out ? 0 : 1;
    keep_by_id[P.id[p]] = out ? 0 : 1;
    if (out) atomicAdd(&removed_per_mat[P.mat[p]], 1u);
}

__global__ void k_compact(Particles src, Particles dst, const int32_t* __restrict__ keep_phys,
                          const int32_t* __restrict__ dst_index, const int32_t* __restrict__ new_id) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= src.n || !keep_phys[p]) return;
    int64_t q = dst_index[p];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dst.x[a][q] = src.x[a][p];
        dst.v[a][q] = src.v[a][p];
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        dst.C[e][q] = src.C[e][p];
        dst.F[e][q] = src.F[e][p];
    }
    dst.Jp[q] = src.Jp[p];
#pragma unroll
    for (int e = 0; e < 6; ++e) dst.tau[e][q] = src.tau[e][p];
    dst.mat[q] = src.mat[p];
    dst.emitter[q] = src.emitter[p];
    dst.id[q] = new_id[src.id[p]];
#pragma unroll
    for (int e = 0; e < 4; ++e) dst.Vq[e][q] = src.Vq[e][p];
}


__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* __restrict__ in, int64_t n,
                                                              int32_t* __restrict__ tile_sums) {
    __shared__ int sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k * kScanThreads + threadIdx.x;
        v += i < n ? in[i] : 0;
    }
    int total;
    block_exclusive_scan(v, sh, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t* __restrict__ sums, int64_t m, int32_t* __restrict__ grand_total) {
    __shared__ int sh[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < m; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        int v = i < m ? sums[i] : 0;
        int total;
        int ex = block_exclusive_scan(v, sh, &total);
        if (i < m) sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

// Shared tile index with one pad word per 32, so thread t reading its values t * kScanItems + k hits 32
// different banks across a warp.
__device__ __forceinline__ int scan_pad(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t* __restrict__ in, int64_t n,
                                                              const int32_t* __restrict__ tile_offsets,
                                                              int32_t* __restrict__ out) {
    __shared__ int sh[32];
    __shared__ int tile[kScanTile + kScanTile / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int l = k * kScanThreads + threadIdx.x;
        tile[scan_pad(l)] = base + l < n ? in[base + l] : 0;
    }
    __syncthreads();
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += tile[scan_pad(threadIdx.x * kScanItems + k)];
    int run = block_exclusive_scan(sum, sh, nullptr) + tile_offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int l = scan_pad(threadIdx.x * kScanItems + k);
        const int x = tile[l];
        tile[l] = run;
        run += x;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int l = k * kScanThreads + threadIdx.x;
        if (base + l < n) out[base + l] = tile[scan_pad(l)];
    }
}

// ------------------------------------------------------------------------------------------------------
// Occupancy (kernels.py:272-298): B-spline splat of particle volume, then a nearest-node test.
// ------------------------------------------------------------------------------------------------------
__global__ void k_scatter_volume(Particles P, GridDesc g, float* __restrict__ vol) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int base[3];
    float fx, w[3][3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xp = (P.x[a][p] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx);
        bspline_weights(fx, w[a]);
    }
    if (!inside) return;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                atomicAdd(&vol[node_index(g, base[0] + i, base[1] + j, base[2] + k)], w[0][i] * w[1][j] * w[2][k] * g.p_vol);
}

__global__ void k_query_fill(GridDesc g, const float* __restrict__ vol, float cell_vol, int64_t m,
                             const float* __restrict__ pts, uint8_t* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int idx[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float gq = (pts[q * 3 + a] - g.origin[a]) * g.inv_dx;
        idx[a] = (int)copysignf(floorf(fabsf(gq) + 0.5f), gq);  // round half away from zero
        if (idx[a] < 0 || idx[a] >= g.dims[a]) inside = false;
    }
    out[q] = inside && vol[node_index(g, idx[0], idx[1], idx[2])] >= 0.5f * cell_vol ? 1 : 0;
}

// Deterministic mode: the same splat in fixed point, 2^-20 particle volumes per unit (integer sums do not
// depend on the order they arrive in; a node holds at most 27 x 8 x 2^20 < 2^28 units at 8 per cell).
constexpr float kVolUnits = 1048576.0f;  // 2^20

__global__ void k_scatter_volume_fixed(Particles P, GridDesc g, unsigned int* __restrict__ vol) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int base[3];
    float fx, w[3][3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xp = (P.x[a][p] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx);
        bspline_weights(fx, w[a]);
    }
    if (!inside) return;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                atomicAdd(&vol[node_index(g, base[0] + i, base[1] + j, base[2] + k)],
                          __float2uint_rn(w[0][i] * w[1][j] * w[2][k] * kVolUnits));
}

// threshold: 0.5 dx^3 in the same units (0.5 dx^3 / p_vol * 2^20)
__global__ void k_query_fill_fixed(GridDesc g, const unsigned int* __restrict__ vol, double threshold, int64_t m,
                                   const float* __restrict__ pts, uint8_t* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int idx[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float gq = (pts[q * 3 + a] - g.origin[a]) * g.inv_dx;
        idx[a] = (int)copysignf(floorf(fabsf(gq) + 0.5f), gq);  // round half away from zero
        if (idx[a] < 0 || idx[a] >= g.dims[a]) inside = false;
    }
    out[q] = inside && (double)vol[node_index(g, idx[0], idx[1], idx[2])] >= threshold ? 1 : 0;
}

// grid read-back: blocked layout -> C order (i, j, k) with 4 floats per node
__global__ void k_grid_unblock(GridDesc g, const float4* __restrict__ grid, float4* __restrict__ out) {
    int64_t n = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int k = (int)(q % g.dims[2]);
    int j = (int)((q / g.dims[2]) % g.dims[1]);
    int i = (int)(q / ((int64_t)g.dims[2] * g.dims[1]));
    out[q] = grid[node_index(g, i, j, k)];
}

// ------------------------------------------------------------------------------------------------------
// Narrow-band voxel grid of a collider: classify every voxel, then (after a scan) write candidate lists.
// ------------------------------------------------------------------------------------------------------
__global__ void k_sdf_classify(ColliderDev col, const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris,
                               int64_t n_vox, int max_cand, int2* __restrict__ cells, int32_t* __restrict__ counts) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_vox) return;
    float R2;
    int c = sdf_voxel_classify(col, nodes, tris, v, max_cand, &R2);
    cells[v] = make_int2(0, c);
    counts[v] = c > 0 ? c : 0;
}

__global__ void k_sdf_fill(ColliderDev col, const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris,
                           int64_t n_vox, int max_cand, int2* __restrict__ cells, const int32_t* __restrict__ starts,
                           int32_t* __restrict__ cand) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_vox) return;
    const int2 cell = cells[v];
    cells[v] = make_int2(starts[v], cell.y);
    if (cell.y <= 0) return;
    float R2, c[3], r;
    sdf_voxel_classify(col, nodes, tris, v, max_cand, &R2);  // the same radius as the classify pass
    sdf_voxel_center(col.sdf, v, c, &r);
    tris_within(nodes, tris, c, R2, cand + starts[v], cell.y);
}

// ------------------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------------------
static inline unsigned int blocks_for(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

void launch_collider_poses(cudaStream_t st, const ColliderDev* cols, int n_col, ColliderPose* poses, int steps,
                           float s_given, float inv_frame_dt) {
    if (n_col <= 0) return;
    int64_t total = (int64_t)(steps > 0 ? steps : 1) * n_col;
    k_collider_poses<<<blocks_for(total, 128), 128, 0, st>>>(cols, n_col, poses, steps, s_given, inv_frame_dt);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// The tile G2P's tensor maps for one scene: the arena as a 2-D tensor of floats (particle, plane: cap x 38,
// rows cap * 4 bytes apart), boxes of 256 x 1; the grid as a 4-D tensor (256 floats of a block, then the
// blocks along k, j, i), boxes of 2 x 2 x 2 blocks. Out-of-range box parts read as zero.
static bool encode_tile_maps(const SubstepArgs& a, TileMaps* m) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t pdim[2] = {(cuuint64_t)a.cap, (cuuint64_t)kParticleFields};
    const cuuint64_t pstride[1] = {(cuuint64_t)a.cap * sizeof(float)};
    const cuuint32_t pbox[2] = {(cuuint32_t)kTileChunk, 1u};
    const cuuint32_t ones[4] = {1u, 1u, 1u, 1u};
    if (fn(&m->planes, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, a.arena, pdim, pstride, pbox, ones,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const GridDesc& g = a.g;
    const cuuint64_t gdim[4] = {256u, (cuuint64_t)g.nb[2], (cuuint64_t)g.nb[1], (cuuint64_t)g.nb[0]};
    const cuuint64_t gstride[3] = {1024u, (cuuint64_t)g.nb[2] * 1024u, (cuuint64_t)g.nb[2] * g.nb[1] * 1024u};
    const cuuint32_t gbox[4] = {256u, 2u, 2u, 2u};
    return fn(&m->grid, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a.grid, gdim, gstride, gbox, ones,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The tile G2P (one grid, FP32 return mapping): persistent, at most three CTAs per SM. False when its tensor
// maps could not be encoded (the caller launches the plain G2P, which gives the same results).
static bool g2p_tile_launch(cudaStream_t st, const SubstepArgs& a, bool pdl, const OneScene& sc) {
    TileMaps maps;
    if (!encode_tile_maps(a, &maps)) return false;
    const int64_t chunks = (a.n + kTileChunk - 1) / kTileChunk;
    const unsigned int ctas = (unsigned int)std::min<int64_t>(chunks, (int64_t)sm_count() * 3);
    launch_step_kernel_smem(k_g2p_tile<3>, ctas, 256, kTileSmemBytes + 128, st, pdl, maps, sc);
    return true;
}

// The P2G build for a scene: chunk walk or not, with the fixed-point path (deterministic mode) or not, blocks
// flagged for the sweep or listed, leader sums merged along z or not.
static void (*p2g_build(bool walk, bool fixed, bool sweep, bool merge))(OneScene) {
    if (fixed) return walk ? k_p2g_scatter<OneScene, true, true, 2> : k_p2g_scatter<OneScene, false, true, 2>;
    if (sweep) return walk ? k_p2g_scatter<OneScene, true, false, 1> : k_p2g_scatter<OneScene, false, false, 1>;
    if (merge)
        return walk ? k_p2g_scatter<OneScene, true, false, 0, true> : k_p2g_scatter<OneScene, false, false, 0, true>;
    return walk ? k_p2g_scatter<OneScene, true, false, 0> : k_p2g_scatter<OneScene, false, false, 0>;
}

void launch_substep(cudaStream_t st, const SubstepArgs& a, const LaunchShape& shape, cudaEvent_t* ev, bool capturing) {
    const unsigned int list_ctas = shape.list_ctas ? shape.list_ctas : sm_count() * kCtasPerSm;
    const OneScene sc{a};
    // while a graph is being captured the records become event nodes that fire on every replay; with them
    // in place the kernels around them launch in plain stream order
    auto mark = [&](int i) {
        if (ev) cudaEventRecordWithFlags(ev[i], st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    };
    const bool pdl = shape.pdl != 0;
    // P2G and the plain G2P builds: one CTA per chunk of 256 particles, or (particles per thread above one)
    // one per ppt chunks, walking them; the FP64 and two-grid G2P builds always take one chunk per CTA
    const unsigned int chunks = blocks_for(a.n, 256);
    const bool walk = shape.ppt > 1;
    const unsigned int wctas = walk ? blocks_for(chunks, shape.ppt) : chunks;
    mark(0);
    launch_step_kernel(k_step_begin<OneScene>, 1, 1, st, pdl, sc);
    launch_step_kernel(k_clear_blocks<OneScene>, list_ctas, 256, st, pdl, sc);
    mark(1);
    if (a.n > 0) {
        if (shape.p2g_tile && !a.fixed)
            launch_step_kernel_smem(k_p2g_tile<OneScene>, blocks_for(a.n, 256), 256, kP2gTileBytes, st, pdl, sc);
        else
            launch_step_kernel(p2g_build(walk, a.fixed != nullptr, a.block_sweep != 0, shape.p2g_merge != 0), wctas, 256,
                               st, pdl, sc);
        if (a.block_sweep) {
            const int64_t nblk = (int64_t)a.g.nb[0] * a.g.nb[1] * a.g.nb[2];
            launch_step_kernel(k_list_blocks<OneScene>,
                               (unsigned int)std::min<int64_t>(blocks_for(nblk, 256), (int64_t)sm_count() * kCtasPerSm),
                               256, st, pdl, sc);
        }
    }
    mark(2);
    launch_step_kernel(k_grid_update<OneScene>, list_ctas, 256, st, pdl, sc);
    if (a.cd.n_col > 0) launch_step_kernel(k_grid_colliders<OneScene>, list_ctas, 128, st, pdl, sc);
    mark(3);
    if (a.n > 0) {
        if (a.grid2 && shape.g2p_variant == 1)  // two-grid mode (never with the FP64 clamp build)
            launch_step_kernel(k_g2p<OneScene, 1, false, true>, chunks, 256, st, pdl, sc);
        else if (a.grid2)
            launch_step_kernel(k_g2p<OneScene, 3, false, true>, chunks, 256, st, pdl, sc);
        else if (a.fp64_clamp && shape.g2p_variant == 1)  // the FP64 build at 128 registers
            launch_step_kernel(k_g2p<OneScene, 2, true>, chunks, 256, st, pdl, sc);
        else if (a.fp64_clamp)  // the FP64 build at 80 registers (the redo's working set spills)
            launch_step_kernel(k_g2p<OneScene, 3, true>, chunks, 256, st, pdl, sc);
        else if (shape.g2p_variant == 1)
            launch_step_kernel(walk ? k_g2p<OneScene, 1, false, false, true> : k_g2p<OneScene, 1>, wctas, 256, st, pdl,
                               sc);
        else if (shape.g2p_variant == 2 && g2p_tile_launch(st, a, pdl, sc))
            ;  // the tile G2P (its maps could not be made otherwise: then the plain build below)
        else if (shape.g2p_variant == 3 || walk)  // 80 registers, 3 CTAs of 256 per SM (the walk: this cap)
            launch_step_kernel(walk ? k_g2p<OneScene, 3, false, false, true> : k_g2p<OneScene, 3>, wctas, 256, st, pdl,
                               sc);
        else  // 64 registers, 4 CTAs of 256 per SM
            launch_step_kernel(k_g2p<OneScene, 4>, chunks, 256, st, pdl, sc);
    }
    if (a.cd.n_col > 0) launch_step_kernel(k_project_particles<OneScene>, list_ctas, 128, st, pdl, sc);
    mark(4);
}

void launch_sort(cudaStream_t st, const Particles& P, const GridDesc& g, const SortScratch& ss, int64_t n_nodes,
                 int32_t* scan_tmp, int64_t scan_cap) {
    if (P.n == 0) return;
    cudaMemsetAsync(ss.count, 0, sizeof(unsigned int) * (size_t)(n_nodes + 1), st);
    k_sort_keys<<<blocks_for(P.n, 256), 256, 0, st>>>(P, g, ss, n_nodes);
    launch_exclusive_scan(st, reinterpret_cast<const int32_t*>(ss.count), n_nodes + 1, ss.start, scan_tmp,
                          scan_tmp + scan_cap);
    k_sort_scatter<<<blocks_for(P.n, 256), 256, 0, st>>>(P.n, ss);
}

void launch_particle_stress(cudaStream_t st, const Particles& P, int64_t off, int64_t n, const Material* mats,
                            unsigned int* fp64) {
    if (n <= 0) return;
    k_particle_stress<<<blocks_for(n, 128), 128, 0, st>>>(P, off, n, mats, fp64);
}

void launch_permute(cudaStream_t st, const void* src_arena, void* dst_arena, int64_t cap, int64_t n,
                    const int32_t* order) {
    if (n == 0) return;
    k_permute<<<blocks_for(n, 256), 256, 0, st>>>(static_cast<const uint32_t*>(src_arena),
                                                 static_cast<uint32_t*>(dst_arena), cap, n, order);
}

void launch_sdf_classify(cudaStream_t st, const ColliderDev& col, const BvhNode* nodes, const MeshTri* tris,
                         int64_t n_vox, int max_cand, int2* cells, int32_t* counts) {
    k_sdf_classify<<<blocks_for(n_vox, 128), 128, 0, st>>>(col, nodes, tris, n_vox, max_cand, cells, counts);
}

void launch_sdf_fill(cudaStream_t st, const ColliderDev& col, const BvhNode* nodes, const MeshTri* tris, int64_t n_vox,
                     int max_cand, int2* cells, const int32_t* starts, int32_t* cand) {
    k_sdf_fill<<<blocks_for(n_vox, 128), 128, 0, st>>>(col, nodes, tris, n_vox, max_cand, cells, starts, cand);
}

// CTAs of the cooperative multi-substep kernel that fit on the device at once (all must be resident).
static int coop_resident_ctas() {
    static int cached[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 0;
    if (!cached[dev]) {
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_substeps_coop<1>, 256, 0) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        cached[dev] = per_sm * sms;
    }
    return cached[dev];
}

cudaError_t launch_substeps_coop(cudaStream_t st, const SubstepArgs& a, int reps, unsigned int* bar) {
    const int resident = coop_resident_ctas();
    if (resident <= 0) return cudaErrorCooperativeLaunchTooLarge;
    const int64_t chunks = std::max<int64_t>((a.n + 255) / 256, 1);
    const unsigned int grid = (unsigned int)std::min<int64_t>(chunks, resident);
    cudaError_t e = cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    OneScene sc{a};
    void* args[] = {&sc, &reps, &bar};
    return cudaLaunchCooperativeKernel((const void*)k_substeps_coop<1>, dim3(grid), dim3(256), args, 0, st);
}

// One barrier on its own, for checking the bounded wait (bar as for k_substeps_coop).
__global__ void k_barrier_selftest(unsigned int* bar) { grid_barrier(bar, bar + 2); }

cudaError_t barrier_selftest(cudaStream_t st, bool stall, unsigned int* bar, unsigned int* timed_out) {
    // stall: the arrival count starts so high that no CTA is ever the last to arrive
    const unsigned int init[3] = {stall ? 0x80000000u : 0u, 0u, 0u};
    cudaError_t e = cudaMemcpyAsync(bar, init, sizeof(init), cudaMemcpyHostToDevice, st);
    void* args[] = {&bar};
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(2), dim3(32), args, 0, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(timed_out, bar + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

cudaError_t prepare_substep_kernels() {
    cudaError_t e =
        cudaFuncSetAttribute(k_p2g_tile<OneScene>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP2gTileBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_g2p_tile<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kTileSmemBytes + 128));
    return e;
}


int substep_kernel_count(const SubstepArgs& a) {
    return 3 + (a.n > 0 ? 2 + (a.block_sweep ? 1 : 0) : 0) + (a.cd.n_col > 0 ? 2 : 0);
}


void launch_max_speed(cudaStream_t st, const Particles& P, unsigned int* out) {
    if (P.n == 0) return;
    unsigned int b = blocks_for(P.n, 256);
    b = std::min(b, sm_count() * kCtasPerSm);
    k_max_speed<<<b, 256, 0, st>>>(P, out);
}

void launch_state_in(cudaStream_t st, const Particles& P, int64_t off, int64_t n, const float* x, const float* v,
                     const float* C, const float* F, const float* Jp, const int32_t* mat, const int32_t* emitter) {
    if (n == 0) return;
    k_state_in<<<blocks_for(n, 256), 256, 0, st>>>(P, off, n, x, v, C, F, Jp, mat, emitter);
}

void launch_state_out(cudaStream_t st, const Particles& P, float* x, float* v, float* C, float* F, float* Jp,
                      int32_t* mat, int32_t* emitter) {
    if (P.n == 0) return;
    k_state_out<<<blocks_for(P.n, 256), 256, 0, st>>>(P, x, v, C, F, Jp, mat, emitter);
}

void launch_flag_escaped(cudaStream_t st, const Particles& P, const EscapeBounds& eb, int32_t* keep_phys,
                         int32_t* keep_by_id, unsigned int* removed_per_mat) {
    if (P.n == 0) return;
    k_flag_escaped<<<blocks_for(P.n, 256), 256, 0, st>>>(P, eb, keep_phys, keep_by_id, removed_per_mat);
}

void launch_compact(cudaStream_t st, const Particles& src, const Particles& dst, const int32_t* keep_phys,
                    const int32_t* dst_index, const int32_t* new_id) {
    if (src.n == 0) return;
    k_compact<<<blocks_for(src.n, 256), 256, 0, st>>>(src, dst, keep_phys, dst_index, new_id);
}

int64_t scan_tile_count(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

void launch_exclusive_scan(cudaStream_t st, const int32_t* in, int64_t n, int32_t* out, int32_t* tile_tmp,
                           int32_t* total) {
    if (n == 0) return;
    int64_t tiles = scan_tile_count(n);
    k_scan_tiles<<<(unsigned int)tiles, kScanThreads, 0, st>>>(in, n, tile_tmp);
    k_scan_sums<<<1, 1024, 0, st>>>(tile_tmp, tiles, total);
    k_scan_apply<<<(unsigned int)tiles, kScanThreads, 0, st>>>(in, n, tile_tmp, out);
}

void launch_scatter_volume(cudaStream_t st, const Particles& P, const GridDesc& g, float* vol) {
    if (P.n == 0) return;
    k_scatter_volume<<<blocks_for(P.n, 256), 256, 0, st>>>(P, g, vol);
}

void launch_scatter_volume_fixed(cudaStream_t st, const Particles& P, const GridDesc& g, unsigned int* vol) {
    if (P.n == 0) return;
    k_scatter_volume_fixed<<<blocks_for(P.n, 256), 256, 0, st>>>(P, g, vol);
}

void launch_query_fill_fixed(cudaStream_t st, const GridDesc& g, const unsigned int* vol, double cell_vol, int64_t m,
                             const float* pts, uint8_t* out) {
    if (m == 0) return;
    const double threshold = 0.5 * cell_vol / (double)g.p_vol * (double)kVolUnits;
    k_query_fill_fixed<<<blocks_for(m, 256), 256, 0, st>>>(g, vol, threshold, m, pts, out);
}

void launch_conservation(cudaStream_t st, const Particles& P, const Material* mats, double* out) {
    cudaMemsetAsync(out, 0, sizeof(double) * 9, st);
    if (P.n == 0) return;
    k_conservation<<<std::min<unsigned int>(blocks_for(P.n, 256), sm_count() * kCtasPerSm), 256, 0, st>>>(P, mats, out);
}

void launch_grid_unblock(cudaStream_t st, const GridDesc& g, const float4* grid, float4* out) {
    int64_t n = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
    k_grid_unblock<<<blocks_for(n, 256), 256, 0, st>>>(g, grid, out);
}

void launch_query_fill(cudaStream_t st, const GridDesc& g, const float* vol, float cell_vol, int64_t m,
                       const float* pts, uint8_t* out) {
    if (m == 0) return;
    k_query_fill<<<blocks_for(m, 256), 256, 0, st>>>(g, vol, cell_vol, m, pts, out);
}

}  // namespace mpm
