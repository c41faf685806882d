// sm_103a kernels of the MLS-MPM substep and of the particle-state bookkeeping around it.
//
// One substep = step_begin (substep fraction + collider poses, on the device) -> clear -> P2G -> grid update
// (normalise, gravity, walls, mesh colliders) -> G2P (+ particle projection out of colliders). Every kernel
// reads dt and s from a StepParams record in device memory, so a captured graph of one substep replays
// for every substep of an advance.
#include <cuda_runtime.h>

#include "mpm_substep.cuh"
#include "mpm_internal.h"

namespace mpm {

// ------------------------------------------------------------------------------------------------------
// step_begin: advance the substep counter, set s = (k + 1) / steps (warp/solver.py:218-219), then the pose
// of every collider at s.
// ------------------------------------------------------------------------------------------------------
__global__ void k_step_begin(StepParams* sp, ColliderDev* cols, int n_col) {
    __shared__ float s_sh;
    if (threadIdx.x == 0) {
        StepParams p = *sp;
        if (p.steps > 0) {
            p.k += 1;
            p.s = (float)((double)(p.k + 1) / (double)p.steps);
            *sp = p;
        }
        s_sh = p.s;
    }
    __syncthreads();
    const float s = s_sh;
    const float inv_frame_dt = sp->inv_frame_dt;
    for (int c = threadIdx.x; c < n_col; c += blockDim.x) collider_pose_at(cols[c], s, inv_frame_dt);
}

__global__ void __launch_bounds__(256) k_p2g_scatter(Particles P, const Material* __restrict__ mats, GridDesc g,
                                                     const StepParams* __restrict__ sp, float4* __restrict__ grid,
                                                     unsigned int* fp64_lanes) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    p2g_particle(P, p, mats, g, sp->dt, grid, fp64_lanes);
}

// One CTA of 64 threads per 4x4x4 block; nodes without mass return at once.
__global__ void __launch_bounds__(64) k_grid_update(GridDesc g, float4* __restrict__ grid, const StepParams* __restrict__ sp,
                                                    const ColliderDev* __restrict__ cols, int n_col,
                                                    const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris) {
    const int64_t blk = blockIdx.x;
    const int l = threadIdx.x;
    const int bk = (int)(blk % g.nb[2]);
    const int bj = (int)((blk / g.nb[2]) % g.nb[1]);
    const int bi = (int)(blk / ((int64_t)g.nb[2] * g.nb[1]));
    const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
    grid_update_node(g, &grid[blk * 64 + l], idx, sp->dt, cols, n_col, nodes, tris);
}

__global__ void __launch_bounds__(256) k_g2p(Particles P, const Material* __restrict__ mats, GridDesc g,
                                             const StepParams* __restrict__ sp, const float4* __restrict__ grid,
                                             const ColliderDev* __restrict__ cols, int n_col,
                                             const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris,
                                             unsigned int* fp64_lanes) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    g2p_particle(P, p, mats, g, sp->dt, grid, cols, n_col, nodes, tris, fp64_lanes);
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
    dst.mat[q] = src.mat[p];
    dst.emitter[q] = src.emitter[p];
    dst.id[q] = new_id[src.id[p]];
}

// exclusive scan of int32 in three passes: per-CTA sums, one CTA over the sums, per-CTA scan + offset
constexpr int kScanTile = 1024;

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

__global__ void k_scan_tiles(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ tile_sums) {
    __shared__ int sh[32];
    int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
    int v = i < n ? in[i] : 0;
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

__global__ void k_scan_apply(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ tile_offsets,
                             int32_t* __restrict__ out) {
    __shared__ int sh[32];
    int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int ex = block_exclusive_scan(v, sh, nullptr);
    if (i < n) out[i] = ex + tile_offsets[blockIdx.x];
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
// launchers
// ------------------------------------------------------------------------------------------------------
static inline unsigned int blocks_for(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

void launch_step_begin(cudaStream_t st, StepParams* sp, ColliderDev* cols, int n_col) {
    k_step_begin<<<1, 32, 0, st>>>(sp, cols, n_col);
}

void launch_p2g(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                float4* grid, unsigned int* fp64) {
    if (P.n == 0) return;
    k_p2g_scatter<<<blocks_for(P.n, 256), 256, 0, st>>>(P, mats, g, sp, grid, fp64);
}

void launch_grid_update(cudaStream_t st, const GridDesc& g, float4* grid, const StepParams* sp, const ColliderDev* cols,
                        int n_col, const BvhNode* nodes, const MeshTri* tris) {
    int64_t nblk = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
    k_grid_update<<<(unsigned int)nblk, 64, 0, st>>>(g, grid, sp, cols, n_col, nodes, tris);
}

void launch_g2p(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                const float4* grid, const ColliderDev* cols, int n_col, const BvhNode* nodes, const MeshTri* tris,
                unsigned int* fp64) {
    if (P.n == 0) return;
    k_g2p<<<blocks_for(P.n, 256), 256, 0, st>>>(P, mats, g, sp, grid, cols, n_col, nodes, tris, fp64);
}

void launch_max_speed(cudaStream_t st, const Particles& P, unsigned int* out) {
    if (P.n == 0) return;
    unsigned int b = blocks_for(P.n, 256);
    if (b > 152 * 8) b = 152 * 8;
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
    k_scan_tiles<<<(unsigned int)tiles, kScanTile, 0, st>>>(in, n, tile_tmp);
    k_scan_sums<<<1, 1024, 0, st>>>(tile_tmp, tiles, total);
    k_scan_apply<<<(unsigned int)tiles, kScanTile, 0, st>>>(in, n, tile_tmp, out);
}

void launch_scatter_volume(cudaStream_t st, const Particles& P, const GridDesc& g, float* vol) {
    if (P.n == 0) return;
    k_scatter_volume<<<blocks_for(P.n, 256), 256, 0, st>>>(P, g, vol);
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
