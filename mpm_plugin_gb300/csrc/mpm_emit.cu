// Volume sampling of emitter meshes on the device: the lattice points inside a closed mesh by z-ray parity
// per (x, y) lattice column (mpm_core/geometry.py:89-151), before the seeded jitter the caller adds.
//
// Every floating-point operation that decides a point is the reference's, in FP64 and in its order, with
// each operation rounded on its own (no fused multiply-adds), so the same points come out in the same
// order: per triangle its column range from the xy bounding box (geometry.py:111-117) and its signed xy
// area (118-120); per covered column the barycentric test of the nudged column centre and the crossing
// height (121-129); per column the crossings sorted and the lattice heights with an odd number of
// crossings below them (138-147); columns in increasing index, heights increasing (136-137, 141-147).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/mpm_gb300.h"
#include "mpm_internal.h"

namespace {

struct LatticeArgs {
    const double* tri;  // (T, 3, 3)
    int64_t n_tris;
    const double* xs;
    const double* ys;
    const double* zs;
    int nx, ny, nz;
    double spacing, nudge_x, nudge_y;
    long long first_x, first_y;
};

struct TriRange {
    int i0, i1, j0, j1;  // columns covered (empty when i1 < i0)
    double area;
};

__device__ __forceinline__ TriRange tri_range(const LatticeArgs& L, int64_t t) {
    const double* v = L.tri + t * 9;
    TriRange r;
    const double tmin0 = fmin(fmin(v[0], v[3]), v[6]), tmin1 = fmin(fmin(v[1], v[4]), v[7]);
    const double tmax0 = fmax(fmax(v[0], v[3]), v[6]), tmax1 = fmax(fmax(v[1], v[4]), v[7]);
    const long long i0 = (long long)ceil(__dsub_rn(__ddiv_rn(__dsub_rn(tmin0, L.nudge_x), L.spacing), 0.5)) - L.first_x;
    const long long i1 = (long long)floor(__dsub_rn(__ddiv_rn(__dsub_rn(tmax0, L.nudge_x), L.spacing), 0.5)) - L.first_x;
    const long long j0 = (long long)ceil(__dsub_rn(__ddiv_rn(__dsub_rn(tmin1, L.nudge_y), L.spacing), 0.5)) - L.first_y;
    const long long j1 = (long long)floor(__dsub_rn(__ddiv_rn(__dsub_rn(tmax1, L.nudge_y), L.spacing), 0.5)) - L.first_y;
    r.i0 = (int)max(i0, 0ll);
    r.i1 = (int)min(i1, (long long)L.nx - 1);
    r.j0 = (int)max(j0, 0ll);
    r.j1 = (int)min(j1, (long long)L.ny - 1);
    // (b0 - a0) (c1 - a1) - (b1 - a1) (c0 - a0)
    r.area = __dsub_rn(__dmul_rn(__dsub_rn(v[3], v[0]), __dsub_rn(v[7], v[1])),
                       __dmul_rn(__dsub_rn(v[4], v[1]), __dsub_rn(v[6], v[0])));
    if (r.area == 0.0) r.i1 = r.i0 - 1;  // vertical triangle: rays never cross it
    return r;
}

// Per triangle: +1 on every column its range covers (pass 0), or its index into the column's list (pass 1).
__global__ void k_tri_columns(LatticeArgs L, unsigned int* __restrict__ count, const int32_t* __restrict__ start,
                              unsigned int* __restrict__ fill, int32_t* __restrict__ pairs, int pass) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.n_tris) return;
    const TriRange r = tri_range(L, t);
    for (int i = r.i0; i <= r.i1; ++i)
        for (int j = r.j0; j <= r.j1; ++j) {
            const int64_t col = (int64_t)i * L.ny + j;
            if (pass == 0) {
                atomicAdd(&count[col], 1u);
            } else {
                const unsigned int k = atomicAdd(&fill[col], 1u);
                pairs[start[col] + k] = (int32_t)t;
            }
        }
}

// Per column: crossings of its listed triangles, sorted; then the lattice heights inside (pass 0 counts
// them, pass 1 writes the points at out_start).
__global__ void k_column_points(LatticeArgs L, const unsigned int* __restrict__ count, const int32_t* __restrict__ start,
                                const int32_t* __restrict__ pairs, double* __restrict__ zbuf,
                                int32_t* __restrict__ inside, const int32_t* __restrict__ out_start,
                                double* __restrict__ out, int pass) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (int64_t)L.nx * L.ny) return;
    const int i = (int)(col / L.ny), j = (int)(col % L.ny);
    const int64_t s = start[col];
    const int n = (int)count[col];
    int hits = 0;
    if (pass == 0) {
        const double px = __dadd_rn(L.xs[i], L.nudge_x), py = __dadd_rn(L.ys[j], L.nudge_y);
        for (int k = 0; k < n; ++k) {
            const double* v = L.tri + (int64_t)pairs[s + k] * 9;
            const double area = __dsub_rn(__dmul_rn(__dsub_rn(v[3], v[0]), __dsub_rn(v[7], v[1])),
                                          __dmul_rn(__dsub_rn(v[4], v[1]), __dsub_rn(v[6], v[0])));
            // w0 = ((b0 - px)(c1 - py) - (b1 - py)(c0 - px)) / area, w1 likewise from c and a
            const double w0 = __ddiv_rn(__dsub_rn(__dmul_rn(__dsub_rn(v[3], px), __dsub_rn(v[7], py)),
                                                  __dmul_rn(__dsub_rn(v[4], py), __dsub_rn(v[6], px))), area);
            const double w1 = __ddiv_rn(__dsub_rn(__dmul_rn(__dsub_rn(v[6], px), __dsub_rn(v[1], py)),
                                                  __dmul_rn(__dsub_rn(v[7], py), __dsub_rn(v[0], px))), area);
            const double w2 = __dsub_rn(__dsub_rn(1.0, w0), w1);
            if (w0 >= 0.0 && w1 >= 0.0 && w2 >= 0.0)
                zbuf[s + hits++] = __dadd_rn(__dadd_rn(__dmul_rn(w0, v[2]), __dmul_rn(w1, v[5])), __dmul_rn(w2, v[8]));
        }
        for (int a = 1; a < hits; ++a) {  // insertion sort of the (few) crossings
            const double z = zbuf[s + a];
            int b = a - 1;
            while (b >= 0 && zbuf[s + b] > z) {
                zbuf[s + b + 1] = zbuf[s + b];
                --b;
            }
            zbuf[s + b + 1] = z;
        }
        // count the crossings into the column's first slot of `inside` (hits) and the points (inside)
        int h = 0, pts = 0;
        for (int q = 0; q < L.nz; ++q) {
            while (h < hits && zbuf[s + h] < L.zs[q]) ++h;  // crossings strictly below (searchsorted, left)
            pts += h & 1;
        }
        inside[col] = pts;
        inside[(int64_t)L.nx * L.ny + col] = hits;
        return;
    }
    hits = inside[(int64_t)L.nx * L.ny + col];
    int64_t o = out_start[col];
    int h = 0;
    for (int q = 0; q < L.nz; ++q) {
        while (h < hits && zbuf[s + h] < L.zs[q]) ++h;
        if (h & 1) {
            out[o * 3 + 0] = L.xs[i];
            out[o * 3 + 1] = L.ys[j];
            out[o * 3 + 2] = L.zs[q];
            ++o;
        }
    }
}

int fail(int code, const std::string& msg) {
    mpm::set_last_error(msg);
    return code;
}

struct DeviceBuffers {
    void* p[8] = {};
    ~DeviceBuffers() {
        for (void* q : p) cudaFree(q);
    }
};

}  // namespace

extern "C" int mpm_volume_lattice(const double* tri, int64_t n_tris, const double* xs, int32_t nx, const double* ys,
                                  int32_t ny, const double* zs, int32_t nz, double spacing, const double nudge[2],
                                  int64_t first_x, int64_t first_y, int32_t device, double* out, int64_t capacity,
                                  int64_t* n_out) {
    if (!n_out || n_tris < 0 || nx < 0 || ny < 0 || nz < 0 || !nudge || !(spacing > 0.0) ||
        (n_tris > 0 && !tri) || (nx > 0 && !xs) || (ny > 0 && !ys) || (nz > 0 && !zs))
        return fail(MPM_ERR_ARGUMENT, "bad arguments");
    *n_out = 0;
    const int64_t cols = (int64_t)nx * ny;
    if (n_tris == 0 || cols == 0 || nz == 0) return MPM_OK;
    if (cols > (int64_t)1 << 30) return fail(MPM_ERR_VALUE, "lattice has too many columns");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) cudaSetDevice(device);
    cudaStream_t st = nullptr;
    DeviceBuffers buf;
    auto run = [&]() -> cudaError_t {
        cudaError_t e;
        double *d_tri, *d_xs, *d_ys, *d_zs;
        unsigned int *d_count, *d_fill;
        int32_t *d_start, *d_inside;
        if ((e = cudaMalloc(&buf.p[0], sizeof(double) * 9 * (size_t)n_tris + sizeof(double) * (size_t)(nx + ny + nz))))
            return e;
        d_tri = static_cast<double*>(buf.p[0]);
        d_xs = d_tri + 9 * n_tris;
        d_ys = d_xs + nx;
        d_zs = d_ys + ny;
        const int64_t tiles = mpm::scan_tile_count(cols + 1) + 2;
        if ((e = cudaMalloc(&buf.p[1], sizeof(int32_t) * (size_t)(cols * 6 + 8 + tiles)))) return e;
        d_count = static_cast<unsigned int*>(buf.p[1]);
        d_fill = d_count + cols;
        d_start = reinterpret_cast<int32_t*>(d_fill + cols);         // cols + 1
        d_inside = d_start + cols + 1;                                // 2 * cols (points, then crossings)
        int32_t* d_out_start = d_inside + 2 * cols;                   // cols + 1
        int32_t* d_tmp = d_out_start + cols + 1;
        if ((e = cudaMemcpy(d_tri, tri, sizeof(double) * 9 * (size_t)n_tris, cudaMemcpyHostToDevice))) return e;
        if ((e = cudaMemcpy(d_xs, xs, sizeof(double) * nx, cudaMemcpyHostToDevice))) return e;
        if ((e = cudaMemcpy(d_ys, ys, sizeof(double) * ny, cudaMemcpyHostToDevice))) return e;
        if ((e = cudaMemcpy(d_zs, zs, sizeof(double) * nz, cudaMemcpyHostToDevice))) return e;
        if ((e = cudaMemset(d_count, 0, sizeof(unsigned int) * 2 * (size_t)cols))) return e;
        LatticeArgs L{d_tri, n_tris, d_xs, d_ys, d_zs, nx, ny, nz, spacing, nudge[0], nudge[1],
                      (long long)first_x, (long long)first_y};
        const unsigned int tb = (unsigned int)((n_tris + 127) / 128), cb = (unsigned int)((cols + 127) / 128);
        k_tri_columns<<<tb, 128, 0, st>>>(L, d_count, nullptr, nullptr, nullptr, 0);
        mpm::launch_exclusive_scan(st, reinterpret_cast<const int32_t*>(d_count), cols, d_start, d_tmp, d_start + cols);
        if ((e = cudaGetLastError())) return e;
        int32_t pairs_total = 0;
        if ((e = cudaMemcpy(&pairs_total, d_start + cols, sizeof(int32_t), cudaMemcpyDeviceToHost))) return e;
        if ((e = cudaMalloc(&buf.p[2], sizeof(int32_t) * (size_t)std::max(pairs_total, 1) + 16 +
                                           sizeof(double) * (size_t)std::max(pairs_total, 1))))
            return e;
        int32_t* d_pairs = static_cast<int32_t*>(buf.p[2]);
        double* d_z = reinterpret_cast<double*>(static_cast<char*>(buf.p[2]) +
                                                ((sizeof(int32_t) * (size_t)std::max(pairs_total, 1) + 15) & ~(size_t)15));
        k_tri_columns<<<tb, 128, 0, st>>>(L, d_count, d_start, d_fill, d_pairs, 1);
        k_column_points<<<cb, 128, 0, st>>>(L, d_count, d_start, d_pairs, d_z, d_inside, nullptr, nullptr, 0);
        mpm::launch_exclusive_scan(st, d_inside, cols, d_out_start, d_tmp, d_out_start + cols);
        if ((e = cudaGetLastError())) return e;
        int32_t total = 0;
        if ((e = cudaMemcpy(&total, d_out_start + cols, sizeof(int32_t), cudaMemcpyDeviceToHost))) return e;
        *n_out = total;
        if (!out || capacity < total || total == 0) return cudaSuccess;
        if ((e = cudaMalloc(&buf.p[3], sizeof(double) * 3 * (size_t)total))) return e;
        double* d_out = static_cast<double*>(buf.p[3]);
        k_column_points<<<cb, 128, 0, st>>>(L, d_count, d_start, d_pairs, d_z, d_inside, d_out_start, d_out, 1);
        if ((e = cudaGetLastError())) return e;
        return cudaMemcpy(out, d_out, sizeof(double) * 3 * (size_t)total, cudaMemcpyDeviceToHost);
    };
    cudaError_t e = run();
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? MPM_ERR_MEMORY : MPM_ERR_CUDA, cudaGetErrorString(e));
    }
    return MPM_OK;
}
