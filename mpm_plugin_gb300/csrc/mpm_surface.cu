// Surfacing of one particle set on the GPU (the reference's mpm_surface/field.py:35-142): density and
// momentum splat with a cubic B-spline kernel, normalisation, marching cubes with shared vertices, and
// trilinear vertex velocities. Field layout: a dense C-order grid (k fastest), one float4 per node
// (momentum xyz, density) for the splat, then velocity xyz in place and the normalised density alongside.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <string>

#include "../../include/mpm_gb300.h"
#include "mpm_internal.h"
#include "mpm_mc_table.h"

namespace mpm {

__constant__ int8_t c_mc_ntri[256];
__constant__ int8_t c_mc_edge[256][kMcMaxTris * 3];

struct SurfGrid {
    int d0, d1, d2;
    __device__ __forceinline__ int64_t at(int i, int j, int k) const { return ((int64_t)i * d1 + j) * d2 + k; }
    __device__ __forceinline__ int64_t count() const { return (int64_t)d0 * d1 * d2; }
};

// Unnormalised cubic B-spline on q in [0, 1) (field.py:24-32).
__device__ __forceinline__ float cubic_kernel(float q) {
    if (q < 0.5f) return 1.0f - 6.0f * q * q + 6.0f * q * q * q;
    if (q < 1.0f) {
        const float t = 1.0f - q;
        return 2.0f * t * t * t;
    }
    return 0.0f;
}

// One particle's kernel-weighted density and momentum over the nodes of its box (field.py:35-57). Rows of
// the box are limited to the span the kernel's sphere can reach (one node of slack either side, the weight
// test decides), which skips the box corners without changing which nodes receive anything.
__global__ void __launch_bounds__(256) k_surf_splat(int64_t n, const float* __restrict__ x,
                                                    const float* __restrict__ v, float o0, float o1, float o2,
                                                    float inv_cell, float cell, float h, SurfGrid G,
                                                    float4* __restrict__ acc) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float g0 = (x[3 * p] - o0) * inv_cell, g1 = (x[3 * p + 1] - o1) * inv_cell,
                g2 = (x[3 * p + 2] - o2) * inv_cell;
    const float vx = v[3 * p], vy = v[3 * p + 1], vz = v[3 * p + 2];
    const float r = h * inv_cell;
    const int lo_i = max((int)floorf(g0 - r), 0), lo_j = max((int)floorf(g1 - r), 0),
              lo_k = max((int)floorf(g2 - r), 0);
    const int hi_i = min((int)ceilf(g0 + r), G.d0 - 1), hi_j = min((int)ceilf(g1 + r), G.d1 - 1),
              hi_k = min((int)ceilf(g2 + r), G.d2 - 1);
    const float r2 = (r + 1.0f) * (r + 1.0f);
    for (int i = lo_i; i <= hi_i; ++i) {
        const float di = (float)i - g0;
        for (int j = lo_j; j <= hi_j; ++j) {
            const float dj = (float)j - g1;
            const float rem = r2 - di * di - dj * dj;
            if (!(rem > 0.0f)) continue;
            const float span = sqrtf(rem);
            const int k0 = max(lo_k, (int)floorf(g2 - span)), k1 = min(hi_k, (int)ceilf(g2 + span));
            for (int k = k0; k <= k1; ++k) {
                const float dk = (float)k - g2;
                const float d = sqrtf(di * di + dj * dj + dk * dk) * cell;
                const float w = cubic_kernel(d / h);
                if (w > 0.0f) {
                    float4* a = &acc[G.at(i, j, k)];
                    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(w * vx),
                                 "f"(w * vy), "f"(w * vz), "f"(w)
                                 : "memory");
                }
            }
        }
    }
}

// Momentum to velocity where there is density; density to a fraction of the rest density (field.py:60-66).
__global__ void k_surf_normalize(int64_t N, float4* __restrict__ acc, float* __restrict__ dens, float inv_rest) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= N) return;
    float4 a = acc[q];
    const float d = a.w;
    if (d > 0.0f) {
        a.x = a.x / d;
        a.y = a.y / d;
        a.z = a.z / d;
        acc[q] = a;
    }
    dens[q] = d * inv_rest;
}

// Edges from each node towards +x, +y, +z that cross the iso level: bit a of bits[q]; cnt[q] = their count.
__global__ void k_surf_edges(SurfGrid G, const float* __restrict__ dens, float iso, uint8_t* __restrict__ bits,
                             int32_t* __restrict__ cnt) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.count()) return;
    const int k = (int)(q % G.d2), j = (int)((q / G.d2) % G.d1), i = (int)(q / ((int64_t)G.d2 * G.d1));
    const bool in0 = dens[q] > iso;
    unsigned int b = 0;
    if (i + 1 < G.d0 && (dens[G.at(i + 1, j, k)] > iso) != in0) b |= 1u;
    if (j + 1 < G.d1 && (dens[G.at(i, j + 1, k)] > iso) != in0) b |= 2u;
    if (k + 1 < G.d2 && (dens[G.at(i, j, k + 1)] > iso) != in0) b |= 4u;
    bits[q] = (uint8_t)b;
    cnt[q] = __popc(b);
}

// Velocity at a point in grid index units: trilinear over the cell, indices clamped (field.py:69-89).
__device__ __forceinline__ float3 sample_velocity(SurfGrid G, const float4* __restrict__ vel, float3 g) {
    const int i = min(max((int)floorf(g.x), 0), G.d0 - 2), j = min(max((int)floorf(g.y), 0), G.d1 - 2),
              k = min(max((int)floorf(g.z), 0), G.d2 - 2);
    const float fx = g.x - (float)i, fy = g.y - (float)j, fz = g.z - (float)k;
    float3 acc = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const float wa = a == 0 ? 1.0f - fx : fx;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const float wb = b == 0 ? 1.0f - fy : fy;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float wc = c == 0 ? 1.0f - fz : fz;
                const float w = wa * wb * wc;
                const float4 u = vel[G.at(i + a, j + b, k + c)];
                acc.x += w * u.x;
                acc.y += w * u.y;
                acc.z += w * u.z;
            }
        }
    }
    return acc;
}

// The vertex on each crossing edge (linear interpolation of the field to the iso level), in node order then
// axis order, and its velocity.
__global__ void k_surf_verts(SurfGrid G, const float* __restrict__ dens, const float4* __restrict__ vel, float iso,
                             const uint8_t* __restrict__ bits, const int32_t* __restrict__ voff,
                             float* __restrict__ verts, float* __restrict__ vvel) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.count()) return;
    const unsigned int b = bits[q];
    if (!b) return;
    const int k = (int)(q % G.d2), j = (int)((q / G.d2) % G.d1), i = (int)(q / ((int64_t)G.d2 * G.d1));
    int64_t id = voff[q];
    const float d0 = dens[q];
    for (int a = 0; a < 3; ++a) {
        if (!((b >> a) & 1u)) continue;
        const int64_t nb = G.at(i + (a == 0), j + (a == 1), k + (a == 2));
        const float t = (iso - d0) / (dens[nb] - d0);
        float3 p = make_float3((float)i, (float)j, (float)k);
        if (a == 0) p.x += t;
        if (a == 1) p.y += t;
        if (a == 2) p.z += t;
        const float3 u = sample_velocity(G, vel, p);
        verts[3 * id] = p.x;
        verts[3 * id + 1] = p.y;
        verts[3 * id + 2] = p.z;
        vvel[3 * id] = u.x;
        vvel[3 * id + 1] = u.y;
        vvel[3 * id + 2] = u.z;
        ++id;
    }
}

// Case of each cell (indexed by its lowest node) and its triangle count.
__global__ void k_surf_cells(SurfGrid G, const float* __restrict__ dens, float iso, uint8_t* __restrict__ cube,
                             int32_t* __restrict__ tcnt) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.count()) return;
    const int k = (int)(q % G.d2), j = (int)((q / G.d2) % G.d1), i = (int)(q / ((int64_t)G.d2 * G.d1));
    int m = 0;
    if (i + 1 < G.d0 && j + 1 < G.d1 && k + 1 < G.d2) {
#pragma unroll
        for (int c = 0; c < 8; ++c)
            if (dens[G.at(i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2))] > iso) m |= 1 << c;
    }
    cube[q] = (uint8_t)m;
    tcnt[q] = c_mc_ntri[m];
}

// Triangles of each cell from the case table; an edge's vertex is found at the node that owns the edge.
__global__ void k_surf_tris(SurfGrid G, const uint8_t* __restrict__ cube, const int32_t* __restrict__ toff,
                            const uint8_t* __restrict__ bits, const int32_t* __restrict__ voff,
                            int32_t* __restrict__ tris) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.count()) return;
    const int m = cube[q];
    const int nt = c_mc_ntri[m];
    if (!nt) return;
    const int k = (int)(q % G.d2), j = (int)((q / G.d2) % G.d1), i = (int)(q / ((int64_t)G.d2 * G.d1));
    int64_t t = toff[q];
    for (int s = 0; s < nt; ++s, ++t) {
        for (int c = 0; c < 3; ++c) {
            const int e = c_mc_edge[m][3 * s + c];
            const int a = e >> 2, sb = e & 3, u = (a + 1) % 3, w = (a + 2) % 3;
            int o[3] = {0, 0, 0};
            o[u] = sb & 1;
            o[w] = sb >> 1;
            const int64_t owner = G.at(i + o[0], j + o[1], k + o[2]);
            tris[3 * t + c] = voff[owner] + __popc((unsigned int)bits[owner] & ((1u << a) - 1u));
        }
    }
}

// Per-axis bounds of the particle positions: min and max as order-preserving integers, and a flag per axis
// for a NaN (numpy's min and max return NaN then, and so does mpm_surface_upload).
__device__ __forceinline__ int ordered_int(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float from_ordered_int(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_surf_bounds(int64_t n, const float* __restrict__ x, int* __restrict__ out) {
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    unsigned int nan = 0;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float f = x[3 * p + a];
            if (f != f) {
                nan |= 1u << a;
            } else {
                const int o = ordered_int(f);
                lo[a] = min(lo[a], o);
                hi[a] = max(hi[a], o);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = __reduce_min_sync(0xffffffffu, lo[a]);
        hi[a] = __reduce_max_sync(0xffffffffu, hi[a]);
    }
    nan = __reduce_or_sync(0xffffffffu, nan);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&out[a], lo[a]);
            atomicMax(&out[3 + a], hi[a]);
        }
        if (nan) atomicOr(&out[6], (int)nan);
    }
}

namespace {

// Device buffers that only grow, kept from frame to frame.
struct Pool {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        const size_t want = need + need / 4 + 256;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct Surfacer {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    Pool x, v, acc, dens, bits, cube, cnt, voff, tcnt, toff, tile, small, verts, vvel, tris;
    int64_t n = 0, n_nodes = 0, n_verts = 0, n_tris = 0;
    bool built = false;
    void release() {
        for (Pool* q : {&x, &v, &acc, &dens, &bits, &cube, &cnt, &voff, &tcnt, &toff, &tile, &small, &verts, &vvel,
                        &tris})
            q->release();
        n = n_nodes = n_verts = n_tris = 0;
        built = false;
    }
};

bool g_table_ready[64] = {};

int surf_fail(Surfacer* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}

unsigned int blocks_of(int64_t n) { return (unsigned int)((n + 255) / 256); }

struct DeviceScope {
    int prev = 0;
    explicit DeviceScope(int d) {
        cudaGetDevice(&prev);
        cudaSetDevice(d);
    }
    ~DeviceScope() { cudaSetDevice(prev); }
};

}  // namespace
}  // namespace mpm

using namespace mpm;

extern "C" {

int mpm_mc_table(int8_t* ntri, int8_t* edges) {
    if (!ntri || !edges) return MPM_ERR_ARGUMENT;
    const McTable t = build_mc_table();
    for (int m = 0; m < 256; ++m) {
        ntri[m] = t.ntri[m];
        for (int e = 0; e < kMcMaxTris * 3; ++e) edges[m * kMcMaxTris * 3 + e] = t.edge[m][e];
    }
    return MPM_OK;
}

int mpm_surface_create(int32_t device, void** surfacer) {
    if (!surfacer) return MPM_ERR_ARGUMENT;
    *surfacer = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    DeviceScope scope(device);
    Surfacer* s = new Surfacer();
    s->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && device < 64 && !g_table_ready[device]) {
        const McTable t = build_mc_table();
        e = cudaMemcpyToSymbol(c_mc_ntri, t.ntri, sizeof(t.ntri));
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_mc_edge, t.edge, sizeof(t.edge));
        if (e == cudaSuccess) g_table_ready[device] = true;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
        return MPM_ERR_CUDA;
    }
    *surfacer = s;
    return MPM_OK;
}

int mpm_surface_destroy(void* surfacer) {
    Surfacer* s = static_cast<Surfacer*>(surfacer);
    if (!s) return MPM_OK;
    DeviceScope scope(s->device);
    cudaStreamSynchronize(s->stream);
    s->release();
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return MPM_OK;
}

const char* mpm_surface_last_error(void* surfacer) {
    return surfacer ? static_cast<Surfacer*>(surfacer)->err.c_str() : "";
}

int mpm_surface_upload(void* surfacer, int64_t n, const float* x, const float* v, float lo[3], float hi[3]) {
    Surfacer* s = static_cast<Surfacer*>(surfacer);
    if (!s) return MPM_ERR_ARGUMENT;
    if (n <= 0 || !x || !v || !lo || !hi) return surf_fail(s, MPM_ERR_ARGUMENT, "bad particle arrays");
    DeviceScope scope(s->device);
    cudaStream_t st = s->stream;
    s->built = false;
    const size_t bytes = sizeof(float) * 3 * (size_t)n;
    int h_b[7];
    cudaError_t e = s->x.ensure(bytes);
    if (e == cudaSuccess) e = s->v.ensure(bytes);
    if (e == cudaSuccess) e = s->small.ensure(64);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->x.p, x, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->v.p, v, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const int init[7] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 0};
        e = cudaMemcpyAsync(s->small.p, init, sizeof(init), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) {
        const unsigned int blocks = (unsigned int)std::min<int64_t>(blocks_of(n), (int64_t)mpm::sm_count() * mpm::kCtasPerSm);
        k_surf_bounds<<<blocks, 256, 0, st>>>(n, s->x.as<float>(), s->small.as<int>());
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_b, s->small.p, sizeof(h_b), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        s->n = 0;
        return surf_fail(s, e == cudaErrorMemoryAllocation ? MPM_ERR_MEMORY : MPM_ERR_CUDA,
                         std::string("surface upload: ") + cudaGetErrorString(e));
    }
    s->n = n;
    for (int a = 0; a < 3; ++a) {
        const bool nan = (h_b[6] >> a) & 1;
        int l = h_b[a], u = h_b[3 + a];  // order-preserving integers back to float bits
        l = l >= 0 ? l : l ^ 0x7fffffff;
        u = u >= 0 ? u : u ^ 0x7fffffff;
        std::memcpy(&lo[a], &l, 4);
        std::memcpy(&hi[a], &u, 4);
        if (nan) lo[a] = hi[a] = std::nanf("");
    }
    return MPM_OK;
}

int mpm_surface_build(void* surfacer, const float origin[3], const int32_t dims[3], float cell, float inv_cell,
                      float h, float inv_rest, float iso, int64_t* n_verts, int64_t* n_tris) {
    Surfacer* s = static_cast<Surfacer*>(surfacer);
    if (!s) return MPM_ERR_ARGUMENT;
    if (!origin || !dims || !n_verts || !n_tris) return surf_fail(s, MPM_ERR_ARGUMENT, "bad surfacing arguments");
    if (s->n <= 0) return surf_fail(s, MPM_ERR_ARGUMENT, "no particles uploaded");
    if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2) return surf_fail(s, MPM_ERR_VALUE, "field grid under 2 nodes");
    if (!(cell > 0.0f) || !(h > 0.0f)) return surf_fail(s, MPM_ERR_VALUE, "cell and kernel radius must be positive");
    DeviceScope scope(s->device);
    s->built = false;
    const SurfGrid G{dims[0], dims[1], dims[2]};
    const int64_t N = (int64_t)dims[0] * dims[1] * dims[2];
    if (N >= (int64_t)1 << 31) return surf_fail(s, MPM_ERR_VALUE, "field grid of 2^31 nodes or more");
    auto run = [&]() -> cudaError_t {
        cudaStream_t st = s->stream;
        cudaError_t e;
        if ((e = s->acc.ensure(sizeof(float4) * N)) || (e = s->dens.ensure(sizeof(float) * N)) ||
            (e = s->bits.ensure(N)) || (e = s->cube.ensure(N)) || (e = s->cnt.ensure(sizeof(int32_t) * N)) ||
            (e = s->voff.ensure(sizeof(int32_t) * N)) || (e = s->tcnt.ensure(sizeof(int32_t) * N)) ||
            (e = s->toff.ensure(sizeof(int32_t) * N)) ||
            (e = s->tile.ensure(sizeof(int32_t) * (scan_tile_count(N) + 1))) || (e = s->small.ensure(64)))
            return e;
        float4* acc = s->acc.as<float4>();
        float* dens = s->dens.as<float>();
        uint8_t *bits = s->bits.as<uint8_t>(), *cube = s->cube.as<uint8_t>();
        int32_t *cnt = s->cnt.as<int32_t>(), *voff = s->voff.as<int32_t>(), *tcnt = s->tcnt.as<int32_t>(),
                *toff = s->toff.as<int32_t>(), *tile = s->tile.as<int32_t>(), *tot = s->small.as<int32_t>() + 8;
        if ((e = cudaMemsetAsync(acc, 0, sizeof(float4) * (size_t)N, st))) return e;
        k_surf_splat<<<blocks_of(s->n), 256, 0, st>>>(s->n, s->x.as<float>(), s->v.as<float>(), origin[0], origin[1],
                                                     origin[2], inv_cell, cell, h, G, acc);
        k_surf_normalize<<<blocks_of(N), 256, 0, st>>>(N, acc, dens, inv_rest);
        k_surf_edges<<<blocks_of(N), 256, 0, st>>>(G, dens, iso, bits, cnt);
        launch_exclusive_scan(st, cnt, N, voff, tile, tot);
        k_surf_cells<<<blocks_of(N), 256, 0, st>>>(G, dens, iso, cube, tcnt);
        launch_exclusive_scan(st, tcnt, N, toff, tile, tot + 1);
        int32_t h_tot[2] = {0, 0};
        if ((e = cudaMemcpyAsync(h_tot, tot, sizeof(h_tot), cudaMemcpyDeviceToHost, st))) return e;
        if ((e = cudaStreamSynchronize(st))) return e;
        s->n_nodes = N;
        s->n_verts = h_tot[0];
        s->n_tris = h_tot[1];
        if ((e = s->verts.ensure(sizeof(float) * 3 * (size_t)(s->n_verts + 1))) ||
            (e = s->vvel.ensure(sizeof(float) * 3 * (size_t)(s->n_verts + 1))) ||
            (e = s->tris.ensure(sizeof(int32_t) * 3 * (size_t)(s->n_tris + 1))))
            return e;
        if (s->n_verts > 0)
            k_surf_verts<<<blocks_of(N), 256, 0, st>>>(G, dens, acc, iso, bits, voff, s->verts.as<float>(),
                                                      s->vvel.as<float>());
        if (s->n_tris > 0) k_surf_tris<<<blocks_of(N), 256, 0, st>>>(G, cube, toff, bits, voff, s->tris.as<int32_t>());
        if ((e = cudaGetLastError())) return e;
        return cudaStreamSynchronize(st);
    };
    const cudaError_t e = run();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return surf_fail(s, e == cudaErrorMemoryAllocation ? MPM_ERR_MEMORY : MPM_ERR_CUDA,
                         std::string("surfacing: ") + cudaGetErrorString(e));
    }
    s->built = true;
    *n_verts = s->n_verts;
    *n_tris = s->n_tris;
    return MPM_OK;
}

int mpm_surface_read(void* surfacer, float* verts, int32_t* tris, float* vel) {
    Surfacer* s = static_cast<Surfacer*>(surfacer);
    if (!s) return MPM_ERR_ARGUMENT;
    if (!s->built) return surf_fail(s, MPM_ERR_ARGUMENT, "nothing built");
    if ((s->n_verts > 0 && (!verts || !vel)) || (s->n_tris > 0 && !tris))
        return surf_fail(s, MPM_ERR_ARGUMENT, "null output");
    DeviceScope scope(s->device);
    cudaError_t e = cudaSuccess;
    if (s->n_verts > 0) {
        e = cudaMemcpyAsync(verts, s->verts.p, sizeof(float) * 3 * (size_t)s->n_verts, cudaMemcpyDeviceToHost,
                            s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(vel, s->vvel.p, sizeof(float) * 3 * (size_t)s->n_verts, cudaMemcpyDeviceToHost,
                                s->stream);
    }
    if (e == cudaSuccess && s->n_tris > 0)
        e = cudaMemcpyAsync(tris, s->tris.p, sizeof(int32_t) * 3 * (size_t)s->n_tris, cudaMemcpyDeviceToHost,
                            s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return surf_fail(s, MPM_ERR_CUDA, std::string("surface read: ") + cudaGetErrorString(e));
    }
    return MPM_OK;
}

int mpm_surface_read_field(void* surfacer, float* density, float* field) {
    Surfacer* s = static_cast<Surfacer*>(surfacer);
    if (!s) return MPM_ERR_ARGUMENT;
    if (!s->built || !density || !field) return surf_fail(s, MPM_ERR_ARGUMENT, "no field to read");
    DeviceScope scope(s->device);
    cudaError_t e = cudaMemcpyAsync(density, s->dens.p, sizeof(float) * (size_t)s->n_nodes, cudaMemcpyDeviceToHost,
                                    s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(field, s->acc.p, sizeof(float4) * (size_t)s->n_nodes, cudaMemcpyDeviceToHost,
                            s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return surf_fail(s, MPM_ERR_CUDA, std::string("field read: ") + cudaGetErrorString(e));
    }
    return MPM_OK;
}

}  // extern "C"
