// Occupancy query that allocates no device memory (mpm_is_occupied_noalloc in include/mpm_gb300.h).
//
// For callers that cannot allocate device memory when they ask: for example a serving process that has
// handed its whole HBM budget to resident scenes at start-up and may not take more per request, or a host
// application whose own allocator owns the device and forbids cudaMalloc/cudaFree from plugins (cudaFree
// also synchronises the device, which such callers must avoid). The caller passes particle positions, query
// points and the output on the device; the B-spline volume grid the query needs lives in the file-scope
// array below, a fixed 16 MiB (4,194,304 grid nodes) that every GPU which loads this library keeps until the
// process exits. All calls share it: two calls whose work overlaps on the GPU (different streams, or
// different host threads without ordering) race on it and give wrong answers.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/mpm_gb300.h"
#include "mpm_device.cuh"
#include "mpm_host.h"
#include "mpm_internal.h"

namespace {

constexpr int64_t kNoAllocNodes = 4 * 1024 * 1024;  // 16 MiB of float
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_occupancy_scratch[kNoAllocNodes];

std::mutex g_scratch_mu;
float* g_scratch_ptr[kMaxDevices] = {};

// The array's device address on the current device. In host code the array's name is only a host-side
// stand-in, so its address is looked up once per device with that device current.
cudaError_t scratch_address(int device, float** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[device]) {
        float* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_occupancy_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[device] = p;
    }
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

__global__ void k_noalloc_scatter(const float* __restrict__ x, int64_t n, mpm::GridDesc g, float* __restrict__ vol) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int base[3];
    float fx, w[3][3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
        float xp = (x[p * 3 + a] - g.origin[a]) * g.inv_dx;
        inside &= mpm::stencil_axis(xp, g.dims[a], &base[a], &fx);
        mpm::bspline_weights(fx, w[a]);
    }
    if (!inside) return;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                atomicAdd(&vol[mpm::node_index(g, base[0] + i, base[1] + j, base[2] + k)],
                          w[0][i] * w[1][j] * w[2][k] * g.p_vol);
}

__global__ void k_noalloc_query(mpm::GridDesc g, const float* __restrict__ vol, float cell_vol, int64_t m,
                                const float* __restrict__ pts, uint8_t* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int idx[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
        float gq = (pts[q * 3 + a] - g.origin[a]) * g.inv_dx;
        idx[a] = (int)copysignf(floorf(fabsf(gq) + 0.5f), gq);  // nearest node, halves away from zero
        if (idx[a] < 0 || idx[a] >= g.dims[a]) inside = false;
    }
    out[q] = inside && vol[mpm::node_index(g, idx[0], idx[1], idx[2])] >= 0.5f * cell_vol ? 1 : 0;
}

int fail(int code, const std::string& msg) {
    mpm::set_last_error(msg);  // read back with mpm_last_error(NULL)
    return code;
}

}  // namespace

extern "C" int mpm_is_occupied_noalloc(const MpmDomainDesc* domain, int32_t particles_per_cell, int64_t n,
                                       const float* d_x, int64_t m, const float* d_points, uint8_t* d_out,
                                       int32_t device, void* stream) {
    if (!domain || particles_per_cell <= 0 || n < 0 || m < 0 || (n > 0 && !d_x) || (m > 0 && (!d_points || !d_out)))
        return fail(MPM_ERR_ARGUMENT, "bad arguments");
    if (const char* why = mpm::domain_problem(*domain)) return fail(MPM_ERR_VALUE, why);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return fail(MPM_ERR_CUDA, "no CUDA device");
    }
    if (device < 0 || device >= count || device >= kMaxDevices)
        return fail(MPM_ERR_ARGUMENT, "device index out of range");
    const double gravity[3] = {0.0, 0.0, 0.0};
    mpm::HostDomain hd{};
    mpm::GridDesc g = mpm::make_grid(*domain, gravity, particles_per_cell, &hd);
    const int64_t nodes = (int64_t)g.nb[0] * g.nb[1] * g.nb[2] * 64;
    if (nodes > kNoAllocNodes)
        return fail(MPM_ERR_VALUE, "domain needs " + std::to_string(nodes) + " grid nodes; the static scratch holds " +
                                       std::to_string(kNoAllocNodes) + " (16 MiB): use mpm_is_occupied");
    if (m == 0) return MPM_OK;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        return fail(MPM_ERR_CUDA, "cudaGetDevice failed");
    }
    if (prev != device && cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return fail(MPM_ERR_CUDA, "cudaSetDevice failed");  // before any address is looked up or cached
    }
    float* vol = nullptr;
    cudaError_t e = scratch_address(device, &vol);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(vol, 0, (size_t)nodes * sizeof(float), st);  // starts from zero
    // launched through cudaLaunchKernel, whose return value is this launch's own status (an error pending
    // from the caller's earlier calls is neither reported here nor cleared)
    if (e == cudaSuccess && n > 0) {
        void* args[] = {&d_x, &n, &g, &vol};
        e = cudaLaunchKernel(reinterpret_cast<const void*>(k_noalloc_scatter), dim3((unsigned int)((n + 255) / 256)),
                             dim3(256), args, 0, st);
    }
    if (e == cudaSuccess) {
        float cell_vol = (float)std::pow(hd.dx, 3.0);
        void* args[] = {&g, &vol, &cell_vol, &m, &d_points, &d_out};
        e = cudaLaunchKernel(reinterpret_cast<const void*>(k_noalloc_query), dim3((unsigned int)((m + 255) / 256)),
                             dim3(256), args, 0, st);
    }
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(MPM_ERR_CUDA, cudaGetErrorString(e));
    return MPM_OK;
}
