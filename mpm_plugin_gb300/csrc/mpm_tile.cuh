// G2P through TMA tile loads (MPM_OPT_G2P_VARIANT 2; one scene, one grid, FP32 return mapping).
//
// A persistent kernel: each CTA of 256 threads walks chunks of 256 consecutive particles (chunk c, c + G,
// c + 2G, ... for G CTAs), one particle per thread. Everything a chunk reads is brought into shared memory
// by the tensor memory accelerator (cp.async.bulk.tensor) ahead of the chunk, on mbarriers, so the warps
// compute from shared memory while the next chunk's data is in flight:
//   * the particle planes G2P reads (x 3, F 9, Jp, mat) as 1 KiB tiles of a 2-D tensor map over the arena
//     (particle, plane); x runs two chunks ahead (a ring of three x buffers), the other planes one ahead;
//   * the grid nodes of its stencils: a particle's stencil (base .. base + 2 per axis) lies inside the 2 x 2 x
//     2 grid blocks starting at its base node's block, one 8 KiB box of a 4-D tensor map over the blocked grid
//     (256 floats of a block, block k, j, i). The chunk's distinct base blocks (one or two when the particles
//     are in grid-block order, which the periodic reorder by grid node gives) take up to kTileSlots such
//     boxes; a particle whose base block did not get a slot gathers from the grid in global memory.
// One chunk ahead: when chunk i starts, x of chunk i + 1 has arrived (it was requested a whole chunk
// earlier); the chunk's base blocks are found from it and the boxes and the other planes of chunk i + 1 are
// requested; then the CTA waits for chunk i's own tiles (requested while chunk i - 1 computed) and computes.
// Results are stored straight to the particle arrays (their tiles of later chunks are other addresses).
//
// Every mbarrier wait is bounded: after kTileSpins polls the kernel sets the error word (reported by the
// host after its next synchronisation), waits once more (bounded) for the copies it issued, and returns.
#pragma once

#include <cuda.h>  // CUtensorMap (the type only; tensor maps are encoded through the runtime's driver entry point)

#include "mpm_substep_kernels.cuh"

namespace mpm {

constexpr int kTileChunk = 256;
constexpr int kTileSlots = 2;
constexpr int kTileRest = 11;  // planes after x: F 9, Jp, mat
constexpr int kTileSlotNodes = 512;
constexpr unsigned int kTileSpins = 1u << 22;
// arena planes of the staged fields (mpm_types.h make_particles: x 0-2, F 15-23, Jp 24, mat 31)
__host__ __device__ constexpr int tile_arena_plane(int q) { return q < 3 ? q : (q < 12 ? 12 + q : (q == 12 ? 24 : 31)); }

struct TileMaps {
    CUtensorMap planes;  // 2-D: (particle, plane) over the arena; box 256 x 1 floats
    CUtensorMap grid;    // 4-D: (float within a block, block k, block j, block i); box 256 x 2 x 2 x 2 floats
};

struct __align__(128) TileStage {
    float4 slot[kTileSlots][kTileSlotNodes];  // grid boxes, node order of the box's blocks
    float rest[kTileRest][kTileChunk];        // F 9, Jp, mat (bits)
    int slot_key[kTileSlots];                 // base block of the slot (linear block index), -1: free
    unsigned char pslot[kTileChunk];          // per particle: its slot, 0xff: gathers from global memory
};

struct __align__(128) TileShared {
    float xbuf[3][3][kTileChunk];  // ring of x tiles (chunk i in buffer i % 3)
    TileStage st[2];               // chunk i in stage i % 2
    unsigned long long bar_x[3], bar_rest[2];
};
constexpr size_t kTileSmemBytes = sizeof(TileShared);

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned int bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Polls the barrier's phase with the given parity; false when it did not complete within kTileSpins polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned int parity) {
    const uint32_t a = smem_addr(bar);
    for (unsigned int i = 0; i < kTileSpins; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Orders this thread's earlier generic-proxy accesses to shared memory before its later async-proxy ones
// (a TMA load into a buffer the warps have just read).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(smem_addr(bar))
        : "memory");
}

// G2P inputs of thread t's particle from the staged tiles.
struct TileIn {
    static constexpr bool kPrefetch = false;
    const float* xs;    // the chunk's x buffer: 3 planes of 256
    const float* rest;  // F 9, Jp, mat planes of 256
    int t;
    __device__ __forceinline__ float x(int a) const { return xs[a * kTileChunk + t]; }
    __device__ __forceinline__ float F(int e) const { return rest[e * kTileChunk + t]; }
    __device__ __forceinline__ float Jp() const { return rest[9 * kTileChunk + t]; }
    __device__ __forceinline__ int mat() const { return __float_as_int(rest[10 * kTileChunk + t]); }
};

// Stencil nodes from the particle's slot in shared memory (box of the 2 x 2 x 2 blocks from its base
// block; node offset = block i' 256 + block j' 128 + block k' 64 + local i 16 + local j 4 + local k), or
// from the global grid when it has none. One generic pointer and per-axis terms for both.
struct TileSource {
    const GridDesc* g;
    const float4* grid;
    const float4* slot;  // null: global
    struct Stencil {
        const float4* ptr;
        int64_t x[3];
        int y[3], z[3];
        __device__ __forceinline__ float4 operator()(int i, int j, int k) const { return ptr[x[i] + (int64_t)(y[j] + z[k])]; }
    };
    __device__ __forceinline__ Stencil stencil(const int base[3]) const {
        Stencil s;
        if (slot) {
            const int b0 = base[0] >> 2, b1 = base[1] >> 2, b2 = base[2] >> 2;
            s.ptr = slot;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int i = base[0] + d, j = base[1] + d, k = base[2] + d;
                s.x[d] = ((i >> 2) - b0) * 256 + (i & 3) * 16;
                s.y[d] = ((j >> 2) - b1) * 128 + (j & 3) * 4;
                s.z[d] = ((k >> 2) - b2) * 64 + (k & 3);
            }
        } else {
            const StencilIndex at = stencil_index(*g, base);
            s.ptr = grid;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                s.x[d] = at.x[d];
                s.y[d] = at.y[d];
                s.z[d] = at.z[d];
            }
        }
        return s;
    }
};

// Base grid block (linear index) of particle p's stencil from its staged x, or -1 when the stencil leaves the
// padded grid (the particle gathers nothing) or p is past the end.
__device__ __forceinline__ int tile_key(const GridDesc& g, const float* x, int t, bool live) {
    if (!live) return -1;
    int base[3];
    float fx;
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) inside &= stencil_axis((x[a * kTileChunk + t] - g.origin[a]) * g.inv_dx, g.dims[a], &base[a], &fx);
    if (!inside) return -1;
    return ((base[0] >> 2) * g.nb[1] + (base[1] >> 2)) * g.nb[2] + (base[2] >> 2);
}

// Slots of chunk `chunk` (x already in xb): the distinct base blocks claim up to kTileSlots slots (a
// compare-and-swap into the first free or matching slot), then thread 0 requests the slots' grid boxes and
// the chunk's other planes on bar. All threads of the CTA call it.
__device__ __forceinline__ void tile_build(const SubstepArgs& a, const TileMaps& maps, TileStage& st, const float* xb,
                                           int64_t chunk, unsigned long long* bar) {
    const int t = (int)threadIdx.x;
    if (t < kTileSlots) st.slot_key[t] = -1;
    __syncthreads();
    const int64_t p = chunk * kTileChunk + t;
    const int key = tile_key(a.g, xb, t, p < a.n);
    unsigned char slot = 0xff;
    if (key >= 0) {
#pragma unroll
        for (int s = 0; s < kTileSlots; ++s) {
            int cur = *(volatile int*)&st.slot_key[s];
            if (cur == -1) {
                cur = atomicCAS(&st.slot_key[s], -1, key);
                if (cur == -1) cur = key;
            }
            if (cur == key) {
                slot = (unsigned char)s;
                break;
            }
        }
    }
    st.pslot[t] = slot;
    __syncthreads();
    if (t == 0) {
        int used = 0;
#pragma unroll
        for (int s = 0; s < kTileSlots; ++s) used += st.slot_key[s] >= 0;
        fence_proxy_async();
        mbar_expect_tx(bar, (unsigned int)(used * kTileSlotNodes * sizeof(float4) + kTileRest * kTileChunk * sizeof(float)));
        const int c0 = (int)(chunk * kTileChunk);
#pragma unroll
        for (int q = 0; q < kTileRest; ++q) tma_load_2d(st.rest[q], &maps.planes, c0, tile_arena_plane(3 + q), bar);
        const GridDesc& g = a.g;
        for (int s = 0; s < kTileSlots; ++s) {
            const int key_s = st.slot_key[s];
            if (key_s < 0) continue;
            const int bk = key_s % g.nb[2], bj = (key_s / g.nb[2]) % g.nb[1], bi = key_s / (g.nb[2] * g.nb[1]);
            tma_load_4d(st.slot[s], &maps.grid, 0, bk, bj, bi, bar);
        }
    }
}

__device__ __forceinline__ void tile_request_x(const TileMaps& maps, float* xb, int64_t chunk, unsigned long long* bar) {
    fence_proxy_async();
    mbar_expect_tx(bar, 3 * kTileChunk * sizeof(float));
    const int c0 = (int)(chunk * kTileChunk);
#pragma unroll
    for (int a = 0; a < 3; ++a) tma_load_2d(xb + a * kTileChunk, &maps.planes, c0, a, bar);
}

// Gives up after a failed wait: records the error, waits (bounded) for what is still in flight on the
// barriers this CTA armed, and lets the caller return.
__device__ __forceinline__ void tile_abort(const SubstepArgs& a, TileShared& sh, const unsigned int* xpar,
                                           const unsigned int* rpar, const bool* x_armed, const bool* r_armed) {
    if (threadIdx.x == 0) {
        atomicOr(a.err, 1u);
        for (int r = 0; r < 3; ++r)
            if (x_armed[r]) mbar_wait(&sh.bar_x[r], xpar[r]);
        for (int r = 0; r < 2; ++r)
            if (r_armed[r]) mbar_wait(&sh.bar_rest[r], rpar[r]);
    }
    __syncthreads();
}

template <int kMinCtas>
__global__ void __launch_bounds__(256, kMinCtas) k_g2p_tile(const __grid_constant__ TileMaps maps, OneScene sc) {
    pdl_begin();
    extern __shared__ __align__(128) unsigned char tile_smem[];  // kTileSmemBytes + 128 bytes
    TileShared& sh = *reinterpret_cast<TileShared*>(tile_smem + ((128u - (smem_addr(tile_smem) & 127u)) & 127u));
    const SubstepArgs a = sc.get(0);
    const int64_t chunks = (a.n + kTileChunk - 1) / kTileChunk;
    const int64_t c0 = blockIdx.x, G = gridDim.x;
    if (c0 >= chunks) return;
    const int t = (int)threadIdx.x;
    const int64_t iters = (chunks - c0 + G - 1) / G;  // chunks of this CTA: c0 + i G, i < iters
    // phase parity of each barrier's next wait, and whether a copy on it is outstanding (thread 0's view)
    unsigned int xpar[3] = {0u, 0u, 0u}, rpar[2] = {0u, 0u};
    bool x_armed[3] = {false, false, false}, r_armed[2] = {false, false};
    if (t == 0) {
        for (int r = 0; r < 3; ++r) mbar_init(&sh.bar_x[r], 1);
        for (int r = 0; r < 2; ++r) mbar_init(&sh.bar_rest[r], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (t == 0) {
        tile_request_x(maps, sh.xbuf[0][0], c0, &sh.bar_x[0]);
        x_armed[0] = true;
        if (iters > 1) {
            tile_request_x(maps, sh.xbuf[1][0], c0 + G, &sh.bar_x[1]);
            x_armed[1] = true;
        }
    }
    // chunk 0's slots
    bool ok = mbar_wait(&sh.bar_x[0], 0u);
    if (!__syncthreads_and(ok)) {
        tile_abort(a, sh, xpar, rpar, x_armed, r_armed);
        return;
    }
    xpar[0] ^= 1u;
    x_armed[0] = false;
    tile_build(a, maps, sh.st[0], sh.xbuf[0][0], c0, &sh.bar_rest[0]);
    r_armed[0] = true;
    const unsigned int cur = a.sp->seq & 1u;
    const float4* grid = grid_of(a, cur);
    const Particles P = particles_of(a);
    for (int64_t i = 0; i < iters; ++i) {
        const int s = (int)(i & 1), xr = (int)(i % 3);
        // x two chunks ahead (its buffer held chunk i - 1's x)
        if (i + 2 < iters && t == 0) {
            const int r2 = (int)((i + 2) % 3);
            tile_request_x(maps, sh.xbuf[r2][0], c0 + (i + 2) * G, &sh.bar_x[r2]);
            x_armed[r2] = true;
        }
        // the next chunk's slots and planes (its stage held chunk i - 1)
        if (i + 1 < iters) {
            const int r1 = (int)((i + 1) % 3);
            ok = mbar_wait(&sh.bar_x[r1], xpar[r1]);
            if (!__syncthreads_and(ok)) {
                tile_abort(a, sh, xpar, rpar, x_armed, r_armed);
                return;
            }
            xpar[r1] ^= 1u;
            x_armed[r1] = false;
            tile_build(a, maps, sh.st[s ^ 1], sh.xbuf[r1][0], c0 + (i + 1) * G, &sh.bar_rest[s ^ 1]);
            r_armed[s ^ 1] = true;
        }
        ok = mbar_wait(&sh.bar_rest[s], rpar[s]);
        if (!__syncthreads_and(ok)) {
            tile_abort(a, sh, xpar, rpar, x_armed, r_armed);
            return;
        }
        rpar[s] ^= 1u;
        r_armed[s] = false;
        const int64_t p = (c0 + i * G) * kTileChunk + t;
        if (p < a.n) {
            const TileStage& st = sh.st[s];
            const TileIn in{sh.xbuf[xr][0], st.rest[0], t};
            const unsigned char sl = st.pslot[t];
            const TileSource src{&a.g, grid, sl == 0xff ? nullptr : st.slot[sl]};
            float nx[3];
            g2p_particle_from<TileSource, false, TileIn>(P, p, in, a.mats, a.g, a.sp->dt, src, a.fp64, nx);
            if (a.cd.n_col > 0) {
                ColliderData cd = a.cd;
                cd.poses += a.sp->pose_base;
                if (near_any_collider(nx, cd)) warp_append(a.wl.part_cand, &a.wl.counts[3], (int32_t)p);
            }
        }
        __syncthreads();  // stage s and x buffer xr are free again
    }
}

}  // namespace mpm
