/* mpm_gb300: C-ABI of the GB300 (sm_103a) MLS-MPM substep backend.
 *
 * This library is the device side of a new backend for the reference's solver interface
 * (mpm_core/solver.py:37-82 of jonatanhedborg/mpm_plugin). Its Python binding (mpm_plugin_gb300/_abi.py, ctypes)
 * implements mpm_core.solver.Solver on top of these calls and registers it with
 * mpm_core.backends.register_backend (mpm_core/backends/__init__.py:21-22). Each entry point below names the
 * reference interface it replaces (file:line in the reference project).
 *
 * Conventions: plain pointers and sizes only. Every call returns an int status (MPM_OK = 0) and, on failure,
 * mpm_last_error(h) describes it (mpm_last_error(NULL) for failures before a handle exists). Host arrays are
 * C-contiguous row-major float32/int32: positions and velocities (N,3), C and F (N,3,3), Jp (N,). Particle
 * order is the reference's: insertion order, with removed particles dropped and the rest kept in order.
 * One handle is one domain on one GPU; a handle is used by one host thread at a time.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MPM_OK = 0,
    MPM_ERR_VALUE = 1,           /* maps to ValueError (bad ids, sizes, transform counts) */
    MPM_ERR_NOT_IMPLEMENTED = 2, /* maps to NotImplementedError (unknown material model) */
    MPM_ERR_CUDA = 3,            /* a CUDA runtime error; message has the CUDA error string */
    MPM_ERR_ARGUMENT = 4,        /* null handle or pointer */
    MPM_ERR_MEMORY = 5           /* device allocation failed */
};

enum { MPM_MODEL_ELASTIC = 0, MPM_MODEL_VON_MISES = 1, MPM_MODEL_DRUCKER_PRAGER = 2, MPM_MODEL_SNOW = 3 };

/* mpm_core/scene.py:36-67 Domain: axis-aligned box, resolution along its longest side, six walls. */
typedef struct MpmDomainDesc {
    double min[3], max[3];
    int32_t resolution;
    int32_t wall_lo[3]; /* x-, y-, z-: 1 = wall, 0 = open side */
    int32_t wall_hi[3]; /* x+, y+, z+ */
    double wall_friction;
} MpmDomainDesc;

/* mpm_core/materials.py:24-59 MaterialParams (model as MPM_MODEL_*). */
typedef struct MpmMaterialDesc {
    int32_t model;
    double youngs_modulus, poisson_ratio, density;
    double yield_stress, friction_angle_deg, hardening, critical_compression, critical_stretch, max_hardening;
} MpmMaterialDesc;

/* mpm_core/solver.py:30-34 ColliderGeometry: a triangle mesh in the collider's local space. */
typedef struct MpmColliderDesc {
    int32_t n_verts, n_tris;
    const float *verts;   /* (n_verts, 3) */
    const int32_t *tris;  /* (n_tris, 3) */
    int32_t closed;
    double friction;
} MpmColliderDesc;

/* mpm_core/solver.py:23-27 AdvanceStats. */
typedef struct MpmAdvanceStats {
    int32_t substeps;
    double dt;
    int32_t removed;
} MpmAdvanceStats;

/* Replaces WarpSolver.__init__ (mpm_core/backends/warp/solver.py:27-78), reached through
 * create_solver (mpm_core/backends/__init__.py:25-28). MPM_ERR_NOT_IMPLEMENTED for an unknown model. */
int mpm_create(const MpmDomainDesc *domain, const MpmMaterialDesc *materials, int32_t n_materials,
               const double gravity[3], int32_t particles_per_cell, int32_t device, void **handle);
int mpm_destroy(void *handle);
const char *mpm_last_error(void *handle);

/* Solver.add_particles (mpm_core/solver.py:52-54; warp/solver.py:100-125). n == 0 is a no-op;
 * MPM_ERR_VALUE "material id out of range" for a bad id. New particles get C = 0, F = I, Jp = 1. */
int mpm_add_particles(void *handle, int64_t n, const float *x, const float *v, const int32_t *material_ids,
                      const int32_t *emitter_ids);

/* Solver.set_colliders (mpm_core/solver.py:56-58; warp/solver.py:142-152): replaces all colliders and
 * resets their transforms to identity. */
int mpm_set_colliders(void *handle, int32_t n, const MpmColliderDesc *colliders);

/* Solver.set_collider_transforms (mpm_core/solver.py:60-62; warp/solver.py:154-172): (n,4,4) row-major
 * world matrices at the start and end of the next advance. MPM_ERR_VALUE if n != collider count. */
int mpm_set_collider_transforms(void *handle, int32_t n, const float *start16, const float *end16);

/* Solver.advance (mpm_core/solver.py:64-65; warp/solver.py:176-240): CFL time step, substeps, removal of
 * particles past open sides. With no particles: {0, frame_dt, 0}. */
int mpm_advance(void *handle, double frame_dt, MpmAdvanceStats *stats);

/* One substep with a given dt and substep fraction s (WarpSolver._substep, warp/solver.py:187-211), for
 * fixed-dt runs and parity checks. frame_dt is the advance duration the collider velocities refer to. */
int mpm_substep(void *handle, double dt, double s, double frame_dt);

/* Solver.particle_count (mpm_core/solver.py:67-69). */
/* `count` substeps of a fixed dt in one call (no CFL choice, no removal): the substeps of one advance of
 * frame_dt, collider poses interpolated at s = (k + 1) / count (warp/solver.py:216-219). No counterpart in the
 * reference; the fixed-dt workloads (and tests) use it to run many substeps without a call per substep. */
int mpm_run_substeps(void *handle, double dt, int32_t count, double frame_dt);

int mpm_particle_count(void *handle, int64_t *n);

/* Solver.get_particles (mpm_core/solver.py:71-72; warp/solver.py:131-132). Any output may be NULL. */
int mpm_get_particles(void *handle, float *x, float *v, int32_t *material_ids, int32_t *emitter_ids);

/* Solver.is_occupied (mpm_core/solver.py:74-76; warp/solver.py:244-255; kernels.py:272-298). */
int mpm_is_occupied(void *handle, int64_t m, const float *points, uint8_t *out);

/* Solver.save_state / load_state (mpm_core/solver.py:78-82; warp/solver.py:134-138): keys x, v, C, F, Jp,
 * mat, emitter. load_state replaces every particle; MPM_ERR_VALUE for an out-of-range material id. */
int mpm_save_state(void *handle, float *x, float *v, float *C, float *F, float *Jp, int32_t *mat, int32_t *emitter);
int mpm_load_state(void *handle, int64_t n, const float *x, const float *v, const float *C, const float *F,
                   const float *Jp, const int32_t *mat, const int32_t *emitter);

/* Runtime options (no reference counterpart; tuning and measurement of this backend). */
enum {
    MPM_OPT_USE_GRAPH = 1,     /* 1 (default): replay a captured CUDA graph per substep */
    MPM_OPT_KERNEL_TIMING = 2, /* 1: record CUDA events between the kernel groups of every substep (event nodes
                                  in the captured graph); 2: events at the two ends of each substep only, so
                                  the kernels inside stay chained as untimed; each substep then waits for its
                                  own completion */
    MPM_OPT_SORT_INTERVAL = 3, /* N (default 4): after every N substeps the particle storage is reordered into
                                  grid-block order (ids travel along, so host order is unchanged); 0: never */
    MPM_OPT_DETERMINISTIC = 4, /* 1: bit-reproducible runs. P2G and the occupancy splat sum in 64-bit fixed point
                                  (exact integer additions, independent of particle order and atomic timing);
                                  results agree with the default mode within float rounding. 0 (default) */
    MPM_OPT_G2P_VARIANT = 5,   /* G2P build: 0 (default) capped at 64 registers, 4 CTAs of 256 per SM; 1 uncapped;
                                  2 the tile build (TMA loads of particle planes and grid boxes); 3 capped at
                                  80 registers, 3 CTAs per SM. With MPM_OPT_FP64_CLAMP on: 0, 2 and 3 the
                                  FP64 build at 80 registers, 1 at 128 */
    MPM_OPT_LIST_CTAS = 6,     /* CTAs of the kernels that walk the active-block and candidate lists (default:
                                  8 per SM of the device, from cudaDevAttrMultiProcessorCount) */
    MPM_OPT_P2G_GROUP = 7,     /* P2G sums same-cell lanes within aligned groups of this many lanes before one
                                  reduction each: 1, 2, 4, 8, 16 or 32 (default) */
    MPM_OPT_PDL = 8,           /* 1 (default): the substep kernels use programmatic dependent launch, so each
                                  kernel's launch overlaps the tail of the one before; 0: plain stream order */
    MPM_OPT_FP64_CLAMP = 9,    /* FP64 in the Drucker-Prager and snow return mapping: 1 a particle whose FP32
                                  decision is marginal where the outcome jumps (the Drucker-Prager separation
                                  test: |tr log sigma| within a relative 1e-6 of the strain, the strain above
                                  1e-6) is redone in FP64 (SVD, projection, hardening, stress); 2 every
                                  particle whose clamp is active is; 0 (default): FP32, with the FP64 redo only
                                  for SVDs that did not converge */
    MPM_OPT_P2G_TILE = 10,     /* 1: P2G sums each CTA's contributions in shared-memory tiles of the nodes its
                                  particles touch, then adds them to the grid; 0 (default): warp segments
                                  (shuffle sums of same-cell lanes) only. Deterministic mode uses segments */
    MPM_OPT_COOP = 11,         /* substeps of mpm_advance / mpm_run_substeps in cooperative launches of up to 64
                                  substeps each (the kernels' phases separated by grid-wide barriers): 0
                                  (default) never, 1 always (without kernel timing, the FP64 clamp or the tile
                                  P2G), 2 for scenes of up to 131,072 particles. Slower than the graphs of
                                  separate kernels on a GB300 at the sizes measured */
    MPM_OPT_FUSED_P2G = 12,    /* 1: two grids that alternate between substeps; G2P adds each particle it has
                                  updated to the next substep's grid right away (and the collider projection
                                  the particles it moved), so the next substep's P2G reads no particle state.
                                  Within mpm_advance / mpm_run_substeps, and between mpm_substep calls with the
                                  same dt (a scatter for a call that does not follow is dropped). Not in
                                  deterministic mode, with the FP64 clamp or in a batch (those run one grid).
                                  Costs a second grid of device memory. 0 (default) */
    MPM_OPT_BLOCK_SWEEP = 13   /* 1: P2G marks the grid blocks it touches with plain stores, and a short kernel
                                  after it lists the marked blocks (a sweep over the block flags) for the grid
                                  update; 0 (default): P2G lists a block itself the first time it touches it
                                  (an atomic exchange on the flag and an atomic add on the list's length).
                                  One grid only (two-grid mode, cooperative launches and batches list
                                  blocks in P2G) */,
    MPM_OPT_PARTICLES_PER_THREAD = 14 /* 1 (default), 2, 4 or 8: particles per thread of the plain solver's
                                  P2G and G2P kernels. Their grid holds ceil(chunks / k) CTAs of 256 threads that
                                  walk the 256-particle chunks grid-stride, so each thread takes about k
                                  particles one after another. (Batches walk their scenes' chunks with at most
                                  8 CTAs per SM whatever this is; the tile builds keep their own grids.) */,
    MPM_OPT_P2G_MERGE = 15     /* 1 (default): P2G also merges the sums of segment leaders whose stencils share
                                  an x-y column and differ by one or two nodes in z, so a shared node gets one
                                  reduction; 0: one reduction per node and leader. Not in deterministic
                                  mode (its fixed-point sums do not merge) */
};
int mpm_set_option(void *handle, int32_t option, int64_t value);

/* The CUDA stream (cudaStream_t) all work of this handle runs on, for callers that time or order it. */
int mpm_get_stream(void *handle, void **stream);
int mpm_synchronize(void *handle);

/* Per-kernel totals since the last reset, when MPM_OPT_KERNEL_TIMING is on: names are
 * "p2g", "grid_update", "g2p", "other" (timing 1), then "substep" (timing 2: whole substeps, reorders
 * included); ms[i] total milliseconds and launches[i] counts, n_slots of them (at most 5). */
int mpm_kernel_times(void *handle, int32_t n_slots, float *ms, int64_t *launches, int32_t reset);

/* Read-back for checks and tooling (no reference counterpart; the reference's grid lives in Warp arrays
 * grid_v / grid_m, warp/solver.py:73-74). mpm_grid_dims: padded node counts (grid_shape + 6).
 * mpm_read_grid: dims[0]*dims[1]*dims[2] nodes in C order, 4 floats each: velocity xyz after the grid update
 * (momentum where the mass is zero) and mass, as left by the last substep.
 * mpm_read_collider_pose: collider c's pose of the last substep as 3x4 row-major matrices: the world
 * transform M, its inverse, and dM, the time derivative the collider velocity is taken from. */
int mpm_grid_dims(void *handle, int32_t dims[3]);
/* The padded node counts a solver created with this domain would have (grid_shape + 6 per axis,
 * mpm_core/scene.py:60-67 and warp/solver.py:37-40), without creating one or touching a device: for footprint
 * estimates before admission. MPM_ERR_VALUE for a domain mpm_create would refuse. */
int mpm_domain_grid_dims(const MpmDomainDesc *domain, int32_t dims[3]);
int mpm_read_grid(void *handle, float *out);
int mpm_read_collider_pose(void *handle, int32_t c, float *M12, float *Minv12, float *dM12);

/* Kernels of this library launched on the handle's stream since it was created. */
int mpm_launch_count(void *handle, int64_t *launches);

/* Read-back that does not hold up the next advance (no counterpart in the reference, whose get_particles
 * and save_state return once the copy is done, bake.py:205-206). The requested arrays (any may be NULL; the
 * layouts and particle order of mpm_save_state) are gathered into device storage on the handle's stream and
 * copied into the host buffers on a separate copy stream; the call returns at once and the caller may advance
 * again. The host buffers must stay valid and unread until mpm_read_wait returns. Page-locked buffers
 * (mpm_host_alloc) make the copy asynchronous. One read is in flight per handle: a second mpm_read_begin
 * first waits for the one before. */
int mpm_read_begin(void *handle, float *x, float *v, float *C, float *F, float *Jp, int32_t *mat, int32_t *emitter);
int mpm_read_wait(void *handle);
int mpm_host_alloc(int64_t bytes, void **ptr);
int mpm_host_free(void *ptr);

/* Conservation accumulators in FP64 over the particles (no counterpart in the reference; the reference's
 * tests sum host copies): out[0] total mass, out[1..3] momentum, out[4..6] mass-weighted position (centre of
 * mass = out[4..6] / out[0]), out[7] kinetic energy, out[8] particles skipped as non-finite. */
int mpm_conservation(void *handle, double *out);

/* Device memory the handle holds now, in bytes (no counterpart in the reference; serving admission). */
int mpm_device_bytes(void *handle, int64_t *bytes);

/* Number of SVD lanes whose FP32 Jacobi sweeps (up to eight) did not diagonalise F^T F - I to 4e-6 since
   the handle was created: redone in FP64 by the G2P build of MPM_OPT_FP64_CLAMP and by the stress of
   particles that enter; the other G2P builds keep the FP32 result. */
int mpm_fp64_lanes(void *handle, int64_t *lanes);
/* Number of Drucker-Prager / snow lanes whose return mapping G2P redid in FP64 under MPM_OPT_FP64_CLAMP since the
 * handle was created (no counterpart in the reference; it reports how far FP64 is confined). */
int mpm_fp64_redo_lanes(void *handle, int64_t *lanes);

/* Occupancy query that allocates no device memory. It has no counterpart in the reference: it is for callers
 * that cannot allocate device memory when they ask, such as a serving process whose device memory budget
 * was handed out at start-up, or a host application whose own allocator owns the device (cudaFree would
 * also synchronise the device). Same answer as mpm_is_occupied for particles at d_x: d_x (n,3), d_points (m,3)
 * and d_out (m) are caller-owned device arrays; the work is queued on `stream` (NULL: the legacy default
 * stream) and d_out is valid once that stream has reached it. Its volume grid lives in a static 16 MiB
 * device array (4,194,304 grid nodes) that every GPU which loads this library keeps until the process exits;
 * a domain whose padded grid needs more nodes is refused with MPM_ERR_VALUE. All calls share that array,
 * so calls whose work overlaps on the GPU race. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture. Errors: mpm_last_error(NULL). */
int mpm_is_occupied_noalloc(const MpmDomainDesc *domain, int32_t particles_per_cell, int64_t n, const float *d_x,
                            int64_t m, const float *d_points, uint8_t *d_out, int32_t device, void *stream);

/* Batches. No counterpart in the reference, whose solver advances one scene per call: a batch advances many
 * independent scenes (handles created on one device) together. Every kernel of a substep is launched once for
 * all scenes of the batch from a device table of the scenes, and the launch sequence of one batched substep is
 * a CUDA graph replayed as often as the scene with the most substeps in the frame needs; each scene keeps its
 * own CFL time step, materials, colliders and particle order, and scenes whose frame is done sit idle. A
 * handle belongs to at most one batch; while it does, all of its work (including its own mpm_* calls) runs on
 * the batch's stream. Destroying a handle removes it from its batch. Errors: mpm_batch_last_error(batch). */
int mpm_batch_create(void **batch);
int mpm_batch_destroy(void *batch); /* member handles stay valid and leave the batch */
const char *mpm_batch_last_error(void *batch);
int mpm_batch_add(void *batch, void *handle);
int mpm_batch_remove(void *batch, void *handle);
int mpm_batch_size(void *batch, int32_t *n);
/* One frame of every scene, in the order they were added: frame_dt[i] for scene i (its advance(frame_dt),
 * mpm_core/solver.py:67-68), stats[i] as mpm_advance returns them. */
int mpm_batch_advance(void *batch, const double *frame_dt, MpmAdvanceStats *stats);
/* MPM_OPT_SORT_INTERVAL, MPM_OPT_G2P_VARIANT, MPM_OPT_LIST_CTAS, MPM_OPT_P2G_GROUP, MPM_OPT_PDL, MPM_OPT_P2G_TILE,
   MPM_OPT_P2G_MERGE for the batch */
int mpm_batch_set_option(void *batch, int32_t option, int64_t value);
int mpm_batch_get_stream(void *batch, void **stream);
/* Kernels launched by the batch and its scenes so far. */
int mpm_batch_launch_count(void *batch, int64_t *launches);

/* Emitter volume sampling on the device (mpm_core/geometry.py:89-151 up to the jitter): the points of the
 * cell-centred lattice xs x ys x zs (float64, as the reference builds it: (first + k + 0.5) * spacing) inside
 * a closed mesh by z-ray parity per (x, y) column, with the column centre nudged by nudge[2] (the reference's
 * _RAY_NUDGE * spacing). tri: (n_tris, 3, 3) float64 vertex coordinates. Every deciding operation is the
 * reference's, in FP64 and its order, each rounded on its own, so the same points come out in the same
 * order (columns in increasing i * ny + j, heights increasing). Writes n_out points (x, y, z float64) to out
 * when capacity >= n_out; call with out = NULL to learn n_out. The caller adds the reference's seeded
 * jitter. At most 2^31 column-triangle pairs. Errors: mpm_last_error(NULL). */
int mpm_volume_lattice(const double *tri, int64_t n_tris, const double *xs, int32_t nx, const double *ys, int32_t ny,
                       const double *zs, int32_t nz, double spacing, const double nudge[2], int64_t first_x,
                       int64_t first_y, int32_t device, double *out, int64_t capacity, int64_t *n_out);

/* The grid barrier of the cooperative substeps on its own (2 CTAs, the handle's device and stream): with
 * stall = 1 its arrival count is preset so that no CTA completes it, and each CTA gives up after its spin
 * limit (about a second) and sets the error flag, which *timed_out receives; with stall = 0 it completes and
 * *timed_out is 0. For tests of the bounded wait: the context stays usable either way. */
int mpm_coop_barrier_selftest(void *handle, int32_t stall, int32_t *timed_out);

/* ---- Surfacing (replaces the GPU part of mpm_surface/field.py:35-142, surface_particles) ----------------
 * A surfacer owns a stream and device buffers that grow as needed and stay from frame to frame.
 * mpm_surface_upload copies the n > 0 particles (x, v: (n, 3) float32 host arrays) to the device and returns
 * the per-axis minimum and maximum of x (NaN on an axis holding a NaN, as numpy's min and max), from which
 * the caller sets up the field grid (field.py:112-117). mpm_surface_build then splats the uploaded
 * particles onto a dims[0] x dims[1] x dims[2] node grid (fewer than 2^31 nodes) at `origin`
 * (float32, the field.py origin rounded) with spacing `cell` (inv_cell = the host's 1 / cell rounded to
 * float32): cubic B-spline kernel of radius h, density and momentum summed (field.py:35-57); velocity =
 * momentum / density where density > 0, density scaled by inv_rest (field.py:60-66); then marching cubes at
 * `iso` (a node is inside when its density is above iso; the case table is built from the cube's geometry,
 * mpm_mc_table), one vertex per crossing grid edge in node order then axis order, triangles in cell order,
 * wound outward; each vertex's velocity sampled trilinearly (field.py:69-89). n_verts and n_tris receive the
 * counts; mpm_surface_read copies verts ((n_verts, 3) float32 in grid index units), tris ((n_tris, 3) int32)
 * and vel ((n_verts, 3) float32) to host memory. Errors: mpm_surface_last_error(surfacer). */
int mpm_surface_create(int32_t device, void **surfacer);
int mpm_surface_destroy(void *surfacer);
const char *mpm_surface_last_error(void *surfacer);
int mpm_surface_upload(void *surfacer, int64_t n, const float *x, const float *v, float lo[3], float hi[3]);
int mpm_surface_build(void *surfacer, const float origin[3], const int32_t dims[3], float cell, float inv_cell,
                      float h, float inv_rest, float iso, int64_t *n_verts, int64_t *n_tris);
int mpm_surface_read(void *surfacer, float *verts, int32_t *tris, float *vel);
/* The last build's fields, for checking: density (dims, float32, normalised) and field (dims x 4 float32:
 * velocity xyz where the raw density is positive, else the zero momentum, and the raw density). */
int mpm_surface_read_field(void *surfacer, float *density, float *field);
/* The marching-cubes case table the surfacer uses (host only): ntri[256] triangle counts, edges[256 * 36]
 * edge ids (triangle t of case m at edges[m * 36 + 3 t .. + 2]; corner c = x + 2 y + 4 z, edge e = 4 a + s
 * along axis a from the corner whose other coordinates, in cyclic axis order, are the bits of s). */
int mpm_mc_table(int8_t *ntri, int8_t *edges);

#ifdef __cplusplus
}
#endif
#endif
