/* CPU oracle of the reference MLS-MPM substep. TEST INFRASTRUCTURE ONLY.
 *
 * This is the checker the CUDA backend is compared against: a plain-C restatement of the reference's
 * Warp kernels (mpm_core/backends/warp/kernels.py, colliders.py) and of the per-substep launch order of
 * mpm_core/backends/warp/solver.py. It is compiled twice, with REAL = float (the reference's own FP32
 * arithmetic) and REAL = double (the FP64 oracle of the same substep). Only the tests, the smoke check and
 * the CPU-baseline leg of bench.py load it; the product never links or calls it.
 *
 * Parity is pinned by the golden fixtures in tests/golden/, which were produced by running the reference's
 * own kernel and solver code (through a CPU emulation of the Warp API) on seeded scenes.
 *
 * Grid layout: dims[0]*dims[1]*dims[2] nodes in C order (k fastest), 4 REALs per node:
 * momentum (later velocity) x, y, z and mass. Particle layout: x, v (N,3); C, F (N,3,3) row-major; Jp (N).
 */
#ifndef MPM_ORACLE_H
#define MPM_ORACLE_H

#include <stdint.h>

#ifdef ORACLE_DOUBLE
typedef double REAL;
#else
typedef float REAL;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Host-side constants, computed in float64 exactly as warp/solver.py:37-53 does, converted to REAL here. */
typedef struct OrcDomain {
    int dims[3];
    int wall_lo_node[3], wall_hi_node[3], lo_on[3], hi_on[3];
    double origin[3];
    double dx, inv_dx, p_vol;
    double gravity[3];
    double wall_friction;
    double wall_lo[3], wall_hi[3], clamp_lo[3], clamp_hi[3];
    double thickness, band; /* collider thickness (2 dx) and contact band (dx), warp/solver.py:20,201 */
} OrcDomain;

/* One entry of the per-material tables built at warp/solver.py:56-71. */
typedef struct OrcMaterial {
    int model; /* 0 elastic, 1 von Mises, 2 Drucker-Prager, 3 snow (kernels.py:8-13) */
    double mu, lam, yield_stress, alpha, hardening, max_hardening, crit_c, crit_s, density;
} OrcMaterial;

/* A collider: its mesh (local space), its flags and its pose pair for the current advance. */
typedef struct OrcCollider {
    void *mesh; /* from orc_mesh_new */
    int closed;
    double friction, margin;
    double aabb_lo[3], aabb_hi[3];
    double t0[3], t1[3], q0[4], q1[4], S0[9], S1[9]; /* quaternions x, y, z, w */
} OrcCollider;

void *orc_mesh_new(int n_verts, const float *verts, int n_tris, const int *tris);
void orc_mesh_free(void *mesh);
/* Closest point query with pseudonormal sign; returns face index, writes sign, barycentrics u, v. */
int orc_mesh_query(const void *mesh, const double p[3], double *sign, double *u, double *v, double *dist2);

void orc_svd3(const REAL *A, REAL *U, REAL *sig, REAL *V);

void orc_p2g(const OrcDomain *d, const OrcMaterial *mats, int n, const REAL *x, const REAL *v, const REAL *C,
             const REAL *F, const REAL *Jp, const int32_t *mat, REAL dt, REAL *grid, int threads);
void orc_grid_update(const OrcDomain *d, REAL dt, REAL *grid, int threads);
void orc_grid_colliders(const OrcDomain *d, int n_col, const OrcCollider *cols, REAL s, REAL inv_frame_dt,
                        REAL *grid, int threads);
void orc_g2p(const OrcDomain *d, const OrcMaterial *mats, int n, REAL *x, REAL *v, REAL *C, REAL *F, REAL *Jp,
             const int32_t *mat, REAL dt, const REAL *grid, int threads);
void orc_project_particles(const OrcDomain *d, int n_col, const OrcCollider *cols, REAL s, REAL inv_frame_dt,
                           int n, REAL *x, REAL *v, int threads);
/* One whole substep in the order of warp/solver.py:187-211; grid is scratch of dims*4 REALs. */
void orc_substep(const OrcDomain *d, const OrcMaterial *mats, int n_col, const OrcCollider *cols, int n, REAL *x,
                 REAL *v, REAL *C, REAL *F, REAL *Jp, const int32_t *mat, REAL dt, REAL s, REAL inv_frame_dt,
                 REAL *grid, int threads);
/* Collider pose at s as 4x4 row-major matrices: M, its inverse, and the central-difference dM/dt. */
void orc_collider_pose(const OrcCollider *c, REAL s, REAL inv_frame_dt, REAL *M16, REAL *Minv16, REAL *dM16);
REAL orc_max_speed(int n, const REAL *v);
void orc_scatter_volume(const OrcDomain *d, int n, const REAL *x, REAL *grid_vol);
void orc_query_fill(const OrcDomain *d, int m, const REAL *pts, const REAL *grid_vol, uint8_t *out);

#ifdef __cplusplus
}
#endif
#endif
