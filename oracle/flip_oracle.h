/*
 * flip_oracle.h — CPU oracle for the flip3d per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates, on the CPU, the
 * reference's sorter, mapper, solver, corrector and driver grid stages so that
 * tests, the smoke check and the CPU-baseline leg of bench.py can check the
 * CUDA path against it. The product (libflipgpu) never links, loads or calls
 * it. Its parity with the reference itself is pinned by golden vectors that
 * tests/golden/make_golden.py generates from the reference sources.
 *
 * Layouts (shared with the CUDA C-ABI in include/flipgpu.h):
 *   particles   pos/vel/nrm float[np][3] (x,y,z), type uint8 (1 fluid, 2 wall)
 *   cell fields x-major: index (i*n + j)*n + k, k fastest (the reference's
 *               A[i][j][k] with k contiguous)
 *   face grids  u0 (n+1)*n*n, u1 n*(n+1)*n, u2 n*n*(n+1), x-major on their
 *               own extents
 *   cell lists  cell_start[n^3+1], perm[np]: the particles of cell c are
 *               perm[cell_start[c] .. cell_start[c+1]) in particle order
 */
#ifndef FLIP_ORACLE_H
#define FLIP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_AIR = 0, ORC_FLUID = 1, ORC_WALL = 2 };

/* Preconditioners: 0 none, 1 the reference's as written (src/solver.cpp:
 * 119-180, whose neighbour terms only act on values equal to 1.0), 2 IC(0)/
 * MIC(0) with the neighbour test on the cell flag (tau 0 = IC(0)). */
enum { ORC_PRECOND_NONE = 0, ORC_PRECOND_REF = 1, ORC_PRECOND_IC = 2 };

typedef struct {
  int n;            /* N: cells per axis */
  float density;    /* DENSITY (0.5): particle spacing in cells */
  double alpha;     /* ALPHA (0.95): FLIP fraction */
  double dt;        /* DT (0.006) */
  double gravity;   /* GRAVITY (9.8) */
  int subcell;      /* SUBCELL (1) */
  int precond;      /* ORC_PRECOND_* */
  double mic_tau;   /* 0 = IC(0), 0.97 = MIC(0) (ORC_PRECOND_IC only) */
  double eps_abs;   /* CG stop: float(r.r) <= eps_abs; <0 = reference 1e-2*n^3 */
  double rel_tol;   /* >0: eps_abs = power-of-4 rounding of rel_tol^2 * b.b */
  int max_iters;    /* <=0: n^3 like the reference */
  uint64_t seed;    /* counter-RNG seed */
} OrcParams;

/* sorter::sort (src/sorter.cpp:22-40) as a stable counting sort. */
void orc_sort(int n, int np, const float *pos, uint32_t *cell_start,
              uint32_t *perm);

/* computeDensity (src/flip3D.cpp:166-190). kernel_h = (float)(4*DENSITY/N). */
void orc_density(int n, int np, const float *pos, const uint8_t *type,
                 const uint32_t *cs, const uint32_t *perm, float kernel_h,
                 float max_dens, float *dens);

/* sorter::levelset over every cell (src/sorter.cpp:70-81). */
void orc_levelset(int n, const uint8_t *type, const float *dens,
                  const uint32_t *cs, const uint32_t *perm, float density,
                  float *L);

/* sorter::markWater (src/sorter.cpp:83-93). */
void orc_mark_water(int n, const uint8_t *type, const float *dens,
                    const uint32_t *cs, const uint32_t *perm, float density,
                    uint8_t *A);

/* mapper::mapP2G (src/mapper.cpp:17-88). */
void orc_p2g(int n, int np, const float *pos, const float *vel,
             const uint8_t *type, const uint32_t *cs, const uint32_t *perm,
             float *u0, float *u1, float *u2);

/* mapper::fetchVelocity for every particle (src/mapper.cpp:90-112);
 * fluid_only skips wall particles (their velocity is never read). */
void orc_g2p(int n, int np, const float *pos, const uint8_t *type,
             const float *u0, const float *u1, const float *u2, float *vel,
             int fluid_only);

/* Driver grid stages (src/flip3D.cpp). */
void orc_enforce_boundary(int n, const uint8_t *A, float *u0, float *u1,
                          float *u2);
void orc_divergence(int n, const uint8_t *A, const float *u0, const float *u1,
                    const float *u2, float *div);
void orc_subtract_gradient(int n, int subcell, const float *L,
                           const float *press, float *u0, float *u1,
                           float *u2);
void orc_extrapolate(int n, const uint8_t *A, float *u0, float *u1, float *u2);

/* solver::solve (src/solver.cpp:224-241): negates b, builds the
 * preconditioner, runs PCG on x. Returns the iteration count. */
int orc_solve(const OrcParams *prm, const uint8_t *A, const float *L, float *x,
              float *b, double *final_r2, double *b2);

/* Preconditioner apply z = M^-1 r for tests (builds the factor each call). */
void orc_precond_apply(const OrcParams *prm, const uint8_t *A, const float *L,
                       const float *r, float *z);

/* compute_Ax (src/solver.cpp:29-41). */
void orc_matvec(int n, int subcell, const uint8_t *A, const float *L,
                const float *x, float *ans);

/* corrector::correct (src/corrector.cpp:49-115) on sorted cell lists that
 * the caller built from the current positions. */
void orc_correct(int n, int np, float *pos, float *vel, const uint8_t *type,
                 const float *nrm, const uint32_t *cs, const uint32_t *perm,
                 float dt, float re, uint64_t seed, int64_t step);

/* corrector::resample (src/corrector.cpp:15-47) at one position. */
void orc_resample(int n, const float *pos, const float *vel,
                  const uint8_t *type, const uint32_t *cs,
                  const uint32_t *perm, const float p[3], float u[3], float re);

/* Whole simulation state for multi-step runs and the CPU baseline. */
typedef struct OrcSim OrcSim;
OrcSim *orc_sim_create(const OrcParams *prm, int np, const float *pos,
                       const float *vel, const uint8_t *type, const float *nrm,
                       float max_dens);
void orc_sim_destroy(OrcSim *s);
/* One simulateStep (src/flip3D.cpp:1194-1264) without preview/mesh I/O.
 * Returns the CG iteration count of the step. */
int orc_sim_step(OrcSim *s);
/* Individual stages, for stage-by-stage parity. */
void orc_sim_stage(OrcSim *s, int stage);
int orc_sim_count(const OrcSim *s);
void orc_sim_get(const OrcSim *s, float *pos, float *vel, float *dens,
                 uint8_t *type);
void orc_sim_get_grid(const OrcSim *s, float *u0, float *u1, float *u2,
                      uint8_t *A, float *L, float *press);
void orc_sim_put(OrcSim *s, const float *pos, const float *vel, const float *dens);
void orc_sim_put_grid(OrcSim *s, const float *u0, const float *u1, const float *u2,
                      const uint8_t *A, const float *L, const float *press);
int orc_sim_last_stuck(const OrcSim *s);
double orc_sim_last_r2(const OrcSim *s);
void orc_sim_set_step(OrcSim *s, int64_t step);
void orc_sim_set_threads(int nthreads);

/* implicit::implicit_func (src/implicit.cpp:14-38) at m points. */
void orc_implicit(int n, const float *pos, const uint8_t *type, const uint32_t *cs,
                  const uint32_t *perm, float density, int m, const float *pts,
                  double *out);

/* mesher::generateMesh (src/mesher.cpp:137-195) with mg = n+1 on the cell
 * lists cs/perm over positions pos. The result stays in an OrcMesh until
 * orc_mesh_free; phi is the field it meshed, (n+1)^3 floats in the
 * reference's layout (x fastest). */
typedef struct OrcMesh OrcMesh;
OrcMesh *orc_mesh(int n, const float *pos, const uint8_t *type, const uint32_t *cs,
                  const uint32_t *perm, float density);
void orc_mesh_counts(const OrcMesh *m, int64_t *nverts, int64_t *nfaces, int64_t *ntris);
void orc_mesh_get(const OrcMesh *m, double *vertices, double *normals, int32_t *faces,
                  float *phi);
void orc_mesh_free(OrcMesh *m);
OrcMesh *orc_sim_mesh(const OrcSim *s);

/* Max-density calibration (src/flip3D.cpp:689-709). */
float orc_max_density(int n, float density);

#ifdef __cplusplus
}
#endif
#endif
