/*
 * ref_harness.cpp — drives the reference's own C++ (built from the read-only
 * reference sources by oracle/Makefile into oracle/_ref/libflipref.so) on
 * arrays supplied by tests/golden/make_golden.py.
 *
 * TEST INFRASTRUCTURE ONLY. Used in the build container to generate golden
 * vectors and to pin the CPU oracle; it never ships and never runs on the GPU
 * box (the reference sources are not there).
 *
 * This translation unit includes the reference driver src/flip3D.cpp so that
 * its file-static stages (computeDensity, solve_picflip, advect_particle, ...)
 * and state can be driven directly. N is fixed at 32 by that file
 * (src/flip3D.cpp:25), so the driver-level entry points (fr_sim_*) run at
 * N=32; the sorter/mapper/solver/corrector entry points take any n.
 *
 * Documented patches, none of which edits a reference file:
 *   - rand() in this unit (reposition, src/flip3D.cpp:438-440) draws keyed
 *     values: draw d of a reposition call is flip_rand31(seed,
 *     PLACE stream of the step, d, 0);
 *   - my_rand_shuffle (src/utility.cpp:28-30, renamed away by -D when
 *     utility.cpp is compiled) is defined here as a keyed Fisher-Yates;
 *   - rand() in src/corrector.cpp is keyed by ref_patch_rand.h;
 *   - solver::solve (src/solver.cpp:224, renamed by -D to
 *     flipref_solver_solve_impl) is wrapped here: for a relative tolerance
 *     the wrapper scales b and x by an exact power of two 2^k before the call
 *     and back after it, which runs the unmodified CG with its absolute stop
 *     test 1e-2*n^3 equivalent to 1e-2*n^3/4^k on the unscaled system.
 */
#include <stdlib.h>
#include <cstdlib>
#include <stdint.h>
#include "../include/flip_rng.h"

extern "C" int flipref_place_rand(void);
#define rand() flipref_place_rand()
#include "flip3D.cpp"
#undef rand
#include "implicit.h"

#include <sys/stat.h>
#include <unistd.h>

namespace solver {
void flipref_solver_solve_impl(char ***A, FLOAT ***L, FLOAT ***x, FLOAT ***b,
                               int n);
}

static uint64_t g_seed = 0;
static int64_t g_rng_step = 0;
static int g_place_count = 0;
static particle *g_pool = NULL;
static int g_pool_n = 0;
static double g_rel_tol = 0.0;
static int g_last_scale_pow = 0;

extern "C" int flipref_place_rand(void) {
  int d = g_place_count++;
  return (int)flip_rand31(g_seed, flip_stream(FLIP_RNG_PLACE, (uint64_t)g_rng_step, 0),
                          (uint64_t)d, 0);
}

extern "C" int flipref_kick_rand(const void *p, const void *np) {
  static thread_local int comp = 0;
  int c = comp;
  comp = (comp + 1) % 3;
  uint64_t i = (uint64_t)((const particle *)p - g_pool);
  uint64_t j = (uint64_t)((const particle *)np - g_pool);
  return (int)flip_rand31(g_seed, flip_stream(FLIP_RNG_KICK, (uint64_t)g_rng_step, c), i, j);
}

void my_rand_shuffle(std::vector<ipos> &waters) {
  if (waters.size() < 2) return;
  for (size_t i = waters.size() - 1; i >= 1; i--) {
    uint32_t r = flip_rand31(g_seed, flip_stream(FLIP_RNG_SHUFFLE, (uint64_t)g_rng_step, 0),
                             (uint64_t)i, 0);
    size_t j = r % (uint32_t)(i + 1);
    ipos t = waters[i];
    waters[i] = waters[j];
    waters[j] = t;
  }
}

/* Wrapper around the reference solve: exact power-of-two scaling for a
 * relative tolerance (see the header comment). */
void solver::solve(char ***A, FLOAT ***L, FLOAT ***x, FLOAT ***b, int n) {
  int k = 0;
  if (g_rel_tol > 0.0) {
    double b2 = 0.0;
    for (int kk = 0; kk < n; kk++)
      for (int jj = 0; jj < n; jj++)
        for (int ii = 0; ii < n; ii++)
          if (A[ii][jj][kk] == FLUID) b2 += b[ii][jj][kk] * b[ii][jj][kk];
    double eps = 1.0e-2 * (n * n * n);
    double target = g_rel_tol * g_rel_tol * b2;
    while (eps > target && eps > 0.0) {
      eps *= 0.25;
      k++;
    }
  }
  g_last_scale_pow = k;
  const FLOAT s = (FLOAT)ldexp(1.0, k);
  if (k) {
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int kk = 0; kk < n; kk++) {
          x[i][j][kk] *= s;
          b[i][j][kk] *= s;
        }
  }
  solver::flipref_solver_solve_impl(A, L, x, b, n);
  if (k) {
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int kk = 0; kk < n; kk++) {
          x[i][j][kk] /= s;
          b[i][j][kk] /= s;
        }
  }
}

/* ------------------------------------------------------------------ utils */

static void ensure_log_dir() {
  /* dump() appends to render/log/console.out in the working directory. */
  mkdir("render", 0755);
  mkdir("render/log", 0755);
}

static void make_pool(int np, const float *pos, const float *vel,
                      const uint8_t *type, const float *nrm, const float *dens) {
  delete[] g_pool;
  g_pool = new particle[np > 0 ? np : 1];
  g_pool_n = np;
  for (int q = 0; q < np; q++) {
    particle &P = g_pool[q];
    memset(&P, 0, sizeof(P));
    for (int c = 0; c < 3; c++) {
      P.p[c] = pos[3 * q + c];
      P.u[c] = vel ? vel[3 * q + c] : 0.0f;
      P.n[c] = nrm ? nrm[3 * q + c] : 0.0f;
    }
    P.type = (char)type[q];
    P.m = 1.0f;
    P.dens = dens ? dens[q] : 0.0f;
  }
}

static void pool_vector(std::vector<particle *> &v) {
  v.clear();
  for (int q = 0; q < g_pool_n; q++) v.push_back(&g_pool[q]);
}

static void read_cells(sorter *s, int n, uint32_t *cs, uint32_t *perm) {
  uint32_t at = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        cs[(i * n + j) * n + k] = at;
        std::vector<particle *> v = s->getNeigboringParticles_cell(i, j, k, 0, 0, 0);
        for (size_t a = 0; a < v.size(); a++) perm[at++] = (uint32_t)(v[a] - g_pool);
      }
  cs[n * n * n] = at;
}

/* flat arrays are float (or char) whatever FLOAT is: the FP64 build
 * (FLOAT = double) widens on the way in and rounds on the way out */
template <class T, class U> static void to3(T ***g, int w, int h, int d, const U *flat) {
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++)
      for (int k = 0; k < d; k++) g[i][j][k] = (T)flat[(i * h + j) * d + k];
}
template <class T, class U> static void from3(T ***g, int w, int h, int d, U *flat) {
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++)
      for (int k = 0; k < d; k++) flat[(i * h + j) * d + k] = (U)g[i][j][k];
}

/* -------------------------------------------------------- sorter / mapper */

extern "C" void fr_sort(int n, int np, const float *pos, const uint8_t *type,
                        uint32_t *cs, uint32_t *perm) {
  make_pool(np, pos, NULL, type, NULL, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  s.sort(v);
  read_cells(&s, n, cs, perm);
}

extern "C" void fr_mark_water(int n, int np, const float *pos,
                              const uint8_t *type, const float *dens,
                              uint8_t *Aout, float *Lout) {
  make_pool(np, pos, NULL, type, NULL, dens);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  s.sort(v);
  char ***AA = alloc3D<char>(n, n, n);
  FLOAT ***hw = alloc3D<FLOAT>(n, n, n);
  s.markWater(AA, hw, (FLOAT)DENSITY);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        Aout[(i * n + j) * n + k] = (uint8_t)AA[i][j][k];
        Lout[(i * n + j) * n + k] = s.levelset(i, j, k, hw, (FLOAT)DENSITY);
      }
}

extern "C" void fr_p2g(int n, int np, const float *pos, const float *vel,
                       const uint8_t *type, float *u0, float *u1, float *u2) {
  make_pool(np, pos, vel, type, NULL, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  s.sort(v);
  FLOAT ***g[3] = {alloc3D<FLOAT>(n + 1, n, n), alloc3D<FLOAT>(n, n + 1, n),
                   alloc3D<FLOAT>(n, n, n + 1)};
  mapper::mapP2G(&s, v, g, n);
  from3(g[0], n + 1, n, n, u0);
  from3(g[1], n, n + 1, n, u1);
  from3(g[2], n, n, n + 1, u2);
}

extern "C" void fr_g2p(int n, int np, const float *pos, const uint8_t *type,
                       const float *u0, const float *u1, const float *u2,
                       float *vel) {
  make_pool(np, pos, NULL, type, NULL, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  FLOAT ***g[3] = {alloc3D<FLOAT>(n + 1, n, n), alloc3D<FLOAT>(n, n + 1, n),
                   alloc3D<FLOAT>(n, n, n + 1)};
  to3(g[0], n + 1, n, n, u0);
  to3(g[1], n, n + 1, n, u1);
  to3(g[2], n, n, n + 1, u2);
  mapper::mapG2P(v, g, n);
  for (int q = 0; q < np; q++)
    for (int c = 0; c < 3; c++) vel[3 * q + c] = g_pool[q].u[c];
}

/* solver::solve on one system; rel_tol > 0 selects the scaled tolerance.
 * Returns the power k of the scale that was used. One n per process: the
 * solver sizes its static scratch at its first call. */
extern "C" int fr_solve(int n, int subcell, double rel_tol, const uint8_t *Ain,
                        const float *Lin, float *x, float *b) {
  ensure_log_dir();
  char ***AA = alloc3D<char>(n, n, n);
  FLOAT ***LL = alloc3D<FLOAT>(n, n, n);
  FLOAT ***xx = alloc3D<FLOAT>(n, n, n);
  FLOAT ***bb = alloc3D<FLOAT>(n, n, n);
  to3(AA, n, n, n, (const char *)Ain);
  to3(LL, n, n, n, Lin);
  to3(xx, n, n, n, x);
  to3(bb, n, n, n, b);
  g_rel_tol = rel_tol;
  solver::setSubcell((char)subcell);
  solver::solve(AA, LL, xx, bb, n);
  from3(xx, n, n, n, x);
  from3(bb, n, n, n, b);
  return g_last_scale_pow;
}

extern "C" void fr_correct(int n, int np, float *pos, float *vel,
                           const uint8_t *type, const float *nrm, float dt,
                           float re, uint64_t seed, int64_t step) {
  make_pool(np, pos, vel, type, nrm, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  g_seed = seed;
  g_rng_step = step;
  corrector::correct(&s, v, dt, re);
  for (int q = 0; q < np; q++)
    for (int c = 0; c < 3; c++) {
      pos[3 * q + c] = g_pool[q].p[c];
      vel[3 * q + c] = g_pool[q].u[c];
    }
}

/* ------------------------------------------------- driver stages at N=32 */

extern "C" int fr_grid_n(void) { return N; }

extern "C" void fr_sim_setup(int np, const float *pos, const float *vel,
                             const uint8_t *type, const float *nrm,
                             float maxd, uint64_t seed, double rel_tol) {
  ensure_log_dir();
  if (!u[0]) {
    u[0] = alloc3D<FLOAT>(N + 1, N, N);
    u[1] = alloc3D<FLOAT>(N, N + 1, N);
    u[2] = alloc3D<FLOAT>(N, N, N + 1);
    u_save[0] = alloc3D<FLOAT>(N + 1, N, N);
    u_save[1] = alloc3D<FLOAT>(N, N + 1, N);
    u_save[2] = alloc3D<FLOAT>(N, N, N + 1);
    A = alloc3D<char>(N, N, N);
    L = alloc3D<FLOAT>(N, N, N);
    press = alloc3D<FLOAT>(N, N, N);
    for (int c = 0; c < 4; c++) wall_normal[c] = alloc3D<FLOAT>(N, N, N);
    sort = new sorter(N);
  }
  FOR_EVERY_X_FLOW { u_save[0][i][j][k] = u[0][i][j][k] = 0.0; } END_FOR
  FOR_EVERY_Y_FLOW { u_save[1][i][j][k] = u[1][i][j][k] = 0.0; } END_FOR
  FOR_EVERY_Z_FLOW { u_save[2][i][j][k] = u[2][i][j][k] = 0.0; } END_FOR
  FOR_EVERY_CELL(N) {
    A[i][j][k] = AIR;
    press[i][j][k] = 0.0;
    L[i][j][k] = 0.0;
  } END_FOR
  make_pool(np, pos, vel, type, nrm, NULL);
  pool_vector(particles);
  max_dens = maxd;
  step = 0;
  g_seed = seed;
  g_rel_tol = rel_tol;
  solver::setSubcell(SUBCELL);
}

/* 0 sort+computeDensity, 1 add_ExtForce, 2 solve_picflip, 3 advect_particle,
 * 4 corrector::correct — the order of simulateStep (src/flip3D.cpp:1194-1264). */
extern "C" void fr_sim_stage(int stage) {
  switch (stage) {
  case 0:
    step++;
    g_rng_step = step;
    sort->sort(particles);
    computeDensity();
    break;
  case 1:
    add_ExtForce();
    break;
  case 2:
    solve_picflip();
    break;
  case 3:
    g_place_count = 0;
    advect_particle();
    break;
  case 4:
    corrector::correct(sort, particles, DT, DENSITY / N);
    break;
  default:
    break;
  }
}

extern "C" int fr_sim_stuck(void) { return gNumStuck; }

/* ---------------------------------------------------------------- mesher */

/* implicit::implicit_func at m points on freshly sorted particles. */
extern "C" void fr_implicit(int n, int np, const float *pos, const uint8_t *type,
                            float density, int m, const float *pts, double *out) {
  make_pool(np, pos, NULL, type, NULL, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  s.sort(v);
  for (int i = 0; i < m; i++) {
    FLOAT p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    out[i] = implicit::implicit_func(&s, p, density);
  }
}

/* mesher::generateMesh keeps buffers sized by its first call (one grid size
 * per process). The result stays here until the next call. */
static std::vector<double> g_mesh_v, g_mesh_n;
static std::vector<int> g_mesh_f;

extern "C" void fr_mesh(int n, int np, const float *pos, const uint8_t *type,
                        float density, int64_t *counts) {
  make_pool(np, pos, NULL, type, NULL, NULL);
  std::vector<particle *> v;
  pool_vector(v);
  sorter s(n);
  s.sort(v);
  mesher::generateMesh(NULL, &s, v, density, n + 1, g_mesh_v, g_mesh_n, g_mesh_f);
  counts[0] = (int64_t)(g_mesh_v.size() / 3);
  counts[1] = (int64_t)(g_mesh_f.size() / 3);
}

/* The mesh write_mesh makes after a driver step (src/flip3D.cpp:999-1004):
 * the driver's current lists and positions. */
extern "C" void fr_sim_mesh(int64_t *counts) {
  mesher::generateMesh(A, sort, particles, DENSITY, N + 1, g_mesh_v, g_mesh_n, g_mesh_f);
  counts[0] = (int64_t)(g_mesh_v.size() / 3);
  counts[1] = (int64_t)(g_mesh_f.size() / 3);
}

extern "C" void fr_mesh_get(double *vert, double *nrm, int32_t *faces) {
  memcpy(vert, g_mesh_v.data(), g_mesh_v.size() * sizeof(double));
  memcpy(nrm, g_mesh_n.data(), g_mesh_n.size() * sizeof(double));
  for (size_t i = 0; i < g_mesh_f.size(); i++) faces[i] = g_mesh_f[i];
}

extern "C" void fr_sim_get(float *pos, float *vel, float *dens, uint8_t *type) {
  for (int q = 0; q < g_pool_n; q++) {
    for (int c = 0; c < 3; c++) {
      if (pos) pos[3 * q + c] = g_pool[q].p[c];
      if (vel) vel[3 * q + c] = g_pool[q].u[c];
    }
    if (dens) dens[q] = g_pool[q].dens;
    if (type) type[q] = (uint8_t)g_pool[q].type;
  }
}

extern "C" void fr_sim_get_grid(float *u0, float *u1, float *u2, uint8_t *Aout,
                                float *Lout, float *pout) {
  from3(u[0], N + 1, N, N, u0);
  from3(u[1], N, N + 1, N, u1);
  from3(u[2], N, N, N + 1, u2);
  from3(A, N, N, N, (char *)Aout);
  from3(L, N, N, N, Lout);
  from3(press, N, N, N, pout);
}

/* The driver's state at FLOAT resolution (the FP64 build's double values
 * unrounded): particle positions, velocities and densities, the face grids,
 * the levelset and the pressure. */
extern "C" void fr_sim_get_d(double *pos, double *vel, double *dens) {
  for (int q = 0; q < g_pool_n; q++) {
    for (int c = 0; c < 3; c++) {
      if (pos) pos[3 * q + c] = g_pool[q].p[c];
      if (vel) vel[3 * q + c] = g_pool[q].u[c];
    }
    if (dens) dens[q] = g_pool[q].dens;
  }
}

extern "C" void fr_sim_get_grid_d(double *u0, double *u1, double *u2, double *Lout,
                                  double *pout) {
  from3(u[0], N + 1, N, N, u0);
  from3(u[1], N, N + 1, N, u1);
  from3(u[2], N, N, N + 1, u2);
  from3(L, N, N, N, Lout);
  from3(press, N, N, N, pout);
}

extern "C" void fr_sim_set_max_density_d(double md) { max_dens = (FLOAT)md; }

static FLOAT max_density_impl(void);

/* Max-density calibration through the reference's computeDensity on the
 * lattice of src/flip3D.cpp:689-709. */
extern "C" float fr_max_density(void) { return (float)max_density_impl(); }
extern "C" double fr_max_density_d(void) { return (double)max_density_impl(); }

static FLOAT max_density_impl(void) {
  if (!sort) sort = new sorter(N);
  FLOAT h = DENSITY / N;
  int np = 1000;
  std::vector<float> pos(3 * np);
  std::vector<uint8_t> type(np, FLUID);
  int m = 0;
  FOR_EVERY_CELL(10) {
    pos[3 * m + 0] = (i + 0.5) * h;
    pos[3 * m + 1] = (j + 0.5) * h;
    pos[3 * m + 2] = (k + 0.5) * h;
    m++;
  } END_FOR
  make_pool(np, pos.data(), NULL, type.data(), NULL, NULL);
  pool_vector(particles);
  sort->sort(particles);
  max_dens = 1.0;
  computeDensity();
  FLOAT md = 0.0;
  for (int q = 0; q < np; q++) md = fmax(md, g_pool[q].dens);
  particles.clear();
  return md;
}

/* flip3D::init's own scene setup (src/flip3D.cpp:649-777: the walls and
 * damBreakTest objects at N=32, jittered with the keyed draws that replace
 * rand() in this unit, wall-cell removal, compute_wall_normal) followed by
 * its saveState (src/flip3D.cpp:453-516): writes render/save/0_scene.dat
 * under the current directory. Returns the particle count. */
extern "C" int fr_init_and_save(uint64_t seed) {
  g_seed = seed;
  g_rng_step = 0;
  g_place_count = 0;
  flip3D::init(0);
  saveState();
  return (int)particles.size();
}

/* exporter::write3D (src/exporter.cpp:160-167) on the last fr_mesh /
 * fr_sim_mesh result: render/obj/<step>_scene.obj and
 * render/sunflow/{template.sc,<step>_scene.sc} under the current directory. */
extern "C" void fr_export(int step, float wall_thick) {
  mkdir("render", 0755);
  std::vector<Object> objs;
  std::vector<particle *> parts;
  exporter::write3D(step, g_mesh_v, g_mesh_n, g_mesh_f, objs, parts, wall_thick);
}

/* write_frame (src/flip3D.cpp:1133-1192) on the driver's particles:
 * render/preview/frame_<step>.bmp under the current directory. */
extern "C" void fr_write_frame(void) {
  mkdir("render", 0755);
  mkdir("render/preview", 0755);
  write_frame();
}
