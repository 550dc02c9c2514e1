/*
 * shim.cpp — the reference's sorter / mapper / solver / corrector call
 * surface (src/sorter.h, src/mapper.h, src/solver.h, src/corrector.h,
 * src/mesher.h, src/implicit.h) on top
 * of the C ABI of libflipgpu, so a driver written against those functions
 * (src/flip3D.cpp) runs them on the GPU. Each call converts the driver's
 * particle records and jagged T*** grids (alloc3D, k contiguous) to the
 * library's flat layouts, runs the GPU entry point and writes the results
 * back in place, as the reference functions do. Errors abort with the
 * library's message: the reference has no error returns.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <vector>

#include "../../include/flipgpu.h"
#include "corrector.h"
#include "implicit.h"
#include "mapper.h"
#include "mesher.h"
#include "solver.h"
#include "sorter.h"

namespace {

void die(FlipGpu *h, const char *what, int rc) {
  fprintf(stderr, "flip3d shim: %s failed (%d): %s\n", what, rc,
          h ? flipgpu_last_error(h) : "no handle");
  abort();
}

#define CHECK(h, call)                 \
  do {                                 \
    int rc_ = (call);                  \
    if (rc_ != FLIPGPU_OK) die((h), #call, rc_); \
  } while (0)

/* A device context: one FlipGpu handle per grid size, grown on demand. */
struct Ctx {
  FlipGpu *h = nullptr;
  int n = 0;
  int cap = 0;
};

char g_subcell = 1;
double g_rel_tol = 0.0;
uint64_t g_seed = 0;
int64_t g_step = 0;
float g_density = 0.5f;
std::map<int, Ctx> g_ctx;

FlipGpuParams params_for(int n, int cap) {
  FlipGpuParams p;
  flipgpu_default_params(&p, n, cap);
  p.subcell = g_subcell;
  p.rel_tol = g_rel_tol;
  p.seed = g_seed;
  p.density = g_density;
  return p;
}

void ensure(Ctx &c, int n, int np) {
  if (!c.h || c.n != n || c.cap < np) {
    if (c.h) flipgpu_destroy(c.h);
    c.h = nullptr;
    c.n = n;
    c.cap = np > 1024 ? np + np / 4 : 1024;
    FlipGpuParams p = params_for(n, c.cap);
    int rc = flipgpu_create(&p, &c.h);
    if (rc != FLIPGPU_OK) die(nullptr, "flipgpu_create", rc);
  } else {
    FlipGpuParams p = params_for(n, c.cap);
    CHECK(c.h, flipgpu_set_params(c.h, &p));
  }
}

Ctx &ctx_for(int n) { return g_ctx[n]; }

struct Soa {
  std::vector<float> pos, vel, nrm, dens;
  std::vector<uint8_t> type;
};

void pack(const std::vector<particle *> &ps, Soa &s) {
  size_t np = ps.size();
  s.pos.resize(3 * np);
  s.vel.resize(3 * np);
  s.nrm.resize(3 * np);
  s.dens.resize(np);
  s.type.resize(np);
  for (size_t q = 0; q < np; q++) {
    const particle *p = ps[q];
    for (int c = 0; c < 3; c++) {
      s.pos[3 * q + c] = p->p[c];
      s.vel[3 * q + c] = p->u[c];
      s.nrm[3 * q + c] = p->n[c];
    }
    s.dens[q] = p->dens;
    s.type[q] = (uint8_t)p->type;
  }
}

void upload(Ctx &c, const std::vector<particle *> &ps) {
  Soa s;
  pack(ps, s);
  ensure(c, c.n, (int)ps.size());
  CHECK(c.h, flipgpu_set_particles(c.h, (int)ps.size(), s.pos.data(), s.vel.data(),
                                   s.type.data(), s.nrm.data(), s.dens.data(), 0));
}

template <class T> void flatten(T ***g, int w, int h, int d, std::vector<T> &out) {
  out.resize((size_t)w * h * d);
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++) memcpy(&out[((size_t)i * h + j) * d], g[i][j], d * sizeof(T));
}
template <class T> void unflatten(const std::vector<T> &in, int w, int h, int d, T ***g) {
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++) memcpy(g[i][j], &in[((size_t)i * h + j) * d], d * sizeof(T));
}

} // namespace

/* ----------------------------------------------------------------- sorter */

struct FlipShimCells {
  Ctx ctx;
  std::vector<particle *> parts;
  std::vector<uint32_t> cs, perm;
  std::vector<float> L;
  std::vector<uint8_t> A;
  bool L_valid = false;
};

sorter::sorter(int gn_) : cells_(new FlipShimCells()), gn(gn_) { cells_->ctx.n = gn_; }

sorter::~sorter() {
  if (cells_->ctx.h) flipgpu_destroy(cells_->ctx.h);
  delete cells_;
}

void sorter::sort(std::vector<particle *> &particles) {
  FlipShimCells &s = *cells_;
  upload(s.ctx, particles);
  CHECK(s.ctx.h, flipgpu_sort(s.ctx.h));
  s.parts = particles;
  s.cs.resize((size_t)gn * gn * gn + 1);
  s.perm.resize(particles.size());
  CHECK(s.ctx.h, flipgpu_get_cells(s.ctx.h, s.cs.data(), s.perm.data(), 0));
  s.L_valid = false;
}

static std::vector<particle *> gather(FlipShimCells &s, int gn, int i0, int i1, int j0, int j1,
                                      int k0, int k1) {
  std::vector<particle *> res;
  if (s.cs.empty()) return res;
  for (int si = i0; si <= i1; si++)
    for (int sj = j0; sj <= j1; sj++)
      for (int sk = k0; sk <= k1; sk++) {
        if (si < 0 || si > gn - 1 || sj < 0 || sj > gn - 1 || sk < 0 || sk > gn - 1) continue;
        size_t c = ((size_t)si * gn + sj) * gn + sk;
        for (uint32_t a = s.cs[c]; a < s.cs[c + 1]; a++) res.push_back(s.parts[s.perm[a]]);
      }
  return res;
}

std::vector<particle *> sorter::getNeigboringParticles_wall(int i, int j, int k, int w, int h,
                                                            int d) {
  return gather(*cells_, gn, i - w, i + w - 1, j - h, j + h - 1, k - d, k + d - 1);
}

std::vector<particle *> sorter::getNeigboringParticles_cell(int i, int j, int k, int w, int h,
                                                            int d) {
  return gather(*cells_, gn, i - w, i + w, j - h, j + h, k - d, k + d);
}

int sorter::getNumParticleAt(int i, int j, int k) {
  size_t c = ((size_t)i * gn + j) * gn + k;
  return cells_->cs.empty() ? 0 : (int)(cells_->cs[c + 1] - cells_->cs[c]);
}

/* markWater and levelset read the particles' current densities: the driver
 * computes them after sorting, so they are uploaded here. */
static void mark(sorter *so, FlipShimCells &s, int gn, FLOAT density) {
  g_density = density;
  upload(s.ctx, s.parts);
  CHECK(s.ctx.h, flipgpu_mark_water(s.ctx.h));
  size_t nc = (size_t)gn * gn * gn;
  s.A.resize(nc);
  s.L.resize(nc);
  CHECK(s.ctx.h, flipgpu_get_grid(s.ctx.h, nullptr, nullptr, nullptr, s.A.data(), s.L.data(),
                                  nullptr, nullptr, 0));
  s.L_valid = true;
  (void)so;
}

FLOAT sorter::levelset(int i, int j, int k, FLOAT ***halfwall, FLOAT density) {
  (void)halfwall;
  if (!cells_->L_valid || g_density != density) mark(this, *cells_, gn, density);
  return cells_->L[((size_t)i * gn + j) * gn + k];
}

void sorter::markWater(char ***A, FLOAT ***halfwall, FLOAT density) {
  (void)halfwall;
  mark(this, *cells_, gn, density);
  for (int i = 0; i < gn; i++)
    for (int j = 0; j < gn; j++)
      for (int k = 0; k < gn; k++) A[i][j][k] = (char)cells_->A[((size_t)i * gn + j) * gn + k];
}

void sorter::deleteAllParticles() {
  FlipShimCells &s = *cells_;
  size_t nc = (size_t)gn * gn * gn;
  for (size_t c = 0; c < nc && !s.cs.empty(); c++)
    for (uint32_t a = s.cs[c]; a < s.cs[c + 1]; a++) delete s.parts[s.perm[a]];
}

/* ----------------------------------------------------------------- mapper */

void mapper::mapP2G(sorter *sort, std::vector<particle *> &particles, FLOAT ****grid, int gn) {
  FlipShimCells &s = *sort->shim();
  upload(s.ctx, particles);
  CHECK(s.ctx.h, flipgpu_p2g(s.ctx.h));
  const size_t nf = (size_t)(gn + 1) * gn * gn;
  std::vector<float> u[3];
  for (int c = 0; c < 3; c++) u[c].resize(nf);
  CHECK(s.ctx.h, flipgpu_get_grid(s.ctx.h, u[0].data(), u[1].data(), u[2].data(), nullptr,
                                  nullptr, nullptr, nullptr, 0));
  unflatten(u[0], gn + 1, gn, gn, grid[0]);
  unflatten(u[1], gn, gn + 1, gn, grid[1]);
  unflatten(u[2], gn, gn, gn + 1, grid[2]);
}

static void put_grid(Ctx &c, FLOAT ****grid, int gn) {
  std::vector<float> u[3];
  flatten(grid[0], gn + 1, gn, gn, u[0]);
  flatten(grid[1], gn, gn + 1, gn, u[1]);
  flatten(grid[2], gn, gn, gn + 1, u[2]);
  CHECK(c.h, flipgpu_set_grid(c.h, u[0].data(), u[1].data(), u[2].data(), nullptr, nullptr,
                              nullptr, nullptr, 0));
}

void mapper::mapG2P(std::vector<particle *> &particles, FLOAT ****grid, int gn) {
  Ctx &c = ctx_for(gn);
  c.n = gn;
  upload(c, particles);
  put_grid(c, grid, gn);
  CHECK(c.h, flipgpu_g2p(c.h));
  std::vector<float> vel(3 * particles.size());
  CHECK(c.h, flipgpu_get_particles(c.h, nullptr, vel.data(), nullptr, nullptr, 0));
  for (size_t q = 0; q < particles.size(); q++)
    for (int k = 0; k < 3; k++) particles[q]->u[k] = vel[3 * q + k];
}

void mapper::fetchVelocity(FLOAT p[3], FLOAT u[3], FLOAT ****grid, int gn) {
  Ctx &c = ctx_for(gn);
  c.n = gn;
  ensure(c, gn, c.cap > 0 ? c.cap : 1024);
  put_grid(c, grid, gn);
  CHECK(c.h, flipgpu_fetch_velocity(c.h, 1, p, u, 0));
}

/* ----------------------------------------------------------------- solver */

void solver::setSubcell(char value) { g_subcell = value; }
void solver::setRelativeTolerance(double rel_tol) { g_rel_tol = rel_tol; }

void solver::solve(char ***A, FLOAT ***L, FLOAT ***x, FLOAT ***b, int n) {
  Ctx &c = ctx_for(n);
  c.n = n;
  ensure(c, n, c.cap > 0 ? c.cap : 1024);
  std::vector<char> Af;
  std::vector<float> Lf, xf, bf;
  flatten(A, n, n, n, Af);
  flatten(L, n, n, n, Lf);
  flatten(x, n, n, n, xf);
  flatten(b, n, n, n, bf);
  CHECK(c.h, flipgpu_set_grid(c.h, nullptr, nullptr, nullptr, (const uint8_t *)Af.data(),
                              Lf.data(), xf.data(), bf.data(), 0));
  FlipGpuSolveStats st;
  CHECK(c.h, flipgpu_solve(c.h, &st));
  CHECK(c.h, flipgpu_get_grid(c.h, nullptr, nullptr, nullptr, nullptr, nullptr, xf.data(),
                              bf.data(), 0));
  unflatten(xf, n, n, n, x);
  unflatten(bf, n, n, n, b);
}

/* -------------------------------------------------------------- corrector */

void corrector::setRandomKey(uint64_t seed, int64_t step) {
  g_seed = seed;
  g_step = step;
}

/* The reference reads the neighbours' current data through the sorter's
 * particle pointers (a reposition loop updates velocities between calls), so
 * the current records of the sorted particles are uploaded first. */
void corrector::resample(sorter *sort, FLOAT p[3], FLOAT u[3], FLOAT re) {
  FlipShimCells &s = *sort->shim();
  if (!s.ctx.h) return;
  Soa cur;
  pack(s.parts, cur);
  CHECK(s.ctx.h, flipgpu_put_state(s.ctx.h, cur.pos.data(), cur.vel.data(), 0));
  CHECK(s.ctx.h, flipgpu_resample(s.ctx.h, 1, p, u, re, 0));
}

void corrector::correct(sorter *sort, std::vector<particle *> &particles, FLOAT dt, FLOAT re) {
  FlipShimCells &s = *sort->shim();
  const int gn = sort->getCellSize();
  if ((double)re != (double)(FLOAT)((double)g_density / gn))
    fprintf(stderr, "flip3d shim: corrector radius %g is not DENSITY/N; using DENSITY/N\n",
            (double)re);
  upload(s.ctx, particles);
  FlipGpuParams p = params_for(gn, s.ctx.cap);
  p.dt = dt;
  CHECK(s.ctx.h, flipgpu_set_params(s.ctx.h, &p));
  CHECK(s.ctx.h, flipgpu_set_step(s.ctx.h, g_step));
  /* the reference's sorter keeps the lists of the positions before the move */
  CHECK(s.ctx.h, flipgpu_sort(s.ctx.h));
  s.parts = particles;
  s.cs.resize((size_t)gn * gn * gn + 1);
  s.perm.resize(particles.size());
  CHECK(s.ctx.h, flipgpu_get_cells(s.ctx.h, s.cs.data(), s.perm.data(), 0));
  s.L_valid = false;
  CHECK(s.ctx.h, flipgpu_correct(s.ctx.h));
  std::vector<float> pos(3 * particles.size()), vel(3 * particles.size());
  CHECK(s.ctx.h, flipgpu_get_particles(s.ctx.h, pos.data(), vel.data(), nullptr, nullptr, 0));
  for (size_t q = 0; q < particles.size(); q++) {
    if (particles[q]->type != FLUID) continue;
    for (int k = 0; k < 3; k++) {
      particles[q]->p[k] = pos[3 * q + k];
      particles[q]->u[k] = vel[3 * q + k];
    }
  }
}

/* ----------------------------------------------------------------- mesher */

/* The handle's density parameter and the particles' current positions (the
 * reference reads them through the sorter's pointers) before a field query. */
static void prepare_field(FlipShimCells &s, int gn, FLOAT density) {
  if (g_density != density) {
    g_density = density;
    FlipGpuParams p = params_for(gn, s.ctx.cap);
    CHECK(s.ctx.h, flipgpu_set_params(s.ctx.h, &p));
  }
  Soa cur;
  pack(s.parts, cur);
  CHECK(s.ctx.h, flipgpu_put_state(s.ctx.h, cur.pos.data(), cur.vel.data(), 0));
}

double implicit::implicit_func(sorter *sort, FLOAT p[3], FLOAT density) {
  FlipShimCells &s = *sort->shim();
  const int gn = sort->getCellSize();
  if (!s.ctx.h) return 8.0 * density / gn - (double)(density / gn); /* no particles */
  prepare_field(s, gn, density);
  double out = 0.0;
  CHECK(s.ctx.h, flipgpu_implicit(s.ctx.h, 1, p, &out, 0));
  return out;
}

void mesher::generateMesh(char ***A, sorter *sort, std::vector<particle *> &particles,
                          FLOAT density, int mg, std::vector<double> &vertices,
                          std::vector<double> &normals, std::vector<int> &faces) {
  (void)A;
  (void)particles;
  FlipShimCells &s = *sort->shim();
  const int gn = sort->getCellSize();
  vertices.clear();
  normals.clear();
  faces.clear();
  if (mg != gn + 1) {
    fprintf(stderr, "flip3d shim: generateMesh needs mg = grid size + 1 (%d), got %d\n", gn + 1,
            mg);
    abort();
  }
  if (!s.ctx.h) return;
  prepare_field(s, gn, density);
  int64_t nv = 0, nf = 0;
  CHECK(s.ctx.h, flipgpu_mesh(s.ctx.h, &nv, &nf));
  vertices.resize(3 * (size_t)nv);
  normals.resize(3 * (size_t)nv);
  std::vector<int32_t> f(3 * (size_t)nf);
  CHECK(s.ctx.h, flipgpu_get_mesh(s.ctx.h, vertices.data(), normals.data(), f.data(), nullptr));
  faces.assign(f.begin(), f.end());
}
