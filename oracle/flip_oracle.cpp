/*
 * flip_oracle.cpp — CPU oracle for the flip3d per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker used by tests/, by
 * __graft_entry__.smoke() and by the CPU-baseline leg of bench.py. The CUDA
 * product never links or calls it.
 *
 * Every function restates one reference function with the reference's own
 * arithmetic: FLOAT is float, and wherever the reference promotes to double
 * (double literals, fmax/fmin with mixed arguments, double locals) this code
 * promotes at the same point and rounds back at the same point, in the same
 * evaluation order. Build with -ffp-contract=off so that no multiply-add is
 * fused (the x86-64 reference build has no FMA; on aarch64 gcc would fuse by
 * default). Cross-cell sums run in the reference's loop order, so results do
 * not depend on the OpenMP thread count.
 *
 * Deliberate differences from the reference (the only two):
 *   - rand()/random_shuffle are replaced by the counter-based generator of
 *     include/flip_rng.h (the reference harness applies the same patch);
 *   - the trilinear fetch of the v grid clamps k+1 to the row where the
 *     reference reads one element past the row (src/mapper.cpp:102 clamps k
 *     with h-2 instead of d-2); that happens only for positions with
 *     n*z > n-0.5, outside the walls, which fluid particles never reach.
 */
#include "flip_oracle.h"
#include "../include/flip_rng.h"
#include "../include/flip_mc_table.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ---------------------------------------------------------------- kernels */

/* kernel::smooth_kernel (src/kernel.cpp:4-6): fmax(1.0 - r2/(h*h), 0.0). */
inline float smooth_kernel(float r2, float h) {
  float q = r2 / (h * h);
  return (float)std::fmax(1.0 - (double)q, 0.0);
}

/* kernel::sharp_kernel (src/kernel.cpp:8-10):
 * fmax(h*h/fmax(r2,1.0e-5) - 1.0, 0.0); the division runs in double. */
inline float sharp_kernel(float r2, float h) {
  float hh = h * h;
  return (float)std::fmax((double)hh / std::fmax((double)r2, 1.0e-5) - 1.0,
                          0.0);
}

/* hypot2 / length2 / length (src/utility.cpp:16-26). */
inline float hypot2(float a, float b, float c) { return a * a + b * b + c * c; }
inline float length2(const float *p0, const float *p1) {
  return hypot2(p0[0] - p1[0], p0[1] - p1[1], p0[2] - p1[2]);
}
inline float length(const float *p0, const float *p1) {
  return hypotf(hypotf(p0[0] - p1[0], p0[1] - p1[1]), p0[2] - p1[2]);
}

/* int i = fmax(0, fmin(gn-1, gn*p)) (src/sorter.cpp:35-37 and every query
 * that uses the same clamp: src/flip3D.cpp:177, src/corrector.cpp:36,
 * src/implicit.cpp:30). */
inline int cell_clamp(float p, int gn) {
  float s = (float)gn * p;
  return (int)std::fmax(0.0, std::fmin((double)(gn - 1), (double)s));
}

/* int i = fmin(N-1, fmax(0, p*N)) (src/flip3D.cpp:903-905, 944). */
inline int cell_clamp_minmax(float p, int gn) {
  float s = p * (float)gn;
  return (int)std::fmin((double)(gn - 1), std::fmax(0.0, (double)s));
}

/* FLOAT x = max(0, min(cs, cs*p)) with the macros of src/utility.h:16-17
 * (src/corrector.cpp:59-61), then truncated by the int parameter. */
inline int cell_clamp_macro(float p, int cs) {
  float v = (float)cs * p;
  float mn = ((float)cs > v) ? v : (float)cs; /* min(cs, v) */
  float mx = (0.0f > mn) ? 0.0f : mn;         /* max(0, mn) */
  return (int)mx;
}

struct Cells {
  int gn;
  const uint32_t *cs;
  const uint32_t *perm;
  /* Visit the particles of cells [i0,i1]x[j0,j1]x[k0,k1] in the order of
   * sorter::getNeigboringParticles_* (src/sorter.cpp:42-64): si, sj, sk
   * loops, out-of-range cells skipped, each cell in particle order. */
  template <class F>
  inline void visit(int i0, int i1, int j0, int j1, int k0, int k1, F f) const {
    for (int si = i0; si <= i1; si++)
      for (int sj = j0; sj <= j1; sj++)
        for (int sk = k0; sk <= k1; sk++) {
          if (si < 0 || si > gn - 1 || sj < 0 || sj > gn - 1 || sk < 0 ||
              sk > gn - 1)
            continue;
          size_t c = ((size_t)si * gn + sj) * gn + sk;
          for (uint32_t a = cs[c]; a < cs[c + 1]; a++) f(perm[a]);
        }
  }
};

inline size_t cidx(int n, int i, int j, int k) {
  return ((size_t)i * n + j) * n + k;
}
/* Face grids: u0 (n+1,n,n), u1 (n,n+1,n), u2 (n,n,n+1). */
inline size_t fidx(int ni, int nj, int nk, int i, int j, int k) {
  (void)ni;
  return ((size_t)i * nj + j) * nk + k;
}

/* linear() (src/mapper.cpp:96-106): trilinear sample of q with extents
 * (w,h,d). The k clamp uses h-2 as the reference does. */
inline float linear(const float *q, float x, float y, float z, int w, int h,
                    int d) {
  x = (float)std::fmax(0.0, std::fmin((double)w, (double)x));
  y = (float)std::fmax(0.0, std::fmin((double)h, (double)y));
  z = (float)std::fmax(0.0, std::fmin((double)d, (double)z));
  int i = (int)((x > (float)(w - 2)) ? (float)(w - 2) : x);
  int j = (int)((y > (float)(h - 2)) ? (float)(h - 2) : y);
  int k = (int)((z > (float)(h - 2)) ? (float)(h - 2) : z);
  /* For the v grid (h = n+1, d = n) k+1 can reach d; the reference then
   * reads one element past the row (undefined). Both implementations here
   * read the row's last element instead. */
  auto Q = [&](int a, int b, int c) -> float {
    if (c > d - 1) c = d - 1;
    return q[((size_t)a * h + b) * d + c];
  };
  float fx0 = (float)(i + 1) - x, fx1 = x - (float)i;
  float fy0 = (float)(j + 1) - y, fy1 = y - (float)j;
  float fz0 = (float)(k + 1) - z, fz1 = z - (float)k;
  return fz0 * ((fx0 * Q(i, j, k) + fx1 * Q(i + 1, j, k)) * fy0 +
                (fx0 * Q(i, j + 1, k) + fx1 * Q(i + 1, j + 1, k)) * fy1) +
         fz1 * ((fx0 * Q(i, j, k + 1) + fx1 * Q(i + 1, j, k + 1)) * fy0 +
                (fx0 * Q(i, j + 1, k + 1) + fx1 * Q(i + 1, j + 1, k + 1)) * fy1);
}

/* mapper::fetchVelocity (src/mapper.cpp:108-112). */
inline void fetch_velocity(int gn, const float *u0, const float *u1,
                           const float *u2, const float *p, float *u) {
  float gx = (float)gn * p[0], gy = (float)gn * p[1], gz = (float)gn * p[2];
  u[0] = linear(u0, gx, (float)((double)gy - 0.5), (float)((double)gz - 0.5),
                gn + 1, gn, gn);
  u[1] = linear(u1, (float)((double)gx - 0.5), gy, (float)((double)gz - 0.5),
                gn, gn + 1, gn);
  u[2] = linear(u2, (float)((double)gx - 0.5), (float)((double)gy - 0.5), gz,
                gn, gn, gn + 1);
}

} // namespace

/* ================================================================ sorter */

extern "C" void orc_sort(int n, int np, const float *pos, uint32_t *cell_start,
                         uint32_t *perm) {
  const size_t nc = (size_t)n * n * n;
  std::vector<uint32_t> key(np);
  std::memset(cell_start, 0, (nc + 1) * sizeof(uint32_t));
  for (int p = 0; p < np; p++) {
    int i = cell_clamp(pos[3 * p + 0], n);
    int j = cell_clamp(pos[3 * p + 1], n);
    int k = cell_clamp(pos[3 * p + 2], n);
    key[p] = (uint32_t)cidx(n, i, j, k);
    cell_start[key[p] + 1]++;
  }
  for (size_t c = 0; c < nc; c++) cell_start[c + 1] += cell_start[c];
  std::vector<uint32_t> fill(cell_start, cell_start + nc);
  for (int p = 0; p < np; p++) perm[fill[key[p]]++] = (uint32_t)p;
}

/* ========================================================== density/levelset */

extern "C" void orc_density(int n, int np, const float *pos,
                            const uint8_t *type, const uint32_t *cs,
                            const uint32_t *perm, float kernel_h,
                            float max_dens, float *dens) {
  Cells cells{n, cs, perm};
#pragma omp parallel for schedule(dynamic, 1024)
  for (int p = 0; p < np; p++) {
    if (type[p] == ORC_WALL) {
      dens[p] = 1.0f;
      continue;
    }
    const float *pp = pos + 3 * p;
    int ci = cell_clamp(pp[0], n), cj = cell_clamp(pp[1], n),
        ck = cell_clamp(pp[2], n);
    float wsum = 0.0f;
    cells.visit(ci - 1, ci + 1, cj - 1, cj + 1, ck - 1, ck + 1,
                [&](uint32_t q) {
                  if (type[q] == ORC_WALL) return;
                  float d2 = length2(pos + 3 * q, pp);
                  float w = 1.0f * smooth_kernel(d2, kernel_h);
                  wsum += w;
                });
    dens[p] = wsum / max_dens;
  }
}

namespace {
/* sorter::levelset (src/sorter.cpp:70-81). */
inline float levelset_cell(const Cells &cells, size_t c, const uint8_t *type,
                           const float *dens, float density) {
  float accm = 0.0f;
  for (uint32_t a = cells.cs[c]; a < cells.cs[c + 1]; a++) {
    uint32_t q = cells.perm[a];
    if (type[q] == ORC_FLUID)
      accm += dens[q];
    else
      return 1.0f;
  }
  float n0 = (float)(1.0 / (double)(density * density * density));
  return (float)(0.2 * (double)n0 - (double)accm);
}
} // namespace

extern "C" void orc_levelset(int n, const uint8_t *type, const float *dens,
                             const uint32_t *cs, const uint32_t *perm,
                             float density, float *L) {
  Cells cells{n, cs, perm};
  const size_t nc = (size_t)n * n * n;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nc; c++)
    L[c] = levelset_cell(cells, (size_t)c, type, dens, density);
}

extern "C" void orc_mark_water(int n, const uint8_t *type, const float *dens,
                               const uint32_t *cs, const uint32_t *perm,
                               float density, uint8_t *A) {
  Cells cells{n, cs, perm};
  const size_t nc = (size_t)n * n * n;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < (long)nc; c++) {
    uint8_t a = ORC_AIR;
    for (uint32_t s = cs[c]; s < cs[c + 1]; s++)
      if (type[perm[s]] == ORC_WALL) a = ORC_WALL;
    if (a != ORC_WALL)
      a = levelset_cell(cells, (size_t)c, type, dens, density) < 0.0f
              ? ORC_FLUID
              : ORC_AIR;
    A[c] = a;
  }
}

/* ================================================================ mapper */

extern "C" void orc_p2g(int n, int np, const float *pos, const float *vel,
                        const uint8_t *type, const uint32_t *cs,
                        const uint32_t *perm, float *u0, float *u1,
                        float *u2) {
  (void)np;
  Cells cells{n, cs, perm};
  const int gn = n;
  const float RE = (float)1.4; /* src/mapper.cpp:14 */
  auto clamp_pos = [&](const float *p, float *out) {
    for (int c = 0; c < 3; c++) {
      float s = (float)gn * p[c];
      out[c] = (float)std::fmax(0.0, std::fmin((double)gn, (double)s));
    }
  };
  /* One face: the weighted average of component `comp` over the fluid
   * particles of the given cell box (src/mapper.cpp:22-39). */
  auto face = [&](const float *fp, int comp, int i0, int i1, int j0, int j1,
                  int k0, int k1) -> float {
    float sumw = 0.0f, sumx = 0.0f;
    cells.visit(i0, i1, j0, j1, k0, k1, [&](uint32_t q) {
      if (type[q] != ORC_FLUID) return;
      float pq[3];
      clamp_pos(pos + 3 * q, pq);
      float w = 1.0f * sharp_kernel(length2(pq, fp), RE);
      sumx += w * vel[3 * q + comp];
      sumw += w;
    });
    return (sumw != 0.0f) ? sumx / sumw : 0.0f;
  };
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < gn + 1; i++)
    for (int j = 0; j < gn + 1; j++)
      for (int k = 0; k < gn + 1; k++) {
        if (j < gn && k < gn) {
          float px[3] = {(float)i, (float)(j + 0.5), (float)(k + 0.5)};
          u0[fidx(gn + 1, gn, gn, i, j, k)] =
              face(px, 0, i - 1, i, j - 2, j + 1, k - 2, k + 1);
        }
        if (i < gn && k < gn) {
          float py[3] = {(float)(i + 0.5), (float)j, (float)(k + 0.5)};
          u1[fidx(gn, gn + 1, gn, i, j, k)] =
              face(py, 1, i - 2, i + 1, j - 1, j, k - 2, k + 1);
        }
        if (i < gn && j < gn) {
          float pz[3] = {(float)(i + 0.5), (float)(j + 0.5), (float)k};
          u2[fidx(gn, gn, gn + 1, i, j, k)] =
              face(pz, 2, i - 2, i + 1, j - 2, j + 1, k - 1, k);
        }
      }
}

extern "C" void orc_g2p(int n, int np, const float *pos, const uint8_t *type,
                        const float *u0, const float *u1, const float *u2,
                        float *vel, int fluid_only) {
#pragma omp parallel for schedule(static)
  for (int p = 0; p < np; p++) {
    if (fluid_only && type[p] != ORC_FLUID) continue;
    fetch_velocity(n, u0, u1, u2, pos + 3 * p, vel + 3 * p);
  }
}

/* ============================================================ grid stages */

static inline float wall_chk(uint8_t a) { return a == ORC_WALL ? 1.0f : -1.0f; }

/* enforce_boundary (src/flip3D.cpp:783-805). */
extern "C" void orc_enforce_boundary(int n, const uint8_t *A, float *u0,
                                     float *u1, float *u2) {
  const int N = n;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N + 1; i++)
    for (int j = 0; j < N + 1; j++)
      for (int k = 0; k < N + 1; k++) {
        if (j < N && k < N) {
          float &u = u0[fidx(N + 1, N, N, i, j, k)];
          if (i == 0 || i == N) u = 0.0f;
          if (i < N && i > 0 &&
              wall_chk(A[cidx(N, i, j, k)]) * wall_chk(A[cidx(N, i - 1, j, k)]) < 0)
            u = 0.0f;
        }
        if (i < N && k < N) {
          float &u = u1[fidx(N, N + 1, N, i, j, k)];
          if (j == 0 || j == N) u = 0.0f;
          if (j < N && j > 0 &&
              wall_chk(A[cidx(N, i, j, k)]) * wall_chk(A[cidx(N, i, j - 1, k)]) < 0)
            u = 0.0f;
        }
        if (i < N && j < N) {
          float &u = u2[fidx(N, N, N + 1, i, j, k)];
          if (k == 0 || k == N) u = 0.0f;
          if (k < N && k > 0 &&
              wall_chk(A[cidx(N, i, j, k)]) * wall_chk(A[cidx(N, i, j, k - 1)]) < 0)
            u = 0.0f;
        }
      }
}

/* Divergence of FLUID cells (src/flip3D.cpp:814-821); other cells keep their
 * previous contents, as the reference's static array does. */
extern "C" void orc_divergence(int n, const uint8_t *A, const float *u0,
                               const float *u1, const float *u2, float *div) {
  const int N = n;
  const float h = (float)(1.0 / N);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      for (int k = 0; k < N; k++) {
        if (A[cidx(N, i, j, k)] != ORC_FLUID) continue;
        float d = u0[fidx(N + 1, N, N, i + 1, j, k)] - u0[fidx(N + 1, N, N, i, j, k)] +
                  u1[fidx(N, N + 1, N, i, j + 1, k)] - u1[fidx(N, N + 1, N, i, j, k)] +
                  u2[fidx(N, N, N + 1, i, j, k + 1)] - u2[fidx(N, N, N + 1, i, j, k)];
        div[cidx(N, i, j, k)] = d / h;
      }
}

/* Pressure-gradient subtraction with the subcell ghost values
 * (src/flip3D.cpp:832-867). */
extern "C" void orc_subtract_gradient(int n, int subcell, const float *L,
                                      const float *press, float *u0, float *u1,
                                      float *u2) {
  const int N = n;
  const float h = (float)(1.0 / N);
  auto grad = [&](size_t cf, size_t cb) -> float {
    float pf = press[cf];
    float pb = press[cb];
    if (subcell && L[cf] * L[cb] < 0.0f) {
      pf = L[cf] < 0.0f
               ? press[cf]
               : (float)((double)L[cf] / std::fmin(1.0e-3, (double)L[cb]) *
                         (double)press[cb]);
      pb = L[cb] < 0.0f
               ? press[cb]
               : (float)((double)L[cb] / std::fmin(1.0e-6, (double)L[cf]) *
                         (double)press[cf]);
    }
    return (pf - pb) / h;
  };
#pragma omp parallel for schedule(static)
  for (int i = 0; i < N + 1; i++)
    for (int j = 0; j < N + 1; j++)
      for (int k = 0; k < N + 1; k++) {
        if (j < N && k < N && i > 0 && i < N)
          u0[fidx(N + 1, N, N, i, j, k)] -= grad(cidx(N, i, j, k), cidx(N, i - 1, j, k));
        if (i < N && k < N && j > 0 && j < N)
          u1[fidx(N, N + 1, N, i, j, k)] -= grad(cidx(N, i, j, k), cidx(N, i, j - 1, k));
        if (i < N && j < N && k > 0 && k < N)
          u2[fidx(N, N, N + 1, i, j, k)] -= grad(cidx(N, i, j, k), cidx(N, i, j, k - 1));
      }
}

/* extrapolate_velocity (src/flip3D.cpp:1011-1054). */
extern "C" void orc_extrapolate(int n, const uint8_t *A, float *u0, float *u1,
                                float *u2) {
  const int N = n;
  float *u[3] = {u0, u1, u2};
  const int ext[3][3] = {{N + 1, N, N}, {N, N + 1, N}, {N, N, N + 1}};
  std::vector<uint8_t> mark[3], wall_mark[3];
  for (int c = 0; c < 3; c++) {
    size_t sz = (size_t)ext[c][0] * ext[c][1] * ext[c][2];
    mark[c].assign(sz, 0);
    wall_mark[c].assign(sz, 0);
  }
  auto Aat = [&](int i, int j, int k) { return A[cidx(N, i, j, k)]; };
  for (int c = 0; c < 3; c++) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ext[c][0]; i++)
      for (int j = 0; j < ext[c][1]; j++)
        for (int k = 0; k < ext[c][2]; k++) {
          int idx[3] = {i, j, k};
          int m[3] = {i, j, k};
          m[c] -= 1; /* the cell on the minus side of the face */
          int a = idx[c];
          bool minus_fluid = a > 0 && Aat(m[0], m[1], m[2]) == ORC_FLUID;
          bool plus_fluid = a < N && Aat(i, j, k) == ORC_FLUID;
          bool minus_wall = a <= 0 || Aat(m[0], m[1], m[2]) == ORC_WALL;
          bool plus_wall = a >= N || Aat(i, j, k) == ORC_WALL;
          size_t f = fidx(ext[c][0], ext[c][1], ext[c][2], i, j, k);
          mark[c][f] = minus_fluid || plus_fluid;
          wall_mark[c][f] = minus_wall && plus_wall;
        }
  }
  for (int c = 0; c < 3; c++) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ext[c][0]; i++)
      for (int j = 0; j < ext[c][1]; j++)
        for (int k = 0; k < ext[c][2]; k++) {
          size_t f = fidx(ext[c][0], ext[c][1], ext[c][2], i, j, k);
          if (mark[c][f] || !wall_mark[c][f]) continue;
          int wsum = 0;
          float sum = 0.0f;
          const int q[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                               {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
          for (int s = 0; s < 6; s++) {
            if (q[s][0] >= 0 && q[s][0] < ext[c][0] && q[s][1] >= 0 &&
                q[s][1] < ext[c][1] && q[s][2] >= 0 && q[s][2] < ext[c][2]) {
              size_t g = fidx(ext[c][0], ext[c][1], ext[c][2], q[s][0], q[s][1], q[s][2]);
              if (mark[c][g]) {
                wsum++;
                sum += u[c][g];
              }
            }
          }
          if (wsum) u[c][f] = sum / (float)wsum;
        }
  }
}

/* ================================================================ solver */

namespace {

struct Solver {
  int n;
  int subcell;
  const uint8_t *A;
  const float *L;

  size_t id(int i, int j, int k) const { return cidx(n, i, j, k); }
  bool in(int i, int j, int k) const {
    return i >= 0 && i <= n - 1 && j >= 0 && j <= n - 1 && k >= 0 && k <= n - 1;
  }

  /* x_ref (src/solver.cpp:19-26). */
  float x_ref(const float *x, int fi, int fj, int fk, int i, int j, int k) const {
    i = std::min(std::max(0, i), n - 1);
    j = std::min(std::max(0, j), n - 1);
    k = std::min(std::max(0, k), n - 1);
    uint8_t a = A[id(i, j, k)];
    if (a == ORC_FLUID) return x[id(i, j, k)];
    if (a == ORC_WALL) return x[id(fi, fj, fk)];
    return subcell ? (float)((double)L[id(i, j, k)] /
                             std::fmin(1.0e-6, (double)L[id(fi, fj, fk)]) *
                             (double)x[id(fi, fj, fk)])
                   : 0.0f;
  }

  /* compute_Ax (src/solver.cpp:29-41). */
  void matvec(const float *x, float *ans) const {
    const float h2 = (float)(1.0 / (n * n));
    const long nc = (long)n * n * n;
#pragma omp parallel for schedule(static)
    for (long g = 0; g < nc; g++) {
      int i = (int)((g % ((long)n * n)) % n), j = (int)((g % ((long)n * n)) / n),
          k = (int)(g / ((long)n * n));
      size_t c = id(i, j, k);
      if (A[c] == ORC_FLUID) {
        double v = 6.0 * (double)x[c];
        v -= x_ref(x, i, j, k, i + 1, j, k);
        v -= x_ref(x, i, j, k, i - 1, j, k);
        v -= x_ref(x, i, j, k, i, j + 1, k);
        v -= x_ref(x, i, j, k, i, j - 1, k);
        v -= x_ref(x, i, j, k, i, j, k + 1);
        v -= x_ref(x, i, j, k, i, j, k - 1);
        ans[c] = (float)(v / (double)h2);
      } else {
        ans[c] = 0.0f;
      }
    }
  }

  /* product (src/solver.cpp:44-54): sequential double sum of float products
   * in FOR_EVERY_COMP order (i fastest). */
  double product(const float *x, const float *y) const {
    double ans = 0.0;
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          size_t c = id(i, j, k);
          if (A[c] == ORC_FLUID) ans += (double)(x[c] * y[c]);
        }
    return ans;
  }

  /* op (src/solver.cpp:78-85): ans = x + a*y on FLUID, 0 elsewhere. */
  void op(const float *x, const float *y, float *ans, float a) const {
    const long nc = (long)n * n * n;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; c++)
      ans[c] = (A[c] == ORC_FLUID) ? x[c] + a * y[c] : 0.0f;
  }

  /* A_ref (src/solver.cpp:97-101). */
  float A_ref(int i, int j, int k, int qi, int qj, int qk) const {
    if (!in(i, j, k) || A[id(i, j, k)] != ORC_FLUID) return 0.0f;
    if (!in(qi, qj, qk) || A[id(qi, qj, qk)] != ORC_FLUID) return 0.0f;
    return -1.0f;
  }

  /* A_diag (src/solver.cpp:103-117). */
  float A_diag(int i, int j, int k) const {
    float diag = 6.0f;
    if (A[id(i, j, k)] != ORC_FLUID) return diag;
    const int q[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                         {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
    for (int m = 0; m < 6; m++) {
      int qi = q[m][0], qj = q[m][1], qk = q[m][2];
      if (!in(qi, qj, qk) || A[id(qi, qj, qk)] == ORC_WALL)
        diag = (float)((double)diag - 1.0);
      else if (A[id(qi, qj, qk)] == ORC_AIR && subcell)
        diag = (float)((double)diag -
                       (double)L[id(qi, qj, qk)] /
                           std::fmin(1.0e-6, (double)L[id(i, j, k)]));
    }
    return diag;
  }

  /* P_ref as written (src/solver.cpp:119-123): the value itself is compared
   * with FLUID (1), so only entries equal to 1.0 pass. */
  template <class T> float P_ref_value(const T *P, int i, int j, int k) const {
    if (!in(i, j, k) || (double)P[id(i, j, k)] != (double)ORC_FLUID) return 0.0f;
    return (float)P[id(i, j, k)];
  }
  /* The corrected test on the cell flag. */
  template <class T> double P_ref_flag(const T *P, int i, int j, int k) const {
    if (!in(i, j, k) || A[id(i, j, k)] != ORC_FLUID) return 0.0;
    return (double)P[id(i, j, k)];
  }

  /* buildPreconditioner (src/solver.cpp:125-139) as written. */
  void build_ref(std::vector<double> &P) const {
    std::fill(P.begin(), P.end(), 0.0);
    const double a = 0.25;
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          if (A[id(i, j, k)] != ORC_FLUID) continue;
          double left = (double)(A_ref(i - 1, j, k, i, j, k) * P_ref_value(P.data(), i - 1, j, k));
          double bottom = (double)(A_ref(i, j - 1, k, i, j, k) * P_ref_value(P.data(), i, j - 1, k));
          double back = (double)(A_ref(i, j, k - 1, i, j, k) * P_ref_value(P.data(), i, j, k - 1));
          double diag = (double)A_diag(i, j, k);
          float sl = (float)left, sb = (float)bottom, sk = (float)back;
          double e = diag - (double)(sl * sl) - (double)(sb * sb) - (double)(sk * sk);
          if (e < a * diag) e = diag;
          P[id(i, j, k)] = 1.0 / (double)sqrtf((float)e);
        }
  }

  /* applyPreconditioner (src/solver.cpp:141-180) as written. */
  void apply_ref(const std::vector<double> &P, const float *r, float *z,
                 std::vector<double> &q) const {
    std::fill(q.begin(), q.end(), 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
          if (A[id(i, j, k)] != ORC_FLUID) continue;
          double left = (double)(A_ref(i - 1, j, k, i, j, k) * P_ref_value(P.data(), i - 1, j, k) * P_ref_value(q.data(), i - 1, j, k));
          double bottom = (double)(A_ref(i, j - 1, k, i, j, k) * P_ref_value(P.data(), i, j - 1, k) * P_ref_value(q.data(), i, j - 1, k));
          double back = (double)(A_ref(i, j, k - 1, i, j, k) * P_ref_value(P.data(), i, j, k - 1) * P_ref_value(q.data(), i, j, k - 1));
          double t = (double)r[id(i, j, k)] - left - bottom - back;
          q[id(i, j, k)] = t * P[id(i, j, k)];
        }
    for (int i = n - 1; i >= 0; i--)
      for (int j = n - 1; j >= 0; j--)
        for (int k = n - 1; k >= 0; k--) {
          if (A[id(i, j, k)] != ORC_FLUID) continue;
          double right = (double)(A_ref(i, j, k, i + 1, j, k) * P_ref_value(P.data(), i, j, k) * P_ref_value(z, i + 1, j, k));
          double top = (double)(A_ref(i, j, k, i, j + 1, k) * P_ref_value(P.data(), i, j, k) * P_ref_value(z, i, j + 1, k));
          double front = (double)(A_ref(i, j, k, i, j, k + 1) * P_ref_value(P.data(), i, j, k) * P_ref_value(z, i, j, k + 1));
          double t = q[id(i, j, k)] - right - top - front;
          z[id(i, j, k)] = (float)(t * P[id(i, j, k)]);
        }
  }

  /* IC(0) / MIC(0) factor in double with the neighbour test on the cell
   * flag: the reference's formula (src/solver.cpp:125-139) with P_ref
   * corrected, plus the standard MIC(0) modification weighted by tau. */
  void build_ic(std::vector<double> &P, double tau) const {
    std::fill(P.begin(), P.end(), 0.0);
    auto fl = [&](int i, int j, int k) { return in(i, j, k) && A[id(i, j, k)] == ORC_FLUID; };
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          if (!fl(i, j, k)) continue;
          double diag = (double)A_diag(i, j, k);
          double e = diag;
          /* neighbour m on the minus side of each axis */
          const int nb[3][3] = {{i - 1, j, k}, {i, j - 1, k}, {i, j, k - 1}};
          for (int ax = 0; ax < 3; ax++) {
            int a = nb[ax][0], b = nb[ax][1], c = nb[ax][2];
            if (!fl(a, b, c)) continue;
            double pm = P[id(a, b, c)];
            e -= pm * pm; /* (A_{c,m} P_m)^2 with A_{c,m} = -1 */
            if (tau != 0.0) {
              /* the other two plus-side couplings of m */
              double other = 0.0;
              const int pl[3][3] = {{a + 1, b, c}, {a, b + 1, c}, {a, b, c + 1}};
              for (int ax2 = 0; ax2 < 3; ax2++) {
                if (ax2 == ax) continue;
                if (fl(a, b, c) && fl(pl[ax2][0], pl[ax2][1], pl[ax2][2])) other += -1.0;
              }
              e -= tau * (-1.0) * other * pm * pm;
            }
          }
          if (e < 0.25 * diag) e = diag;
          P[id(i, j, k)] = 1.0 / std::sqrt(e);
        }
  }

  void apply_ic(const std::vector<double> &P, const float *r, float *z,
                std::vector<double> &q) const {
    std::fill(q.begin(), q.end(), 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
          if (A[id(i, j, k)] != ORC_FLUID) continue;
          double t = (double)r[id(i, j, k)];
          t += P_ref_flag(P.data(), i - 1, j, k) * P_ref_flag(q.data(), i - 1, j, k);
          t += P_ref_flag(P.data(), i, j - 1, k) * P_ref_flag(q.data(), i, j - 1, k);
          t += P_ref_flag(P.data(), i, j, k - 1) * P_ref_flag(q.data(), i, j, k - 1);
          q[id(i, j, k)] = t * P[id(i, j, k)];
        }
    std::vector<double> zz(q.size(), 0.0);
    for (int i = n - 1; i >= 0; i--)
      for (int j = n - 1; j >= 0; j--)
        for (int k = n - 1; k >= 0; k--) {
          if (A[id(i, j, k)] != ORC_FLUID) continue;
          double pc = P[id(i, j, k)];
          double t = q[id(i, j, k)];
          t += pc * P_ref_flag(zz.data(), i + 1, j, k);
          t += pc * P_ref_flag(zz.data(), i, j + 1, k);
          t += pc * P_ref_flag(zz.data(), i, j, k + 1);
          zz[id(i, j, k)] = t * pc;
        }
    for (size_t c = 0; c < zz.size(); c++)
      if (A[c] == ORC_FLUID) z[c] = (float)zz[c];
  }
};

/* The reference eps is 1e-2*n^3 on float(r.r). A relative tolerance is
 * expressed by dividing it by 4^k, the exact analogue of running the
 * reference on inputs scaled by 2^k. */
double effective_eps(const OrcParams *prm, double b2) {
  const int n = prm->n;
  double eps = 1.0e-2 * ((double)n * n * n);
  if (prm->eps_abs >= 0.0) return prm->eps_abs;
  if (prm->rel_tol > 0.0) {
    double target = prm->rel_tol * prm->rel_tol * b2;
    while (eps > target && eps > 0.0) eps *= 0.25;
  }
  return eps;
}

} // namespace

extern "C" void orc_matvec(int n, int subcell, const uint8_t *A,
                           const float *L, const float *x, float *ans) {
  Solver s{n, subcell, A, L};
  s.matvec(x, ans);
}

extern "C" void orc_precond_apply(const OrcParams *prm, const uint8_t *A,
                                  const float *L, const float *r, float *z) {
  const int n = prm->n;
  Solver s{n, prm->subcell, A, L};
  const size_t nc = (size_t)n * n * n;
  std::vector<double> P(nc), q(nc);
  if (prm->precond == ORC_PRECOND_REF) {
    s.build_ref(P);
    s.apply_ref(P, r, z, q);
  } else if (prm->precond == ORC_PRECOND_IC) {
    s.build_ic(P, prm->mic_tau);
    s.apply_ic(P, r, z, q);
  } else {
    std::memcpy(z, r, nc * sizeof(float));
  }
}

/* solver::solve + conjGrad (src/solver.cpp:183-241). */
extern "C" int orc_solve(const OrcParams *prm, const uint8_t *A,
                         const float *L, float *x, float *b, double *final_r2,
                         double *b2_out) {
  const int n = prm->n;
  const size_t nc = (size_t)n * n * n;
  Solver s{n, prm->subcell, A, L};
  for (size_t c = 0; c < nc; c++) b[c] = -b[c]; /* flip (src/solver.cpp:76-80) */
  std::vector<double> P(nc), q(nc);
  if (prm->precond == ORC_PRECOND_REF) s.build_ref(P);
  if (prm->precond == ORC_PRECOND_IC) s.build_ic(P, prm->mic_tau);
  auto precond = [&](const float *r, float *z) {
    if (prm->precond == ORC_PRECOND_REF)
      s.apply_ref(P, r, z, q);
    else if (prm->precond == ORC_PRECOND_IC)
      s.apply_ic(P, r, z, q);
    else
      std::memcpy(z, r, nc * sizeof(float));
  };
  std::vector<float> r(nc), z(nc), sv(nc);
  double b2 = s.product(b, b);
  if (b2_out) *b2_out = b2;
  s.matvec(x, z.data());
  s.op(b, z.data(), r.data(), -1.0f);
  double error2_0 = s.product(r.data(), r.data());
  precond(r.data(), z.data());
  sv = z;
  const double eps = effective_eps(prm, b2);
  double a = s.product(z.data(), r.data());
  const long max_it = prm->max_iters > 0 ? prm->max_iters : (long)nc;
  int iters = 0;
  float error2 = (float)error2_0;
  for (long k = 0; k < max_it; k++) {
    s.matvec(sv.data(), z.data());
    double alpha = a / s.product(z.data(), sv.data());
    s.op(x, sv.data(), x, (float)alpha);
    s.op(r.data(), z.data(), r.data(), (float)(-alpha));
    error2 = (float)s.product(r.data(), r.data());
    error2_0 = std::fmax(error2_0, (double)error2);
    iters = (int)k + 1;
    if ((double)error2 <= eps) break;
    precond(r.data(), z.data());
    double a2 = s.product(z.data(), r.data());
    double beta = a2 / a;
    s.op(z.data(), sv.data(), sv.data(), (float)beta);
    a = a2;
  }
  if (final_r2) *final_r2 = (double)error2;
  return iters;
}

/* ============================================================= corrector */

namespace {
const double SPRING = 50.0; /* src/corrector.cpp:13 */

void resample_at(const Cells &cells, const float *pos, const float *vel,
                 const uint8_t *type, const float *p, float *u, float re) {
  const int cs = cells.gn;
  float wsum = 0.0f;
  float save[3] = {u[0], u[1], u[2]};
  u[0] = u[1] = u[2] = 0.0f;
  int ci = cell_clamp(p[0], cs), cj = cell_clamp(p[1], cs), ck = cell_clamp(p[2], cs);
  cells.visit(ci - 1, ci + 1, cj - 1, cj + 1, ck - 1, ck + 1, [&](uint32_t q) {
    if (type[q] != ORC_FLUID) return;
    float dist2 = length2(p, pos + 3 * q);
    float w = 1.0f * sharp_kernel(dist2, re);
    u[0] += w * vel[3 * q + 0];
    u[1] += w * vel[3 * q + 1];
    u[2] += w * vel[3 * q + 2];
    wsum += w;
  });
  if (wsum != 0.0f) {
    u[0] /= wsum;
    u[1] /= wsum;
    u[2] /= wsum;
  } else {
    u[0] = save[0];
    u[1] = save[1];
    u[2] = save[2];
  }
}
} // namespace

extern "C" void orc_resample(int n, const float *pos, const float *vel,
                             const uint8_t *type, const uint32_t *cs,
                             const uint32_t *perm, const float p[3],
                             float u[3], float re) {
  Cells cells{n, cs, perm};
  resample_at(cells, pos, vel, type, p, u, re);
}

extern "C" void orc_correct(int n, int np, float *pos, float *vel,
                            const uint8_t *type, const float *nrm,
                            const uint32_t *cs, const uint32_t *perm, float dt,
                            float re, uint64_t seed, int64_t step) {
  Cells cells{n, cs, perm};
  const int csz = n;
  std::vector<float> tmp0((size_t)np * 3), tmp1((size_t)np * 3);
  /* Compute pseudo moved point (src/corrector.cpp:54-89). */
#pragma omp parallel for schedule(dynamic, 1024)
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    const float *pp = pos + 3 * p;
    float spring[3] = {0.0f, 0.0f, 0.0f};
    int x = cell_clamp_macro(pp[0], csz), y = cell_clamp_macro(pp[1], csz),
        z = cell_clamp_macro(pp[2], csz);
    cells.visit(x - 1, x + 1, y - 1, y + 1, z - 1, z + 1, [&](uint32_t q) {
      if ((int)q == p) return;
      const float *pq = pos + 3 * q;
      float dist = length(pp, pq);
      float w = (float)(SPRING * 1.0 * (double)smooth_kernel(dist * dist, re));
      if ((double)dist > 0.1 * (double)re) {
        spring[0] += w * (pp[0] - pq[0]) / dist * re;
        spring[1] += w * (pp[1] - pq[1]) / dist * re;
        spring[2] += w * (pp[2] - pq[2]) / dist * re;
      } else if (type[q] == ORC_FLUID) {
        for (int c = 0; c < 3; c++) {
          uint32_t rr = flip_rand31(seed, flip_stream(FLIP_RNG_KICK, (uint64_t)step, c),
                                    (uint64_t)p, (uint64_t)q);
          spring[c] = (float)((double)spring[c] +
                              0.01 * (double)re / (double)dt * (double)(int)(rr % 101) / 100.0);
        }
      } else {
        for (int c = 0; c < 3; c++)
          spring[c] = (float)((double)spring[c] +
                              0.05 * (double)re / (double)dt * (double)nrm[3 * q + c]);
      }
    });
    for (int c = 0; c < 3; c++) tmp0[3 * p + c] = pp[c] + dt * spring[c];
  }
  /* Resample new velocity (src/corrector.cpp:91-101). */
#pragma omp parallel for schedule(dynamic, 1024)
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    for (int c = 0; c < 3; c++) tmp1[3 * p + c] = vel[3 * p + c];
    resample_at(cells, pos, vel, type, &tmp0[3 * p], &tmp1[3 * p], re);
  }
  /* Update (src/corrector.cpp:103-114). */
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    for (int c = 0; c < 3; c++) {
      pos[3 * p + c] = tmp0[3 * p + c];
      vel[3 * p + c] = tmp1[3 * p + c];
    }
  }
}

/* ============================================================ simulation */

struct OrcSim {
  OrcParams prm;
  int np;
  float max_dens;
  int64_t step;
  std::vector<float> pos, vel, nrm, dens;
  std::vector<uint8_t> type;
  std::vector<uint32_t> cs, perm;
  std::vector<float> u[3], u_save[3];
  std::vector<uint8_t> A;
  std::vector<float> L, press, div;
  int last_stuck;
  int last_iters;
  double last_r2;
};

namespace {

void sim_sort(OrcSim *s) {
  orc_sort(s->prm.n, s->np, s->pos.data(), s->cs.data(), s->perm.data());
}

/* reposition (src/flip3D.cpp:405-451) with the counter-based generator. */
void sim_reposition(OrcSim *s, const std::vector<int> &indices) {
  if (indices.empty()) return;
  const int gn = s->prm.n, N = gn;
  const uint8_t *A = s->A.data();
  struct IPos { int i, j, k; };
  std::vector<IPos> waters;
  while (waters.size() < indices.size()) {
    bool done = false;
    for (int i = 0; i < gn && !done; i++)
      for (int j = 0; j < gn && !done; j++)
        for (int k = 0; k < gn && !done; k++) {
          if (i > 0 && A[cidx(N, i - 1, j, k)] != ORC_FLUID) continue;
          if (i < N - 1 && A[cidx(N, i + 1, j, k)] != ORC_FLUID) continue;
          if (j > 0 && A[cidx(N, i, j - 1, k)] != ORC_FLUID) continue;
          if (j < N - 1 && A[cidx(N, i, j + 1, k)] != ORC_FLUID) continue;
          if (k > 0 && A[cidx(N, i, j, k - 1)] != ORC_FLUID) continue;
          if (k < N - 1 && A[cidx(N, i, j, k + 1)] != ORC_FLUID) continue;
          if (A[cidx(N, i, j, k)] != ORC_FLUID) continue;
          waters.push_back({i, j, k});
          if (waters.size() >= indices.size()) done = true;
        }
    if (waters.empty()) return;
  }
  /* my_rand_shuffle (src/utility.cpp:28-30): Fisher-Yates with keyed draws. */
  for (size_t i = waters.size() - 1; i >= 1; i--) {
    uint32_t r = flip_rand31(s->prm.seed, flip_stream(FLIP_RNG_SHUFFLE, (uint64_t)s->step, 0),
                             (uint64_t)i, 0);
    size_t j = r % (uint32_t)(i + 1);
    std::swap(waters[i], waters[j]);
  }
  const float h = (float)(1.0 / gn);
  for (size_t m = 0; m < indices.size(); m++) {
    float *p = &s->pos[3 * (size_t)indices[m]];
    const int cell[3] = {waters[m].i, waters[m].j, waters[m].k};
    for (int c = 0; c < 3; c++) {
      uint32_t r = flip_rand31(s->prm.seed, flip_stream(FLIP_RNG_PLACE, (uint64_t)s->step, 0),
                               (uint64_t)(3 * m + c), 0);
      double frac = 0.5 * (double)(int)(r % 101) / 100;
      p[c] = (float)((double)h * ((double)cell[c] + 0.25 + frac));
    }
  }
  sim_sort(s);
  Cells cells{gn, s->cs.data(), s->perm.data()};
  for (size_t m = 0; m < indices.size(); m++) {
    size_t q = (size_t)indices[m];
    float u[3] = {0.0f, 0.0f, 0.0f};
    resample_at(cells, s->pos.data(), s->vel.data(), s->type.data(), &s->pos[3 * q], u, h);
    for (int c = 0; c < 3; c++) s->vel[3 * q + c] = u[c];
  }
}

/* advect_particle (src/flip3D.cpp:877-969). */
void sim_advect(OrcSim *s) {
  const int N = s->prm.n;
  const int np = s->np;
  float *pos = s->pos.data();
  float *vel = s->vel.data();
  const uint8_t *type = s->type.data();
  const double DT = s->prm.dt;
#pragma omp parallel for schedule(static)
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    float v[3];
    fetch_velocity(N, s->u[0].data(), s->u[1].data(), s->u[2].data(), pos + 3 * p, v);
    for (int c = 0; c < 3; c++) pos[3 * p + c] = (float)((double)pos[3 * p + c] + DT * (double)v[c]);
  }
  sim_sort(s);
  Cells cells{N, s->cs.data(), s->perm.data()};
  const float r = (float)(1.0 / N);
  const double re = 1.5 * (double)s->prm.density / N;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    float *pp = pos + 3 * p;
    for (int c = 0; c < 3; c++)
      pp[c] = (float)std::fmax((double)r, std::fmin(1.0 - (double)r, (double)pp[c]));
    int i = cell_clamp_minmax(pp[0], N), j = cell_clamp_minmax(pp[1], N),
        k = cell_clamp_minmax(pp[2], N);
    float *uu = vel + 3 * p;
    cells.visit(i - 1, i + 1, j - 1, j + 1, k - 1, k + 1, [&](uint32_t q) {
      if (type[q] != ORC_WALL) return;
      const float *pq = pos + 3 * q;
      float dist = length(pp, pq);
      if ((double)dist < re) {
        float normal[3] = {s->nrm[3 * q], s->nrm[3 * q + 1], s->nrm[3 * q + 2]};
        if (normal[0] == 0.0f && normal[1] == 0.0f && normal[2] == 0.0f && dist != 0.0f)
          for (int c = 0; c < 3; c++) normal[c] = (pp[c] - pq[c]) / dist;
        for (int c = 0; c < 3; c++)
          pp[c] = (float)((double)pp[c] + (re - (double)dist) * (double)normal[c]);
        float dot = uu[0] * normal[0] + uu[1] * normal[1] + uu[2] * normal[2];
        for (int c = 0; c < 3; c++) uu[c] -= dot * normal[c];
      }
    });
  }
  /* Stuck particles (src/flip3D.cpp:933-966). */
  std::vector<int> indices;
  const uint8_t *A = s->A.data();
  for (int p = 0; p < np; p++) {
    if (type[p] != ORC_FLUID) continue;
    const float *pp = pos + 3 * p;
    bool remove = false;
    if (A[cidx(N, cell_clamp_minmax(pp[0], N), cell_clamp_minmax(pp[1], N),
               cell_clamp_minmax(pp[2], N))] == ORC_WALL)
      remove = true;
    int i = (int)std::fmin((double)(N - 3), std::fmax(2.0, (double)(pp[0] * (float)N)));
    int j = (int)std::fmin((double)(N - 3), std::fmax(2.0, (double)(pp[1] * (float)N)));
    int k = (int)std::fmin((double)(N - 3), std::fmax(2.0, (double)(pp[2] * (float)N)));
    if ((double)s->dens[p] < 0.04 &&
        (A[cidx(N, i, std::max(0, j - 1), k)] == ORC_WALL ||
         A[cidx(N, i, std::min(N - 1, j + 1), k)] == ORC_WALL))
      remove = true;
    if (remove) indices.push_back(p);
  }
  s->last_stuck = (int)indices.size();
  sim_reposition(s, indices);
}

/* The body of solve_picflip (src/flip3D.cpp:1057-1103) after its sort. */
void sim_picflip(OrcSim *s) {
  const int N = s->prm.n;
  const int np = s->np;
  float *u0 = s->u[0].data(), *u1 = s->u[1].data(), *u2 = s->u[2].data();
  orc_p2g(N, np, s->pos.data(), s->vel.data(), s->type.data(), s->cs.data(),
          s->perm.data(), u0, u1, u2);
  orc_mark_water(N, s->type.data(), s->dens.data(), s->cs.data(), s->perm.data(),
                 s->prm.density, s->A.data());
  for (int c = 0; c < 3; c++) s->u_save[c] = s->u[c];
  orc_enforce_boundary(N, s->A.data(), u0, u1, u2);
  /* project (src/flip3D.cpp:807-868) */
  orc_divergence(N, s->A.data(), u0, u1, u2, s->div.data());
  orc_levelset(N, s->type.data(), s->dens.data(), s->cs.data(), s->perm.data(),
               s->prm.density, s->L.data());
  s->last_iters = orc_solve(&s->prm, s->A.data(), s->L.data(), s->press.data(),
                            s->div.data(), &s->last_r2, nullptr);
  orc_subtract_gradient(N, s->prm.subcell, s->L.data(), s->press.data(), u0, u1, u2);
  orc_enforce_boundary(N, s->A.data(), u0, u1, u2);
  orc_extrapolate(N, s->A.data(), u0, u1, u2);
  for (int c = 0; c < 3; c++)
    for (size_t f = 0; f < s->u[c].size(); f++) s->u_save[c][f] = s->u[c][f] - s->u_save[c][f];
  /* FLIP blend (src/flip3D.cpp:1072-1097) */
  const double alpha = s->prm.alpha;
  float *vel = s->vel.data();
  const float *pos = s->pos.data();
#pragma omp parallel for schedule(static)
  for (int p = 0; p < np; p++) {
    float du[3], pic[3];
    fetch_velocity(N, s->u_save[0].data(), s->u_save[1].data(), s->u_save[2].data(), pos + 3 * p, du);
    fetch_velocity(N, u0, u1, u2, pos + 3 * p, pic);
    for (int c = 0; c < 3; c++) {
      float flipv = du[c] + vel[3 * p + c];
      vel[3 * p + c] = (float)((1.0 - alpha) * (double)pic[c] + alpha * (double)flipv);
    }
  }
}

} // namespace

extern "C" OrcSim *orc_sim_create(const OrcParams *prm, int np, const float *pos,
                                  const float *vel, const uint8_t *type,
                                  const float *nrm, float max_dens) {
  OrcSim *s = new OrcSim();
  s->prm = *prm;
  s->np = np;
  s->max_dens = max_dens;
  s->step = 0;
  s->pos.assign(pos, pos + 3 * (size_t)np);
  s->vel.assign(vel, vel + 3 * (size_t)np);
  s->nrm.assign(nrm, nrm + 3 * (size_t)np);
  s->type.assign(type, type + np);
  s->dens.assign(np, 0.0f);
  const int N = prm->n;
  const size_t nc = (size_t)N * N * N;
  s->cs.assign(nc + 1, 0);
  s->perm.assign(np, 0);
  const size_t fs = (size_t)(N + 1) * N * N;
  for (int c = 0; c < 3; c++) {
    s->u[c].assign(fs, 0.0f);
    s->u_save[c].assign(fs, 0.0f);
  }
  s->A.assign(nc, ORC_AIR);
  s->L.assign(nc, 0.0f);
  s->press.assign(nc, 0.0f);
  s->div.assign(nc, 0.0f);
  s->last_stuck = 0;
  s->last_iters = 0;
  s->last_r2 = 0.0;
  return s;
}

extern "C" void orc_sim_destroy(OrcSim *s) { delete s; }

/* Stages of simulateStep (src/flip3D.cpp:1194-1264):
 *   0 sort + computeDensity, 1 add_ExtForce, 2 solve_picflip,
 *   3 advect_particle, 4 corrector::correct. */
extern "C" void orc_sim_stage(OrcSim *s, int stage) {
  const int N = s->prm.n;
  switch (stage) {
  case 0:
    sim_sort(s);
    orc_density(N, s->np, s->pos.data(), s->type.data(), s->cs.data(), s->perm.data(),
                (float)(4.0 * (double)s->prm.density / N), s->max_dens, s->dens.data());
    break;
  case 1: {
    /* add_ExtForce (src/flip3D.cpp:870-875): every particle, walls too. */
    const double g = -s->prm.dt * s->prm.gravity;
    for (int p = 0; p < s->np; p++)
      s->vel[3 * p + 1] = (float)((double)s->vel[3 * p + 1] + g);
    break;
  }
  case 2:
    sim_picflip(s);
    break;
  case 3:
    sim_advect(s);
    break;
  case 4:
    sim_sort(s);
    orc_correct(N, s->np, s->pos.data(), s->vel.data(), s->type.data(), s->nrm.data(),
                s->cs.data(), s->perm.data(), (float)s->prm.dt,
                (float)((double)s->prm.density / N), s->prm.seed, s->step);
    break;
  default:
    break;
  }
}

extern "C" int orc_sim_step(OrcSim *s) {
  s->step++;
  for (int st = 0; st < 5; st++) orc_sim_stage(s, st);
  return s->last_iters;
}

extern "C" int orc_sim_count(const OrcSim *s) { return s->np; }

extern "C" void orc_sim_get(const OrcSim *s, float *pos, float *vel, float *dens,
                            uint8_t *type) {
  if (pos) std::memcpy(pos, s->pos.data(), s->pos.size() * sizeof(float));
  if (vel) std::memcpy(vel, s->vel.data(), s->vel.size() * sizeof(float));
  if (dens) std::memcpy(dens, s->dens.data(), s->dens.size() * sizeof(float));
  if (type) std::memcpy(type, s->type.data(), s->type.size());
}

extern "C" void orc_sim_get_grid(const OrcSim *s, float *u0, float *u1, float *u2,
                                 uint8_t *A, float *L, float *press) {
  float *dst[3] = {u0, u1, u2};
  for (int c = 0; c < 3; c++)
    if (dst[c]) std::memcpy(dst[c], s->u[c].data(), s->u[c].size() * sizeof(float));
  if (A) std::memcpy(A, s->A.data(), s->A.size());
  if (L) std::memcpy(L, s->L.data(), s->L.size() * sizeof(float));
  if (press) std::memcpy(press, s->press.data(), s->press.size() * sizeof(float));
}

/* Overwrite particle or grid state (null pointers leave a field as it is);
 * stage-level tests start both implementations from one state. */
extern "C" void orc_sim_put(OrcSim *s, const float *pos, const float *vel,
                            const float *dens) {
  if (pos) std::memcpy(s->pos.data(), pos, s->pos.size() * sizeof(float));
  if (vel) std::memcpy(s->vel.data(), vel, s->vel.size() * sizeof(float));
  if (dens) std::memcpy(s->dens.data(), dens, s->dens.size() * sizeof(float));
}

extern "C" void orc_sim_put_grid(OrcSim *s, const float *u0, const float *u1,
                                 const float *u2, const uint8_t *A, const float *L,
                                 const float *press) {
  const float *src[3] = {u0, u1, u2};
  for (int c = 0; c < 3; c++)
    if (src[c]) std::memcpy(s->u[c].data(), src[c], s->u[c].size() * sizeof(float));
  if (A) std::memcpy(s->A.data(), A, s->A.size());
  if (L) std::memcpy(s->L.data(), L, s->L.size() * sizeof(float));
  if (press) std::memcpy(s->press.data(), press, s->press.size() * sizeof(float));
}

extern "C" int orc_sim_last_stuck(const OrcSim *s) { return s->last_stuck; }
extern "C" double orc_sim_last_r2(const OrcSim *s) { return s->last_r2; }
extern "C" void orc_sim_set_step(OrcSim *s, int64_t step) { s->step = step; }

extern "C" void orc_sim_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* Max-density calibration (src/flip3D.cpp:689-709): a 10^3 lattice at
 * spacing DENSITY/N, densities with max_dens = 1, then the maximum. */
extern "C" float orc_max_density(int n, float density) {
  const float h = (float)((double)density / n);
  const int np = 1000;
  std::vector<float> pos(3 * np);
  std::vector<uint8_t> type(np, ORC_FLUID);
  int m = 0;
  for (int i = 0; i < 10; i++)
    for (int j = 0; j < 10; j++)
      for (int k = 0; k < 10; k++, m++) {
        pos[3 * m + 0] = (float)((i + 0.5) * (double)h);
        pos[3 * m + 1] = (float)((j + 0.5) * (double)h);
        pos[3 * m + 2] = (float)((k + 0.5) * (double)h);
      }
  const size_t nc = (size_t)n * n * n;
  std::vector<uint32_t> cs(nc + 1), perm(np);
  orc_sort(n, np, pos.data(), cs.data(), perm.data());
  std::vector<float> dens(np);
  orc_density(n, np, pos.data(), type.data(), cs.data(), perm.data(),
              (float)(4.0 * (double)density / n), 1.0f, dens.data());
  float md = 0.0f;
  for (int p = 0; p < np; p++) md = (float)std::fmax((double)md, (double)dens[p]);
  return md;
}

/* ================================================================ mesher */

namespace {

/* implicit_func (src/implicit.cpp:14-27) over the 5^3 cells around p
 * (src/implicit.cpp:29-38). The value only depends on the set of
 * neighbours: a min over fluid distances, or the wall constant if any wall
 * particle is closer than density/gn. */
double implicit_at(const Cells &cells, const float *pos, const uint8_t *type,
                   const float p[3], float density) {
  const int gn = cells.gn;
  const int ci = cell_clamp(p[0], gn), cj = cell_clamp(p[1], gn), ck = cell_clamp(p[2], gn);
  double phi = 8.0 * (double)density / gn;
  const float wall_r = density / (float)gn;
  bool wall = false;
  cells.visit(ci - 2, ci + 2, cj - 2, cj + 2, ck - 2, ck + 2, [&](uint32_t q) {
    if (wall) return;
    float d = length(pos + 3 * (size_t)q, p);
    if (type[q] == ORC_WALL) {
      if (d < wall_r) wall = true;
      return;
    }
    if ((double)d < phi) phi = d;
  });
  if (wall) return 4.5 * (double)density / gn;
  return phi - (double)wall_r;
}

inline bool is_normal(double x) { return std::isnormal(x); }

} // namespace

struct OrcMesh {
  int mg;
  std::vector<float> phi;     /* (mg)^3, x fastest */
  std::vector<double> vert, nrm;
  std::vector<int32_t> faces;
  int64_t ntris;
};

extern "C" void orc_implicit(int n, const float *pos, const uint8_t *type,
                             const uint32_t *cs, const uint32_t *perm, float density,
                             int m, const float *pts, double *out) {
  Cells cells{n, cs, perm};
  for (int i = 0; i < m; i++) out[i] = implicit_at(cells, pos, type, pts + 3 * i, density);
}

/* generateMesh (src/mesher.cpp:137-195): field, marching cubes
 * (src/rchandra/CIsoSurface.cpp:331-780), long-edge face filter, connections
 * and two smoothing passes. Marching cubes is restated without its maps:
 * every cut grid edge gets one vertex, numbered in increasing edge id
 * 3*node + axis (node = (z*(n+1) + y)*(n+1) + x); triangles come cell by
 * cell with x outermost and z innermost, each cell's in table order. */
extern "C" OrcMesh *orc_mesh(int n, const float *pos, const uint8_t *type,
                             const uint32_t *cs, const uint32_t *perm, float density) {
  OrcMesh *M = new OrcMesh;
  const int mg = n + 1, C = n;
  M->mg = mg;
  const size_t nn = (size_t)mg * mg * mg;
  M->phi.resize(nn);
  Cells cells{n, cs, perm};
  /* density field (src/mesher.cpp:142-153) */
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < mg; i++)
    for (int j = 0; j < mg; j++)
      for (int k = 0; k < mg; k++) {
        const double h = 1.0 / (double)(mg - 1);
        float p[3] = {(float)(i * h), (float)(j * h), (float)(k * h)};
        double value = implicit_at(cells, pos, type, p, density);
        if (i == 0 || i == mg - 1 || j == 0 || j == mg - 1 || k == 0 || k == mg - 1)
          value = std::fmax(value, 0.01);
        M->phi[((size_t)mg * mg) * k + (size_t)mg * j + i] = (float)(-value);
      }
  const float *F = M->phi.data();
  auto node = [&](int x, int y, int z) { return ((size_t)z * mg + y) * mg + x; };
  auto inside = [&](size_t v) { return F[v] < 0.0f; };
  const float L = (float)(1.0 / (double)(mg - 1));
  /* vertices: one per cut edge in increasing edge id */
  std::vector<int32_t> vid(3 * nn, -1);
  std::vector<float> V;
  for (int z = 0; z <= C; z++)
    for (int y = 0; y <= C; y++)
      for (int x = 0; x <= C; x++) {
        const size_t b = node(x, y, z);
        for (int a = 0; a < 3; a++) {
          int fx = x + (a == 0), fy = y + (a == 1), fz = z + (a == 2);
          if (fx > C || fy > C || fz > C) continue;
          const size_t f = node(fx, fy, fz);
          if (inside(b) == inside(f)) continue;
          /* The cell that owns the edge interpolates it: from the far node
           * to the base node for x edges below the top y row and for y edges
           * on the last x column, from the base node otherwise
           * (CalculateIntersection, src/rchandra/CIsoSurface.cpp:580-680). */
          bool rev = (a == 0 && y < C) || (a == 1 && x == C);
          int v1[3] = {x, y, z}, v2[3] = {fx, fy, fz};
          if (rev) std::swap(v1, v2);
          float val1 = F[node(v1[0], v1[1], v1[2])], val2 = F[node(v2[0], v2[1], v2[2])];
          float mu = (0.0f - val1) / (val2 - val1);
          vid[3 * b + a] = (int32_t)(V.size() / 3);
          for (int d = 0; d < 3; d++) {
            float p1 = (float)(unsigned)v1[d] * L, p2 = (float)(unsigned)v2[d] * L;
            V.push_back(p1 + mu * (p2 - p1));
          }
        }
      }
  const size_t nv = V.size() / 3;
  /* triangles */
  signed char tri[256][16];
  unsigned char tcount[256];
  flip_mc_decode(tri, tcount);
  std::vector<int32_t> T;
  for (int x = 0; x < C; x++)
    for (int y = 0; y < C; y++)
      for (int z = 0; z < C; z++) {
        unsigned idx = 0;
        for (int c = 0; c < 8; c++)
          if (inside(node(x + FLIP_MC_CORNER[c][0], y + FLIP_MC_CORNER[c][1],
                          z + FLIP_MC_CORNER[c][2])))
            idx |= 1u << c;
        for (int t = 0; t < 3 * tcount[idx]; t++) {
          const unsigned char *e = FLIP_MC_EDGE_NODE[tri[idx][t]];
          T.push_back(vid[3 * node(x + e[0], y + e[1], z + e[2]) + e[3]]);
        }
      }
  const size_t nt = T.size() / 3;
  M->ntris = (int64_t)nt;
  /* CalculateNormals (src/rchandra/CIsoSurface.cpp:740-778): all triangles */
  std::vector<float> Nf(3 * nv, 0.0f);
  for (size_t t = 0; t < nt; t++) {
    const float *p0 = &V[3 * (size_t)T[3 * t]], *p1 = &V[3 * (size_t)T[3 * t + 1]],
                *p2 = &V[3 * (size_t)T[3 * t + 2]];
    float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    float b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    float nr[3] = {a[2] * b[1] - a[1] * b[2], a[0] * b[2] - a[2] * b[0],
                   a[1] * b[0] - a[0] * b[1]};
    for (int q = 0; q < 3; q++)
      for (int d = 0; d < 3; d++) Nf[3 * (size_t)T[3 * t + q] + d] += nr[d];
  }
  for (size_t v = 0; v < nv; v++) {
    float *x = &Nf[3 * v];
    float len = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    x[0] /= len;
    x[1] /= len;
    x[2] /= len;
  }
  /* faces with every edge shorter than 0.1 (src/mesher.cpp:166-183) */
  const double maxlen2 = 0.1 * 0.1;
  for (size_t t = 0; t < nt; t++) {
    const float *p0 = &V[3 * (size_t)T[3 * t]], *p1 = &V[3 * (size_t)T[3 * t + 1]],
                *p2 = &V[3 * (size_t)T[3 * t + 2]];
    if (length2(p0, p1) < maxlen2 && length2(p1, p2) < maxlen2 && length2(p0, p2) < maxlen2)
      for (int q = 0; q < 3; q++) M->faces.push_back(T[3 * t + q]);
  }
  /* buildConnection (src/mesher.cpp:89-101) */
  std::vector<std::vector<int32_t>> conn(nv);
  for (size_t f = 0; f < M->faces.size(); f += 3) {
    int32_t a = M->faces[f], b = M->faces[f + 1], c = M->faces[f + 2];
    conn[a].push_back(b), conn[a].push_back(c);
    conn[b].push_back(a), conn[b].push_back(c);
    conn[c].push_back(a), conn[c].push_back(b);
  }
  /* smoothMesh(..., 2, 1, 1) (src/mesher.cpp:13-87) */
  std::vector<double> &X = M->vert, &Y = M->nrm;
  X.assign(V.begin(), V.end());
  Y.assign(Nf.begin(), Nf.end());
  std::vector<double> cx(3 * nv, 0.0), cy(3 * nv, 0.0);
  for (int it = 0; it < 2; it++) {
#pragma omp parallel for schedule(static)
    for (long vi = 0; vi < (long)nv; vi++) {
      float wsum = 0.0f;
      double v[3] = {0.0, 0.0, 0.0}, vn[3] = {0.0, 0.0, 0.0};
      auto add = [&](size_t u) {
        for (int d = 0; d < 3; d++)
          if (!is_normal(X[3 * u + d]) || !is_normal(Y[3 * u + d])) return;
        for (int d = 0; d < 3; d++) {
          v[d] += 1.0 * X[3 * u + d];
          vn[d] += 1.0 * Y[3 * u + d];
        }
        wsum += 1.0f;
      };
      add((size_t)vi);
      for (int32_t u : conn[vi]) add((size_t)u);
      float len = hypotf((float)vn[0], hypotf((float)vn[1], (float)vn[2]));
      for (int d = 0; d < 3; d++) {
        if (wsum != 0.0f) cx[3 * vi + d] = v[d] / (double)wsum;
        if (len != 0.0f) cy[3 * vi + d] = vn[d] / len;
      }
    }
    X = cx;
    Y = cy;
  }
  return M;
}

/* The mesh write_mesh makes after a step (src/flip3D.cpp:999-1004): the
 * lists of the last sort over the current positions. */
extern "C" OrcMesh *orc_sim_mesh(const OrcSim *s) {
  return orc_mesh(s->prm.n, s->pos.data(), s->type.data(), s->cs.data(), s->perm.data(),
                  s->prm.density);
}

extern "C" void orc_mesh_counts(const OrcMesh *m, int64_t *nverts, int64_t *nfaces,
                                int64_t *ntris) {
  if (nverts) *nverts = (int64_t)(m->vert.size() / 3);
  if (nfaces) *nfaces = (int64_t)(m->faces.size() / 3);
  if (ntris) *ntris = m->ntris;
}

extern "C" void orc_mesh_get(const OrcMesh *m, double *vertices, double *normals,
                             int32_t *faces, float *phi) {
  if (vertices) std::memcpy(vertices, m->vert.data(), m->vert.size() * sizeof(double));
  if (normals) std::memcpy(normals, m->nrm.data(), m->nrm.size() * sizeof(double));
  if (faces) std::memcpy(faces, m->faces.data(), m->faces.size() * sizeof(int32_t));
  if (phi) std::memcpy(phi, m->phi.data(), m->phi.size() * sizeof(float));
}

extern "C" void orc_mesh_free(OrcMesh *m) { delete m; }
