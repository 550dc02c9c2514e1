/*
 * shim_driver.cpp — calls the GPU shim through the reference's call surface
 * (sorter, mapper, solver, corrector) the way src/flip3D.cpp does, on inputs
 * written by tests/test_gpu_shim.py, and writes every result for comparison
 * with the CPU oracle.
 *
 *   shim_driver in.bin out.bin
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "corrector.h"
#include "implicit.h"
#include "mapper.h"
#include "mesher.h"
#include "solver.h"
#include "sorter.h"

template <class T> static T ***alloc3(int w, int h, int d) {
  T ***f = new T **[w + 1];
  for (int i = 0; i < w; i++) {
    f[i] = new T *[h + 1];
    for (int j = 0; j < h; j++) f[i][j] = new T[d];
    f[i][h] = NULL;
  }
  f[w] = NULL;
  return f;
}

template <class T> static void rd(FILE *f, T *p, size_t n) {
  if (fread(p, sizeof(T), n, f) != n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
}
template <class T> static void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

template <class T> static void load3(FILE *f, T ***g, int w, int h, int d) {
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++) rd(f, g[i][j], d);
}
template <class T> static void save3(FILE *f, T ***g, int w, int h, int d) {
  for (int i = 0; i < w; i++)
    for (int j = 0; j < h; j++) wr(f, g[i][j], d);
}

int main(int argc, char **argv) {
  if (argc != 3) return 1;
  FILE *in = fopen(argv[1], "rb");
  int n, np, nq;
  rd(in, &n, 1);
  rd(in, &np, 1);
  std::vector<float> pos(3 * np), vel(3 * np), nrm(3 * np), dens(np);
  std::vector<unsigned char> type(np);
  rd(in, pos.data(), pos.size());
  rd(in, vel.data(), vel.size());
  rd(in, nrm.data(), nrm.size());
  rd(in, type.data(), type.size());
  rd(in, dens.data(), dens.size());
  FLOAT ***grid[3] = {alloc3<FLOAT>(n + 1, n, n), alloc3<FLOAT>(n, n + 1, n),
                      alloc3<FLOAT>(n, n, n + 1)};
  load3(in, grid[0], n + 1, n, n);
  load3(in, grid[1], n, n + 1, n);
  load3(in, grid[2], n, n, n + 1);
  FLOAT ***b = alloc3<FLOAT>(n, n, n), ***x = alloc3<FLOAT>(n, n, n);
  load3(in, b, n, n, n);
  load3(in, x, n, n, n);
  rd(in, &nq, 1);
  std::vector<float> q(3 * nq);
  rd(in, q.data(), q.size());
  fclose(in);

  std::vector<particle> pool(np);
  std::vector<particle *> ps(np);
  for (int i = 0; i < np; i++) {
    memset(&pool[i], 0, sizeof(particle));
    for (int c = 0; c < 3; c++) {
      pool[i].p[c] = pos[3 * i + c];
      pool[i].u[c] = vel[3 * i + c];
      pool[i].n[c] = nrm[3 * i + c];
    }
    pool[i].type = (char)type[i];
    pool[i].dens = dens[i];
    pool[i].m = 1.0f;
    ps[i] = &pool[i];
  }
  FILE *out = fopen(argv[2], "wb");

  sorter s(n);
  s.sort(ps);
  /* cell lists through the neighbour query, cell by cell */
  std::vector<unsigned> cs(1, 0), perm;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        std::vector<particle *> v = s.getNeigboringParticles_cell(i, j, k, 0, 0, 0);
        for (particle *p : v) perm.push_back((unsigned)(p - &pool[0]));
        cs.push_back((unsigned)perm.size());
        if (s.getNumParticleAt(i, j, k) != (int)v.size()) return 3;
      }
  wr(out, cs.data(), cs.size());
  wr(out, perm.data(), perm.size());
  /* a 3x3x3 query in the middle of the grid */
  std::vector<particle *> nb = s.getNeigboringParticles_cell(n / 2, n / 3, n / 2, 1, 1, 1);
  int nbn = (int)nb.size();
  wr(out, &nbn, 1);
  for (particle *p : nb) {
    unsigned id = (unsigned)(p - &pool[0]);
    wr(out, &id, 1);
  }

  char ***A = alloc3<char>(n, n, n);
  FLOAT ***L = alloc3<FLOAT>(n, n, n);
  FLOAT ***hw = alloc3<FLOAT>(n, n, n);
  s.markWater(A, hw, 0.5f);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) L[i][j][k] = s.levelset(i, j, k, hw, 0.5f);
  save3(out, A, n, n, n);
  save3(out, L, n, n, n);

  FLOAT ***u[3] = {alloc3<FLOAT>(n + 1, n, n), alloc3<FLOAT>(n, n + 1, n),
                   alloc3<FLOAT>(n, n, n + 1)};
  mapper::mapP2G(&s, ps, u, n);
  save3(out, u[0], n + 1, n, n);
  save3(out, u[1], n, n + 1, n);
  save3(out, u[2], n, n, n + 1);

  for (int qq = 0; qq < nq; qq++) {
    FLOAT r[3];
    mapper::fetchVelocity(&q[3 * qq], r, grid, n);
    wr(out, r, 3);
  }
  mapper::mapG2P(ps, grid, n);
  for (int i = 0; i < np; i++) wr(out, pool[i].u, 3);

  solver::setSubcell(1);
  solver::solve(A, L, x, b, n);
  save3(out, x, n, n, n);
  save3(out, b, n, n, n);

  /* corrector on the original particle state */
  for (int i = 0; i < np; i++)
    for (int c = 0; c < 3; c++) {
      pool[i].p[c] = pos[3 * i + c];
      pool[i].u[c] = vel[3 * i + c];
    }
  corrector::setRandomKey(7, 3);
  corrector::correct(&s, ps, 0.006f, (FLOAT)(0.5 / n));
  for (int i = 0; i < np; i++) wr(out, pool[i].p, 3);
  for (int i = 0; i < np; i++) wr(out, pool[i].u, 3);
  /* resample at the first query point against the lists kept by correct */
  FLOAT ru[3] = {0.0f, 0.0f, 0.0f};
  corrector::resample(&s, &q[0], ru, (FLOAT)(1.0 / n));
  wr(out, ru, 3);
  /* implicit field and the mesh write_mesh makes, on the same lists */
  double phi = implicit::implicit_func(&s, &q[0], 0.5f);
  wr(out, &phi, 1);
  std::vector<double> mv, mn;
  std::vector<int> mf;
  mesher::generateMesh(A, &s, ps, 0.5f, n + 1, mv, mn, mf);
  long long counts[2] = {(long long)(mv.size() / 3), (long long)(mf.size() / 3)};
  wr(out, counts, 2);
  wr(out, mv.data(), mv.size());
  wr(out, mn.data(), mn.size());
  wr(out, mf.data(), mf.size());
  fclose(out);
  return 0;
}
