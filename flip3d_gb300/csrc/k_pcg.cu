/*
 * k_pcg.cu — solver::solve (src/solver.cpp:183-241) on the GPU.
 *
 * The CG recurrence keeps its scalars (alpha, beta, z.r, r.r, the stop
 * bound) in device memory; every kernel of an iteration first reads the
 * device `done` flag, so the host launches iterations in chunks and polls the
 * flag once per chunk instead of once per iteration. Dot products are FP64,
 * reduced in a fixed order (grid-stride per thread, fixed block tree, fixed
 * spine), so a solve is deterministic.
 *
 * REF mode follows the reference's arithmetic: the 7-point sum of
 * compute_Ax in double (src/solver.cpp:29-41), op() in float, float(r.r) in
 * the stop test, and the preconditioner as written (src/solver.cpp:119-180),
 * whose neighbour terms act only on entries equal to 1.0: with no diagonal
 * entry equal to 1.0 it is an exact diagonal scaling (two double
 * multiplies); otherwise a sequential pass reproduces it. The one departure
 * is the order of the FP64 dot sums (tree instead of sequential), which
 * moves alpha/beta by ~1e-16 relative.
 *
 * FAST mode: FP32 matvec with a precomputed diagonal (the same operator),
 * Jacobi or IC preconditioner in FP32, FP64 dots, stop when
 * r.r <= rel_tol^2 * b.b.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "devcommon.cuh"

namespace {

constexpr int BLK = 256;
constexpr int RED_BLOCKS = 1024; /* fixed grid for deterministic reductions */
constexpr int SPINE = 1024;

struct SolveArgs {
  int n;
  int subcell;
  int pow2;        /* n is a power of two: dividing by h2 is exact scaling */
  double inv_h2;   /* 1/(double)h2 */
  double h2;       /* (double)(float)(1.0/(n*n)) */
  float inv_h2_f;
};

__device__ __forceinline__ bool in_range(int n, int i, int j, int k) {
  return i >= 0 && i < n && j >= 0 && j < n && k >= 0 && k < n;
}

__device__ __forceinline__ void decode(size_t c, int n, int &i, int &j, int &k) {
  decode_index(c, n, n, i, j, k);
}

/* A_diag (src/solver.cpp:103-117) in float with the reference's double
 * promotions. */
__device__ float a_diag(const uint8_t *__restrict__ A, const float *__restrict__ L, int n,
                        int subcell, int i, int j, int k) {
  float diag = 6.0f;
  const int q[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                       {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
  const float Lc = L[cell_id(n, i, j, k)];
#pragma unroll
  for (int m = 0; m < 6; m++) {
    int qi = q[m][0], qj = q[m][1], qk = q[m][2];
    if (!in_range(n, qi, qj, qk) || A[cell_id(n, qi, qj, qk)] == CELL_WALL) {
      diag = (float)((double)diag - 1.0);
    } else if (A[cell_id(n, qi, qj, qk)] == CELL_AIR && subcell) {
      diag = (float)((double)diag -
                     (double)L[cell_id(n, qi, qj, qk)] / fmin(1.0e-6, (double)Lc));
    }
  }
  return diag;
}

/* --------------------------------------------------------------- setup */

/* flip(b) over every cell (src/solver.cpp:76-80); REF preconditioner
 * diagonal P = 1/sqrtf(diag) for FLUID cells, or FAST-mode FP32 diagonal;
 * flags a REF entry equal to 1.0. */
__global__ void __launch_bounds__(BLK)
k_setup(SolveArgs s, int mode, const uint8_t *__restrict__ A, const float *__restrict__ L,
        float *__restrict__ b, double *__restrict__ P, float *__restrict__ diag,
        float *__restrict__ Pf, int *__restrict__ iflags) {
  size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  const size_t nc = (size_t)s.n * s.n * s.n;
  if (c >= nc) return;
  b[c] = -b[c];
  if (A[c] != CELL_FLUID) {
    if (P) P[c] = 0.0;
    if (diag) diag[c] = 0.0f;
    if (Pf) Pf[c] = 0.0f;
    return;
  }
  int i, j, k;
  decode(c, s.n, i, j, k);
  float d = a_diag(A, L, s.n, s.subcell, i, j, k);
  if (mode == FLIPGPU_SOLVE_REF) {
    double pv = 1.0 / (double)sqrtf(d);
    P[c] = pv;
    if (pv == 1.0) atomicOr(iflags + IF_EXOTIC, 1);
  } else {
    diag[c] = d;
    if (Pf) Pf[c] = 1.0f / d;
  }
}

/* The reference's buildPreconditioner as written, sequentially, for the
 * rare case of a diagonal entry equal to 1.0 (then neighbour terms act). */
__global__ void k_build_ref_seq(int n, const uint8_t *__restrict__ A, double *__restrict__ P,
                                const float *__restrict__ dummy, const int *__restrict__ iflags,
                                const float *__restrict__ L, int subcell) {
  if (threadIdx.x || blockIdx.x || !iflags[IF_EXOTIC]) return;
  (void)dummy;
  auto Pref = [&](int i, int j, int k) -> float {
    if (!in_range(n, i, j, k) || P[cell_id(n, i, j, k)] != 1.0) return 0.0f;
    return (float)P[cell_id(n, i, j, k)];
  };
  auto Aref = [&](int i, int j, int k, int qi, int qj, int qk) -> float {
    if (!in_range(n, i, j, k) || A[cell_id(n, i, j, k)] != CELL_FLUID) return 0.0f;
    if (!in_range(n, qi, qj, qk) || A[cell_id(n, qi, qj, qk)] != CELL_FLUID) return 0.0f;
    return -1.0f;
  };
  for (size_t c = 0; c < (size_t)n * n * n; c++) P[c] = 0.0;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        if (A[cell_id(n, i, j, k)] != CELL_FLUID) continue;
        double left = (double)(Aref(i - 1, j, k, i, j, k) * Pref(i - 1, j, k));
        double bottom = (double)(Aref(i, j - 1, k, i, j, k) * Pref(i, j - 1, k));
        double back = (double)(Aref(i, j, k - 1, i, j, k) * Pref(i, j, k - 1));
        double diag = (double)a_diag(A, L, n, subcell, i, j, k);
        float sl = (float)left, sb = (float)bottom, sk = (float)back;
        double e = diag - (double)(sl * sl) - (double)(sb * sb) - (double)(sk * sk);
        if (e < 0.25 * diag) e = diag;
        P[cell_id(n, i, j, k)] = 1.0 / (double)sqrtf((float)e);
      }
}

/* ------------------------------------------------------------- matvec */

/* compute_Ax (src/solver.cpp:29-41) with its double arithmetic. */
__global__ void __launch_bounds__(BLK)
k_matvec_ref(SolveArgs s, const int *__restrict__ iflags, const uint8_t *__restrict__ A,
             const float *__restrict__ L, const float *__restrict__ x, float *__restrict__ ans) {
  if (iflags[IF_DONE]) return;
  size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  const int n = s.n;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  if (A[c] != CELL_FLUID) {
    ans[c] = 0.0f;
    return;
  }
  int i, j, k;
  decode(c, n, i, j, k);
  const float xc = x[c];
  const float Lc = L[c];
  auto xref = [&](int qi, int qj, int qk) -> float {
    qi = min(max(0, qi), n - 1);
    qj = min(max(0, qj), n - 1);
    qk = min(max(0, qk), n - 1);
    size_t q = cell_id(n, qi, qj, qk);
    uint8_t a = A[q];
    if (a == CELL_FLUID) return x[q];
    if (a == CELL_WALL) return xc;
    return s.subcell ? (float)((double)L[q] / fmin(1.0e-6, (double)Lc) * (double)xc) : 0.0f;
  };
  double v = 6.0 * (double)xc;
  v -= (double)xref(i + 1, j, k);
  v -= (double)xref(i - 1, j, k);
  v -= (double)xref(i, j + 1, k);
  v -= (double)xref(i, j - 1, k);
  v -= (double)xref(i, j, k + 1);
  v -= (double)xref(i, j, k - 1);
  ans[c] = s.pow2 ? (float)(v * s.inv_h2) : (float)(v / s.h2);
}

/* FP32 matvec of the same operator: (diag*x - sum of fluid neighbours)/h2. */
__global__ void __launch_bounds__(BLK)
k_matvec_fast(SolveArgs s, const int *__restrict__ iflags, const uint8_t *__restrict__ A,
              const float *__restrict__ diag, const float *__restrict__ x,
              float *__restrict__ ans) {
  if (iflags[IF_DONE]) return;
  size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  const int n = s.n;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  if (A[c] != CELL_FLUID) {
    ans[c] = 0.0f;
    return;
  }
  int i, j, k;
  decode(c, n, i, j, k);
  float acc = diag[c] * x[c];
  const size_t sj = n, si = (size_t)n * n;
  if (i + 1 < n && A[c + si] == CELL_FLUID) acc -= x[c + si];
  if (i > 0 && A[c - si] == CELL_FLUID) acc -= x[c - si];
  if (j + 1 < n && A[c + sj] == CELL_FLUID) acc -= x[c + sj];
  if (j > 0 && A[c - sj] == CELL_FLUID) acc -= x[c - sj];
  if (k + 1 < n && A[c + 1] == CELL_FLUID) acc -= x[c + 1];
  if (k > 0 && A[c - 1] == CELL_FLUID) acc -= x[c - 1];
  ans[c] = acc * s.inv_h2_f;
}

/* ------------------------------------------------------ preconditioner */

/* applyPreconditioner as written with no entry equal to 1.0: every
 * neighbour term is a signed zero, so q = r*P and z = float(q*P) in double;
 * the zeros' signs are reproduced for exact-zero residuals. */
__global__ void __launch_bounds__(BLK)
k_apply_ref_diag(SolveArgs s, const int *__restrict__ iflags, const uint8_t *__restrict__ A,
                 const double *__restrict__ P, const float *__restrict__ r,
                 float *__restrict__ z) {
  if (iflags[IF_DONE] || iflags[IF_EXOTIC]) return;
  size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  const int n = s.n;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc || A[c] != CELL_FLUID) return;
  int i, j, k;
  decode(c, n, i, j, k);
  const float rc = r[c];
  double t = (double)rc;
  if (rc == 0.0f) {
    bool back = (i > 0 && A[cell_id(n, i - 1, j, k)] == CELL_FLUID) ||
                (j > 0 && A[cell_id(n, i, j - 1, k)] == CELL_FLUID) ||
                (k > 0 && A[cell_id(n, i, j, k - 1)] == CELL_FLUID);
    t = (signbit(rc) && !back) ? -0.0 : 0.0;
  }
  const double pc = P[c];
  double q = t * pc;
  double t2 = q;
  if (q == 0.0) {
    bool fwd = (i + 1 < n && A[cell_id(n, i + 1, j, k)] == CELL_FLUID) ||
               (j + 1 < n && A[cell_id(n, i, j + 1, k)] == CELL_FLUID) ||
               (k + 1 < n && A[cell_id(n, i, j, k + 1)] == CELL_FLUID);
    t2 = (signbit(q) && !fwd) ? -0.0 : 0.0;
  }
  z[c] = (float)(t2 * pc);
}

/* applyPreconditioner as written (src/solver.cpp:141-180), sequentially,
 * when some diagonal entry equals 1.0. */
__global__ void k_apply_ref_seq(int n, const int *__restrict__ iflags,
                                const uint8_t *__restrict__ A, const double *__restrict__ P,
                                const float *__restrict__ r, float *__restrict__ z,
                                double *__restrict__ q) {
  if (threadIdx.x || blockIdx.x || iflags[IF_DONE] || !iflags[IF_EXOTIC]) return;
  auto Aref = [&](int i, int j, int k, int qi, int qj, int qk) -> float {
    if (!in_range(n, i, j, k) || A[cell_id(n, i, j, k)] != CELL_FLUID) return 0.0f;
    if (!in_range(n, qi, qj, qk) || A[cell_id(n, qi, qj, qk)] != CELL_FLUID) return 0.0f;
    return -1.0f;
  };
  auto PrefD = [&](const double *X, int i, int j, int k) -> float {
    if (!in_range(n, i, j, k) || X[cell_id(n, i, j, k)] != 1.0) return 0.0f;
    return (float)X[cell_id(n, i, j, k)];
  };
  auto PrefF = [&](const float *X, int i, int j, int k) -> float {
    if (!in_range(n, i, j, k) || X[cell_id(n, i, j, k)] != 1.0f) return 0.0f;
    return X[cell_id(n, i, j, k)];
  };
  const size_t nc = (size_t)n * n * n;
  for (size_t c = 0; c < nc; c++) q[c] = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        if (A[cell_id(n, i, j, k)] != CELL_FLUID) continue;
        double left = (double)(Aref(i - 1, j, k, i, j, k) * PrefD(P, i - 1, j, k) * PrefD(q, i - 1, j, k));
        double bottom = (double)(Aref(i, j - 1, k, i, j, k) * PrefD(P, i, j - 1, k) * PrefD(q, i, j - 1, k));
        double back = (double)(Aref(i, j, k - 1, i, j, k) * PrefD(P, i, j, k - 1) * PrefD(q, i, j, k - 1));
        double t = (double)r[cell_id(n, i, j, k)] - left - bottom - back;
        q[cell_id(n, i, j, k)] = t * P[cell_id(n, i, j, k)];
      }
  for (int i = n - 1; i >= 0; i--)
    for (int j = n - 1; j >= 0; j--)
      for (int k = n - 1; k >= 0; k--) {
        if (A[cell_id(n, i, j, k)] != CELL_FLUID) continue;
        double right = (double)(Aref(i, j, k, i + 1, j, k) * PrefD(P, i, j, k) * PrefF(z, i + 1, j, k));
        double top = (double)(Aref(i, j, k, i, j + 1, k) * PrefD(P, i, j, k) * PrefF(z, i, j + 1, k));
        double front = (double)(Aref(i, j, k, i, j, k + 1) * PrefD(P, i, j, k) * PrefF(z, i, j, k + 1));
        double t = q[cell_id(n, i, j, k)] - right - top - front;
        z[cell_id(n, i, j, k)] = (float)(t * P[cell_id(n, i, j, k)]);
      }
}

/* FAST Jacobi: z = r / diag on FLUID cells. */
__global__ void __launch_bounds__(BLK)
k_apply_jacobi(SolveArgs s, const int *__restrict__ iflags, const uint8_t *__restrict__ A,
               const float *__restrict__ Pf, const float *__restrict__ r,
               float *__restrict__ z) {
  if (iflags[IF_DONE]) return;
  size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  const size_t nc = (size_t)s.n * s.n * s.n;
  if (c >= nc) return;
  z[c] = (A[c] == CELL_FLUID) ? r[c] * Pf[c] : 0.0f;
}

/* ---------------------------------------------------- vector updates */

/* FP64 partial sums of float(x*y) over FLUID cells (product,
 * src/solver.cpp:44-54); grid-stride over a fixed grid. */
__global__ void __launch_bounds__(BLK)
k_dot(size_t nc, const int *__restrict__ iflags, int check_done, const uint8_t *__restrict__ A,
      const float *__restrict__ x, const float *__restrict__ y, double *__restrict__ partial) {
  if (check_done && iflags[IF_DONE]) return;
  double acc = 0.0;
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK)
    if (A[c] == CELL_FLUID) acc += (double)(x[c] * y[c]);
  double t = block_sum_double<BLK>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

/* r = b - z (op with a = -1, src/solver.cpp:190) and r.r partials. */
__global__ void __launch_bounds__(BLK)
k_residual(size_t nc, const uint8_t *__restrict__ A, const float *__restrict__ b,
           const float *__restrict__ z, float *__restrict__ r, double *__restrict__ partial) {
  double acc = 0.0;
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK) {
    float v = 0.0f;
    if (A[c] == CELL_FLUID) {
      v = b[c] + -1.0f * z[c];
      acc += (double)(v * v);
    }
    r[c] = v;
  }
  double t = block_sum_double<BLK>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

/* x = x + alpha*s, r = r - alpha*z (op, src/solver.cpp:202-203) and r.r. */
__global__ void __launch_bounds__(BLK)
k_update_xr(size_t nc, const int *__restrict__ iflags, const double *__restrict__ scal,
            const uint8_t *__restrict__ A, float *__restrict__ x, float *__restrict__ r,
            const float *__restrict__ s, const float *__restrict__ z,
            double *__restrict__ partial) {
  if (iflags[IF_DONE]) return;
  const float alpha = (float)scal[SC_ALPHA];
  const float nalpha = (float)(-scal[SC_ALPHA]);
  double acc = 0.0;
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK) {
    if (A[c] == CELL_FLUID) {
      x[c] = x[c] + alpha * s[c];
      float rv = r[c] + nalpha * z[c];
      r[c] = rv;
      acc += (double)(rv * rv);
    } else {
      x[c] = 0.0f;
      r[c] = 0.0f;
    }
  }
  double t = block_sum_double<BLK>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

/* s = z + beta*s (op, src/solver.cpp:215). */
__global__ void __launch_bounds__(BLK)
k_update_s(size_t nc, const int *__restrict__ iflags, const double *__restrict__ scal,
           const uint8_t *__restrict__ A, const float *__restrict__ z, float *__restrict__ s) {
  if (iflags[IF_DONE]) return;
  const float beta = (float)scal[SC_BETA];
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK)
    s[c] = (A[c] == CELL_FLUID) ? z[c] + beta * s[c] : 0.0f;
}

/* ------------------------------------------------------------ scalars */

enum { ST_B2 = 0, ST_ERR0, ST_A0, ST_ALPHA, ST_CHECK, ST_BETA };

/* Sums the fixed partials (one block, fixed order) and advances the CG
 * recurrence by one scalar step. */
__global__ void __launch_bounds__(SPINE)
k_scalar(int what, int mode, int nparts, const double *__restrict__ partial,
         double *__restrict__ scal, int *__restrict__ iflags, double eps_abs, double rel_tol,
         double ref_eps, int max_iters) {
  if (what >= ST_ALPHA && iflags[IF_DONE]) return;
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += SPINE) v += partial[i];
  double sum = block_sum_double<SPINE>(v);
  if (threadIdx.x != 0) return;
  switch (what) {
  case ST_B2: {
    scal[SC_B2] = sum;
    double eps;
    if (mode == FLIPGPU_SOLVE_REF) {
      eps = ref_eps;
      if (eps_abs >= 0.0) {
        eps = eps_abs;
      } else if (rel_tol > 0.0) {
        double target = rel_tol * rel_tol * sum;
        while (eps > target && eps > 0.0) eps *= 0.25;
      }
    } else {
      eps = rel_tol * rel_tol * sum;
    }
    scal[SC_EPS] = eps;
    iflags[IF_DONE] = 0;
    iflags[IF_ITERS] = 0;
    iflags[IF_NAN] = 0;
    break;
  }
  case ST_ERR0:
    scal[SC_ERR2_0] = sum;
    scal[SC_ERR2] = sum;
    /* FAST mode stops before iterating when the guess already meets the
     * bound; REF mode always iterates once, as conjGrad does. */
    if (mode != FLIPGPU_SOLVE_REF && sum <= scal[SC_EPS]) iflags[IF_DONE] = 1;
    break;
  case ST_A0:
    scal[SC_A] = sum;
    break;
  case ST_ALPHA:
    scal[SC_ALPHA] = scal[SC_A] / sum;
    break;
  case ST_CHECK: {
    double e2 = (mode == FLIPGPU_SOLVE_REF) ? (double)(float)sum : sum;
    scal[SC_ERR2] = e2;
    int it = ++iflags[IF_ITERS];
    if (e2 <= scal[SC_EPS]) iflags[IF_DONE] = 1;
    else if (!(e2 == e2)) {
      iflags[IF_NAN] = 1;
      iflags[IF_DONE] = 2;
    } else if (it >= max_iters)
      iflags[IF_DONE] = 3;
    break;
  }
  case ST_BETA:
    scal[SC_BETA] = sum / scal[SC_A];
    scal[SC_A] = sum;
    break;
  }
}

/* ---------------------------------------------- persistent CG (one launch) */

/* The whole CG loop in one cooperative launch: two grid barriers per
 * iteration, s = z + beta*s folded into the next matvec (ping-pong s
 * buffers; neighbour values of s are recomputed from z and the old s), and
 * every block sums the per-block partials itself in the same fixed order, so
 * all blocks agree on every scalar without a broadcast and the result does
 * not depend on timing. Each thread owns the same cells in every phase; the
 * only cross-thread reads (neighbours, partials) bypass L1 (ld.cg). */
constexpr int CG_BLOCK = 256;
/* the single-reduction CG runs one block per SM: 384 threads keep a chunk's
 * loads in registers (latency-bound small grids), 512 threads keep more
 * chunks in flight (bandwidth-bound large grids, n >= CG1_LARGE_N) */
constexpr int CG1_BLOCK_SMALL = 384, CG1_BLOCK_LARGE = 512, CG1_LARGE_N = 192;
constexpr unsigned long long BAR_SPIN_LIMIT = 1ull << 26; /* ~seconds, then ETIMEOUT */

/* Geometric multigrid levels of the MG preconditioner (level 0 is the
 * solver's grid; level l has ceil(n / 2^l) cells per axis). */
constexpr int MG_MAX_LEVELS = 10;
struct MgLevel {
  int m;                 /* cells per axis */
  const uint8_t *flags;  /* CELL_FLUID / CELL_AIR / CELL_WALL */
  const float *diag;     /* level 0: the operator's diagonal; coarser: non-wall neighbours */
  float *x, *b, *res;    /* correction, right-hand side, residual */
  float hs, ihs;         /* 1 / h^2 of the level and its inverse */
  int lgm;               /* log2(m) when m is a power of two, else -1 */
};
struct MgArgs {
  MgLevel lv[MG_MAX_LEVELS];
  int nlev;              /* number of levels */
  int lb;                /* levels lb.. are solved by block 0 alone */
  int coarse_sweeps;     /* symmetric Gauss-Seidel sweeps on the coarsest level */
  int nu;                /* red-black sweeps before (and black-red after) the correction */
};

struct CgArgs {
  SolveArgs s;
  size_t nc;
  const uint8_t *A;
  const float *L;
  const float *b;
  float *x, *r, *z, *s0, *s1, *w;
  float *w1, *p;               /* single-reduction CG: second w buffer, directions */
  const unsigned *chunk_list;  /* single-reduction CG: the 32-quad chunks holding liquid */
  const unsigned *chunk_count; /* ... and their number */
  const double *P;
  const float *diag;
  const float *Pf;
  float2 *part;
  unsigned *bar;
  int *iflags;
  double *scal;
  double eps_abs, rel_tol, ref_eps;
  int max_iters;
  /* IC(0)/MIC(0) wavefront */
  float mic_tau;
  int ic_njb, ic_tasks;         /* 32-j line blocks; tasks (IC_W lines x 32 j) */
  const unsigned *ic_order;     /* tasks by increasing i block + j block */
  const unsigned *ic_line;      /* per line (i, j block): holds liquid */
  const uint8_t *ic_cf;         /* per cell: liquid flag and MIC(0) counts */
  float *ic_pf;                 /* skewed factor rows */
  unsigned long long *ic_psk, *ic_qsk, *ic_zsk; /* skewed tagged factor, q, z */
  float2 *ic_part;              /* per-task q.q partials */
  unsigned *ic_ctr;             /* tag counter: this launch tags base + 1 .. */
  int ic_factor;                /* build the factor (else the previous launch's) */
  unsigned *ticket;
  /* MG-preconditioned CG */
  float *p2, *q;               /* second direction buffer, A p */
  MgArgs mg;
  /* inner solve of the mixed-precision refinement (FAST mode): the launch
   * returns at once when *ir_skip is set (the outer loop has finished), and
   * the relative tolerance is *ir_tol (set by the outer loop) instead of
   * rel_tol. Both null outside refinement. */
  const int *ir_skip;
  const double *ir_tol;
};

/* the launch is an inner solve the refinement no longer needs */
__device__ __forceinline__ bool ir_skipped(const CgArgs &a) {
  return a.ir_skip != nullptr && *(volatile const int *)a.ir_skip != 0;
}

__device__ __forceinline__ double cg_rel_tol(const CgArgs &a) {
  return a.ir_tol != nullptr ? *(volatile const double *)a.ir_tol : a.rel_tol;
}

__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *iflags,
                                             unsigned *reset_ticket = nullptr) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    unsigned g = *gen;
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == gridDim.x - 1) {
      /* every block is past its task loop: the ticket counter can restart */
      if (reset_ticket) atomicExch(reset_ticket, 0u);
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g) {
        if (++spins > BAR_SPIN_LIMIT) {
          atomicExch(iflags + IF_TIMEOUT, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    ok = *(volatile int *)(iflags + IF_TIMEOUT) == 0;
  }
  __syncthreads();
  /* one value per block, so a block always leaves the loop as a whole */
  return ok != 0;
}

/* A counting grid barrier: bar[0] counts the arrivals of the whole launch
 * (zeroed before it), so the epoch-th barrier is complete when it reaches
 * epoch x gridDim.x. Thread 0 arrives with a release add after the block's
 * __syncthreads and polls with acquire loads: two L2 round trips, no reset
 * and no generation word. The wait gives up after 2 s of %globaltimer,
 * flags FLIPGPU_ETIMEOUT and returns false in that block (the others give up
 * at their next barrier). */
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool count_barrier(unsigned *bar, unsigned &epoch, int *iflags) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    epoch++;
    const unsigned target = epoch * gridDim.x;
    unsigned v;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(v) : "l"(bar) : "memory");
    v += 1;
    bool good = true;
    unsigned long long t0 = 0;
    unsigned spins = 0;
    while ((int)(v - target) < 0) {
      if ((++spins & 1023u) == 0) {
        const unsigned long long t = global_ns();
        if (t0 == 0) {
          t0 = t;
        } else if (t - t0 > 2000000000ull) {
          atomicExch(iflags + IF_TIMEOUT, 1);
          good = false;
          break;
        }
      }
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

/* Sums of the nb float-pair partials of slots k0 and k1 (k1 < 0: none),
 * identical in every block: strided loads, then a fixed merge tree. */
template <int BLOCK = CG_BLOCK>
__device__ __forceinline__ void sum_partials(const float2 *part, int k0, int k1, unsigned nb,
                                             double &out0, double &out1) {
  FF v0 = ff_zero(), v1 = ff_zero();
  for (unsigned i = threadIdx.x; i < nb; i += BLOCK) {
    float2 a = __ldcg(part + (size_t)k0 * nb + i);
    v0 = ff_merge(v0, FF{a.x, a.y});
    if (k1 >= 0) {
      float2 b = __ldcg(part + (size_t)k1 * nb + i);
      v1 = ff_merge(v1, FF{b.x, b.y});
    }
  }
  out0 = ff_to_double(block_sum_ff<BLOCK>(v0));
  out1 = k1 >= 0 ? ff_to_double(block_sum_ff<BLOCK>(v1)) : 0.0;
}

/* Dot-product term: REF mode sums the float-rounded product, as
 * product() does (src/solver.cpp:51); FAST mode keeps the product exact. */
template <int MODE> __device__ __forceinline__ void dot_acc(FF &acc, float x, float y) {
  if (MODE == FLIPGPU_SOLVE_REF)
    ff_add(acc, x * y);
  else
    ff_add_prod(acc, x, y);
}

template <int BLOCK = CG_BLOCK>
__device__ __forceinline__ void store_partial(float2 *part, int k, unsigned nb, FF v) {
  FF t = block_sum_ff<BLOCK>(v);
  if (threadIdx.x == 0) part[(size_t)k * nb + blockIdx.x] = make_float2(t.hi, t.lo);
}

template <int MODE>
__device__ __forceinline__ float cg_matvec(const CgArgs &a, size_t c, int i, int j, int k,
                                           float sc, const float *zv, const float *so,
                                           float beta_f, bool first) {
  const int n = a.s.n;
  auto snew = [&](size_t q) -> float {
    float zq = __ldcg(zv + q);
    return first ? zq : zq + beta_f * __ldcg(so + q);
  };
  if (MODE == FLIPGPU_SOLVE_REF) {
    const float Lc = a.L[c];
    auto xref = [&](int qi, int qj, int qk) -> float {
      qi = min(max(0, qi), n - 1);
      qj = min(max(0, qj), n - 1);
      qk = min(max(0, qk), n - 1);
      size_t q = cell_id(n, qi, qj, qk);
      uint8_t aa = a.A[q];
      if (aa == CELL_FLUID) return q == c ? sc : snew(q);
      if (aa == CELL_WALL) return sc;
      return a.s.subcell ? (float)((double)a.L[q] / fmin(1.0e-6, (double)Lc) * (double)sc)
                         : 0.0f;
    };
    double v = 6.0 * (double)sc;
    v -= (double)xref(i + 1, j, k);
    v -= (double)xref(i - 1, j, k);
    v -= (double)xref(i, j + 1, k);
    v -= (double)xref(i, j - 1, k);
    v -= (double)xref(i, j, k + 1);
    v -= (double)xref(i, j, k - 1);
    return a.s.pow2 ? (float)(v * a.s.inv_h2) : (float)(v / a.s.h2);
  } else {
    float acc = a.diag[c] * sc;
    const size_t sj = n, si = (size_t)n * n;
    if (i + 1 < n && a.A[c + si] == CELL_FLUID) acc -= snew(c + si);
    if (i > 0 && a.A[c - si] == CELL_FLUID) acc -= snew(c - si);
    if (j + 1 < n && a.A[c + sj] == CELL_FLUID) acc -= snew(c + sj);
    if (j > 0 && a.A[c - sj] == CELL_FLUID) acc -= snew(c - sj);
    if (k + 1 < n && a.A[c + 1] == CELL_FLUID) acc -= snew(c + 1);
    if (k > 0 && a.A[c - 1] == CELL_FLUID) acc -= snew(c - 1);
    return acc * a.s.inv_h2_f;
  }
}

/* z = M^-1 r at one FLUID cell (REF: the reference's preconditioner with no
 * entry equal to 1.0, signed zeros included; FAST: Jacobi). */
template <int MODE>
__device__ __forceinline__ float cg_precond(const CgArgs &a, size_t c, int i, int j, int k,
                                            float rc) {
  if (MODE == FLIPGPU_SOLVE_REF) {
    const int n = a.s.n;
    const uint8_t *A = a.A;
    double t = (double)rc;
    if (rc == 0.0f) {
      bool back = (i > 0 && A[cell_id(n, i - 1, j, k)] == CELL_FLUID) ||
                  (j > 0 && A[cell_id(n, i, j - 1, k)] == CELL_FLUID) ||
                  (k > 0 && A[cell_id(n, i, j, k - 1)] == CELL_FLUID);
      t = (signbit(rc) && !back) ? -0.0 : 0.0;
    }
    const double pc = a.P[c];
    double q = t * pc;
    double t2 = q;
    if (q == 0.0) {
      bool fwd = (i + 1 < n && A[cell_id(n, i + 1, j, k)] == CELL_FLUID) ||
                 (j + 1 < n && A[cell_id(n, i, j + 1, k)] == CELL_FLUID) ||
                 (k + 1 < n && A[cell_id(n, i, j, k + 1)] == CELL_FLUID);
      t2 = (signbit(q) && !fwd) ? -0.0 : 0.0;
    }
    return (float)(t2 * pc);
  } else {
    return rc * a.Pf[c];
  }
}

template <int MODE>
__global__ void __launch_bounds__(CG_BLOCK) k_cg(CgArgs a) {
  if (MODE != FLIPGPU_SOLVE_REF && ir_skipped(a)) return;
  const unsigned nb = gridDim.x;
  const size_t stride = (size_t)nb * CG_BLOCK;
  const size_t t0 = (size_t)blockIdx.x * CG_BLOCK + threadIdx.x;
  const int n = a.s.n;
  const size_t nc = a.nc;

  /* phase 0: r = b - A x, z = M^-1 r; b.b, r.r, z.r */
  FF pbb = ff_zero(), prr = ff_zero(), pzr = ff_zero();
  for (size_t c = t0; c < nc; c += stride) {
    float rv = 0.0f, zv = 0.0f;
    if (a.A[c] == CELL_FLUID) {
      int i, j, k;
      decode(c, n, i, j, k);
      float bc = a.b[c];
      dot_acc<MODE>(pbb, bc, bc);
      float xc = a.x[c];
      /* the initial matvec reads x, which nobody writes in this phase */
      float ax = cg_matvec<MODE>(a, c, i, j, k, xc, a.x, a.x, 0.0f, true);
      rv = bc + -1.0f * ax;
      dot_acc<MODE>(prr, rv, rv);
      zv = cg_precond<MODE>(a, c, i, j, k, rv);
      dot_acc<MODE>(pzr, zv, rv);
    }
    a.r[c] = rv;
    a.z[c] = zv;
  }
  store_partial(a.part, 0, nb, pbb);
  store_partial(a.part, 1, nb, prr);
  store_partial(a.part, 2, nb, pzr);
  if (!grid_barrier(a.bar, a.iflags)) return;
  double b2, rr, azr, unused;
  sum_partials(a.part, 0, 1, nb, b2, rr);
  sum_partials(a.part, 2, -1, nb, azr, unused);
  double eps;
  if (MODE == FLIPGPU_SOLVE_REF) {
    eps = a.ref_eps;
    if (a.eps_abs >= 0.0) {
      eps = a.eps_abs;
    } else if (a.rel_tol > 0.0) {
      double target = a.rel_tol * a.rel_tol * b2;
      while (eps > target && eps > 0.0) eps *= 0.25;
    }
  } else {
    const double rt = cg_rel_tol(a);
    eps = rt * rt * b2;
  }
  int done = 0, iters = 0;
  double e2 = rr;
  if (MODE != FLIPGPU_SOLVE_REF && rr <= eps) done = 1;
  float *so = a.s0, *sn = a.s1;
  float beta_f = 0.0f;
  bool first = true;
  while (!done) {
    /* phase A: s_new = z + beta*s_old (op), w = A s_new, w.s_new */
    FF pws = ff_zero();
    for (size_t c = t0; c < nc; c += stride) {
      float snv = 0.0f, wv = 0.0f;
      if (a.A[c] == CELL_FLUID) {
        int i, j, k;
        decode(c, n, i, j, k);
        float zc = a.z[c];
        snv = first ? zc : zc + beta_f * so[c];
        wv = cg_matvec<MODE>(a, c, i, j, k, snv, a.z, so, beta_f, first);
        dot_acc<MODE>(pws, wv, snv);
      }
      sn[c] = snv;
      a.w[c] = wv;
    }
    store_partial(a.part, 3, nb, pws);
    if (!grid_barrier(a.bar, a.iflags)) return;
    double ws;
    sum_partials(a.part, 3, -1, nb, ws, unused);
    const double alpha = azr / ws;
    const float alpha_f = (float)alpha, nalpha_f = (float)(-alpha);
    /* phase B: x += alpha s, r -= alpha w, z = M^-1 r; r.r, z.r */
    prr = ff_zero();
    pzr = ff_zero();
    for (size_t c = t0; c < nc; c += stride) {
      if (a.A[c] == CELL_FLUID) {
        int i, j, k;
        decode(c, n, i, j, k);
        a.x[c] = a.x[c] + alpha_f * sn[c];
        float rv = a.r[c] + nalpha_f * a.w[c];
        a.r[c] = rv;
        dot_acc<MODE>(prr, rv, rv);
        float zv = cg_precond<MODE>(a, c, i, j, k, rv);
        a.z[c] = zv;
        dot_acc<MODE>(pzr, zv, rv);
      } else {
        a.x[c] = 0.0f;
        a.r[c] = 0.0f;
        a.z[c] = 0.0f;
      }
    }
    store_partial(a.part, 4, nb, prr);
    store_partial(a.part, 5, nb, pzr);
    if (!grid_barrier(a.bar, a.iflags)) return;
    double zr;
    sum_partials(a.part, 4, 5, nb, rr, zr);
    iters++;
    e2 = (MODE == FLIPGPU_SOLVE_REF) ? (double)(float)rr : rr;
    if (e2 <= eps) done = 1;
    else if (!(e2 == e2)) done = 2;
    else if (iters >= a.max_iters) done = 3;
    const double beta = zr / azr;
    azr = zr;
    beta_f = (float)beta;
    first = false;
    float *t = so;
    so = sn;
    sn = t;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iflags[IF_DONE] = done;
    a.iflags[IF_ITERS] = iters;
    a.iflags[IF_NAN] = done == 2;
    a.scal[SC_ERR2] = e2;
    a.scal[SC_B2] = b2;
    a.scal[SC_EPS] = eps;
  }
}

/* Matvec on quads of 4 consecutive k-cells (n % 4 == 0) for the first
 * residual of the single-reduction CG: 16-byte loads, every neighbour load of
 * a quad issued together, k-neighbours passed between lanes by shuffles (a
 * warp's lanes hold consecutive quads of a k-row; warps walk tiles of 32
 * quads so that shuffles always see a full warp). */
struct QuadNb {
  float4 sn;      /* s_new at the neighbour quad (0 where not FLUID) */
};

__device__ __forceinline__ bool fl(unsigned char a) { return a == CELL_FLUID; }

__device__ __forceinline__ float4 quad_snew(uchar4 A4, float4 z4, float4 so4, float beta,
                                            bool first) {
  float4 r;
  r.x = fl(A4.x) ? (first ? z4.x : z4.x + beta * so4.x) : 0.0f;
  r.y = fl(A4.y) ? (first ? z4.y : z4.y + beta * so4.y) : 0.0f;
  r.z = fl(A4.z) ? (first ? z4.z : z4.z + beta * so4.z) : 0.0f;
  r.w = fl(A4.w) ? (first ? z4.w : z4.w + beta * so4.w) : 0.0f;
  return r;
}

/* s_new of the quad and of its i/j neighbours, then w = A s_new. src_z is z
 * (or x in phase 0 with first=true). Returns sn4 and w4. Every lane must
 * call it (shuffles). */
__device__ __forceinline__ void quad_matvec(const CgArgs &a, size_t q, bool valid, int qrow,
                                            size_t qplane, int i, int j, int kq,
                                            const float *src_z, const float *so, float beta,
                                            bool first, float4 &sn4, float4 &w4,
                                            uchar4 &A4) {
  const int n = a.s.n;
  const uchar4 *A4p = reinterpret_cast<const uchar4 *>(a.A);
  const float4 *z4p = reinterpret_cast<const float4 *>(src_z);
  const float4 *so4p = reinterpret_cast<const float4 *>(so);
  A4 = valid ? A4p[q] : make_uchar4(0, 0, 0, 0);
  const bool any = fl(A4.x) || fl(A4.y) || fl(A4.z) || fl(A4.w);
  sn4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (any) {
    float4 z4 = __ldcg(z4p + q);
    float4 so4 = first ? z4 : __ldcg(so4p + q);
    sn4 = quad_snew(A4, z4, so4, beta, first);
  }
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  float left = __shfl_up_sync(FULL, sn4.w, 1);
  int left_fl = __shfl_up_sync(FULL, (int)fl(A4.w), 1);
  float right = __shfl_down_sync(FULL, sn4.x, 1);
  int right_fl = __shfl_down_sync(FULL, (int)fl(A4.x), 1);
  w4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!any) return;
  const size_t c0 = 4 * q;
  const int k0 = 4 * kq;
  /* k-1 of the first cell and k+1 of the last */
  if (k0 == 0) {
    left_fl = 0;
  } else if (lane == 0) {
    unsigned char al = a.A[c0 - 1];
    left_fl = fl(al);
    if (left_fl) {
      float zl = __ldcg(src_z + c0 - 1);
      left = first ? zl : zl + beta * __ldcg(so + c0 - 1);
    }
  }
  if (k0 + 4 >= n) {
    right_fl = 0;
  } else if (lane == 31) {
    unsigned char ar = a.A[c0 + 4];
    right_fl = fl(ar);
    if (right_fl) {
      float zr = __ldcg(src_z + c0 + 4);
      right = first ? zr : zr + beta * __ldcg(so + c0 + 4);
    }
  }
  (void)qrow;
  /* i/j neighbours: issue all loads first */
  const bool has[4] = {i + 1 < n, i > 0, j + 1 < n, j > 0};
  const long off[4] = {(long)qplane, -(long)qplane, (long)qrow, -(long)qrow};
  uchar4 An[4];
  float4 zn[4], son[4];
#pragma unroll
  for (int d = 0; d < 4; d++) {
    if (has[d]) {
      size_t qq = (size_t)((long)q + off[d]);
      An[d] = A4p[qq];
      zn[d] = __ldcg(z4p + qq);
      son[d] = first ? zn[d] : __ldcg(so4p + qq);
    } else {
      An[d] = make_uchar4(0, 0, 0, 0);
      zn[d] = son[d] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  const float4 d4 = __ldg(reinterpret_cast<const float4 *>(a.diag) + q);
  float acc[4] = {d4.x * sn4.x, d4.y * sn4.y, d4.z * sn4.z, d4.w * sn4.w};
#pragma unroll
  for (int d = 0; d < 4; d++) {
    float4 v = quad_snew(An[d], zn[d], son[d], beta, first);
    acc[0] -= v.x;
    acc[1] -= v.y;
    acc[2] -= v.z;
    acc[3] -= v.w;
  }
  const float snv[4] = {sn4.x, sn4.y, sn4.z, sn4.w};
  const bool fv[4] = {fl(A4.x), fl(A4.y), fl(A4.z), fl(A4.w)};
  /* k neighbours inside the quad and across it */
  acc[0] -= (fv[1] ? snv[1] : 0.0f) + (left_fl ? left : 0.0f);
  acc[1] -= (fv[0] ? snv[0] : 0.0f) + (fv[2] ? snv[2] : 0.0f);
  acc[2] -= (fv[1] ? snv[1] : 0.0f) + (fv[3] ? snv[3] : 0.0f);
  acc[3] -= (fv[2] ? snv[2] : 0.0f) + (right_fl ? right : 0.0f);
  const float s = a.s.inv_h2_f;
  w4 = make_float4(fv[0] ? acc[0] * s : 0.0f, fv[1] ? acc[1] * s : 0.0f,
                   fv[2] ? acc[2] * s : 0.0f, fv[3] ? acc[3] * s : 0.0f);
}

/* K per-thread partial sums reduced over the block into
 * part[(k0+q)*nb + blockIdx.x] with one __syncthreads (warp shuffle trees,
 * then thread q merges the warps' value q in a fixed order). */
template <int K, int BLOCK = CG_BLOCK>
__device__ __forceinline__ void store_partials(float2 *part, int k0, unsigned nb, FF (&v)[K]) {
  __shared__ FF wp[K][BLOCK / 32];
#pragma unroll
  for (int q = 0; q < K; q++)
    for (int o = 16; o > 0; o >>= 1) v[q] = ff_merge(v[q], ff_shfl_down(v[q], o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < K; q++) wp[q][wid] = v[q];
  __syncthreads();
  if (threadIdx.x < K) {
    FF t = wp[threadIdx.x][0];
    for (int i = 1; i < BLOCK / 32; i++) t = ff_merge(t, wp[threadIdx.x][i]);
    part[(size_t)(k0 + threadIdx.x) * nb + blockIdx.x] = make_float2(t.hi, t.lo);
  }
}

/* Sums over the nb block partials of slots k0..k0+K-1, by warp 0 (lane-
 * strided merges, then a shuffle tree: the same order in every block);
 * valid in thread 0. Each lane issues its loads for up to 32 x PL blocks
 * before the first merge: one L2 round trip instead of one per 32 blocks. */
template <int K>
__device__ __forceinline__ void warp_sum_partials(const float2 *part, int k0, unsigned nb,
                                                  double (&out)[K]) {
  constexpr int PL = 10;
  const int lane = threadIdx.x & 31;
  FF v[K];
#pragma unroll
  for (int q = 0; q < K; q++) v[q] = ff_zero();
  for (unsigned base = 0; base < nb; base += 32 * PL) {
    float2 buf[K][PL];
#pragma unroll
    for (int t = 0; t < PL; t++) {
      const unsigned i = base + lane + 32 * t;
#pragma unroll
      for (int q = 0; q < K; q++)
        buf[q][t] = i < nb ? __ldcg(part + (size_t)(k0 + q) * nb + i) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int t = 0; t < PL; t++)
      if (base + lane + 32 * t < nb)
#pragma unroll
        for (int q = 0; q < K; q++) v[q] = ff_merge(v[q], FF{buf[q][t].x, buf[q][t].y});
  }
#pragma unroll
  for (int q = 0; q < K; q++) {
    for (int o = 16; o > 0; o >>= 1) v[q] = ff_merge(v[q], ff_shfl_down(v[q], o));
    out[q] = ff_to_double(v[q]);
  }
}

/* FAST-mode Jacobi PCG with one grid-wide reduction per iteration
 * (Chronopoulos-Gear): with u = M^-1 r and w = A u,
 *   p = u + beta p,  s = w + beta s  (s = A p),  x += alpha p,  r -= alpha s,
 *   gamma = r.u, delta = w.u,  beta' = gamma'/gamma,
 *   alpha' = gamma' / (delta' - beta' gamma' / alpha).
 * The vectors are kept scaled by the Jacobi preconditioner M^-1 = 1/diag:
 * U = M^-1 r (= u), Wt = M^-1 w, St = M^-1 s. The new w = A u' needs
 * u' = U - alpha (Wt + beta St) at the neighbours, which every thread
 * recomputes from the previous iteration's U, Wt, St (ping-pong buffers), so
 * one sweep and one barrier make an iteration and a neighbour quad costs
 * three float4 loads and its flags. The residual of the dot products is
 * r = diag U. Quads of 4 k-cells per thread; partial sums alternate between
 * two slot sets so that a slow reader of one iteration's sums never sees
 * the next iteration's. */
struct Cg1Q {
  uchar4 A;
  float4 u, w, s;
};

/* The 32-quad chunks of the single-reduction CG that hold liquid, in
 * increasing order (flags by one warp per chunk, an exclusive scan, a
 * scatter): the CG sweeps visit only these. */
__global__ void __launch_bounds__(BLK) k_cg1_chunk_flags(size_t nq, const uchar4 *__restrict__ A4,
                                                        unsigned *__restrict__ flag) {
  const size_t chunk = ((size_t)blockIdx.x * BLK + threadIdx.x) >> 5;
  const size_t nch = (nq + 31) / 32;
  if (chunk > nch) return; /* whole warps */
  const int lane = threadIdx.x & 31;
  const size_t q = chunk * 32 + lane;
  bool f = false;
  if (chunk < nch && q < nq) {
    const uchar4 v = A4[q];
    f = fl(v.x) || fl(v.y) || fl(v.z) || fl(v.w);
  }
  const unsigned any = __ballot_sync(0xffffffffu, f);
  if (lane == 0) flag[chunk] = (chunk < nch && any) ? 1u : 0u; /* flag[nch] = 0 */
}

__global__ void __launch_bounds__(BLK) k_cg1_chunk_scatter(size_t nch, const unsigned *__restrict__ off,
                                                          unsigned *__restrict__ list) {
  const size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  if (c < nch && off[c + 1] != off[c]) list[off[c]] = (unsigned)c;
}

template <int BLOCK> __global__ void __launch_bounds__(BLOCK, 1) k_cg_cg1(CgArgs a) {
  if (ir_skipped(a)) return;
  const unsigned nb = gridDim.x;
  const int n = a.s.n;
  const int qrow = n / 4;
  const size_t qplane = (size_t)qrow * n;
  const size_t nq = a.nc / 4;
  const size_t warps = (size_t)nb * (BLOCK / 32);
  const size_t wid = (size_t)blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  float4 *x4 = reinterpret_cast<float4 *>(a.x);
  float4 *p4 = reinterpret_cast<float4 *>(a.p);
  const float4 *b4 = reinterpret_cast<const float4 *>(a.b);
  const float4 *pf4 = reinterpret_cast<const float4 *>(a.Pf);
  const float4 *d4p = reinterpret_cast<const float4 *>(a.diag);
  const uchar4 *A4p = reinterpret_cast<const uchar4 *>(a.A);
  float *R[2] = {a.r, a.z}, *W[2] = {a.w, a.w1}, *S[2] = {a.s0, a.s1};
  /* quad index -> (i, j, k/4) in 32-bit arithmetic (nq < 2^31 on this path) */
  auto decode_q = [&](size_t q, int &i, int &j, int &kq) {
    const unsigned q32 = (unsigned)q, row = q32 / (unsigned)qrow;
    kq = (int)(q32 - row * (unsigned)qrow);
    i = (int)(row / (unsigned)n);
    j = (int)(row - (unsigned)i * (unsigned)n);
  };
  const float hs = a.s.inv_h2_f;
  unsigned epoch = 0; /* barriers passed (count_barrier) */

  /* phase 0a: r = b - A x on the liquid, U = M^-1 r; b.b, r.r, gamma = r.U */
  FF pbb = ff_zero(), prr = ff_zero(), pg0 = ff_zero();
  for (size_t base = wid * 32; base < nq; base += warps * 32) {
    size_t q = base + lane;
    bool valid = q < nq;
    int i = 0, j = 0, kq = 0;
    if (valid) decode_q(q, i, j, kq);
    float4 xs, ax;
    uchar4 A4;
    quad_matvec(a, valid ? q : 0, valid, qrow, qplane, i, j, kq, a.x, a.x, 0.0f, true, xs, ax, A4);
    if (!valid) continue;
    const float4 bv = b4[q], pf = pf4[q];
    const bool fv[4] = {fl(A4.x), fl(A4.y), fl(A4.z), fl(A4.w)};
    const float bb[4] = {bv.x, bv.y, bv.z, bv.w}, av[4] = {ax.x, ax.y, ax.z, ax.w};
    const float pfv[4] = {pf.x, pf.y, pf.z, pf.w};
    const float4 xo = x4[q];
    const float xov[4] = {xo.x, xo.y, xo.z, xo.w};
    float uv[4], xv[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      if (fv[t]) {
        ff_add_prod(pbb, bb[t], bb[t]);
        const float rv = bb[t] - av[t];
        ff_add_prod(prr, rv, rv);
        uv[t] = pfv[t] * rv;
        ff_add_prod(pg0, rv, uv[t]);
        xv[t] = xov[t];
      } else {
        uv[t] = xv[t] = 0.0f;
      }
    }
    reinterpret_cast<float4 *>(R[0])[q] = make_float4(uv[0], uv[1], uv[2], uv[3]);
    x4[q] = make_float4(xv[0], xv[1], xv[2], xv[3]);
  }
  __shared__ float s_alpha, s_beta;
  __shared__ int s_done;
  {
    FF v[3] = {pbb, prr, pg0};
    store_partials<3, BLOCK>(a.part, 0, nb, v);
  }
  if (!count_barrier(a.bar, epoch, a.iflags)) return;
  /* the FP64 scalar work runs on thread 0 of each block (the sums are the
   * same in every block) and reaches the others through shared memory */
  double b2 = 0.0, eps = 0.0, e2 = 0.0, gamma = 0.0;
  int done = 0, iters = 0;
  if (threadIdx.x < 32) {
    double t[3];
    warp_sum_partials<3>(a.part, 0, nb, t);
    if (threadIdx.x == 0) {
      b2 = t[0];
      e2 = t[1];
      gamma = t[2];
      const double rt = cg_rel_tol(a);
      eps = rt * rt * b2;
      s_done = e2 <= eps ? 1 : 0;
    }
  }
  __syncthreads();
  done = s_done;

  /* the sweep: for the liquid chunks of this warp (32 quads each, from the
   * chunk list), from U/Wt/St[cur] (and the directions) at step
   * (alpha, beta, first) to U/Wt/St[cur^1]; init: only Wt = M^-1 A U
   * (alpha = 0, no s, no updates). Every load of a chunk (its own quad, the
   * four i/j neighbour quads, the k neighbour cell of the edge lanes) is
   * issued before the first use, so a chunk costs one L2 round trip; no load
   * waits on a cell flag (air values are loaded and then ignored). */
  const unsigned nact = __ldcg(a.chunk_count);
  auto sweep = [&](int cur, float alpha, float beta, auto first_c, auto init_c, FF &pg, FF &pd,
                   FF &pr) {
    constexpr bool first = decltype(first_c)::value, init = decltype(init_c)::value;
    const float *Uo = R[cur], *Wo = W[cur], *So = S[cur];
    float *Un = R[cur ^ 1], *Wn = W[cur ^ 1], *Sn = S[cur ^ 1];
    const float4 zero = make_float4(0, 0, 0, 0);
    auto load_q = [&](Cg1Q &v, size_t qq) {
      v.A = A4p[qq];
      v.u = __ldcg(reinterpret_cast<const float4 *>(Uo) + qq);
      v.w = init ? zero : __ldcg(reinterpret_cast<const float4 *>(Wo) + qq);
      v.s = (init || first) ? zero : __ldcg(reinterpret_cast<const float4 *>(So) + qq);
    };
    /* u' = U - alpha (Wt + beta St) on the liquid, 0 elsewhere */
    auto u1 = [&](unsigned char f, float u, float w, float s) {
      if (!fl(f)) return 0.0f;
      if (init) return u;
      return u - alpha * (first ? w : w + beta * s);
    };
    auto u_of = [&](const Cg1Q &v) {
      return make_float4(u1(v.A.x, v.u.x, v.w.x, v.s.x), u1(v.A.y, v.u.y, v.w.y, v.s.y),
                         u1(v.A.z, v.u.z, v.w.z, v.s.z), u1(v.A.w, v.u.w, v.w.w, v.s.w));
    };
    unsigned cnext = wid < nact ? __ldg(a.chunk_list + wid) : 0u;
    for (size_t t = wid; t < nact; t += warps) {
      const size_t q = (size_t)cnext * 32 + lane;
      if (t + warps < nact) cnext = __ldg(a.chunk_list + t + warps); /* next chunk, early */
      const bool valid = q < nq;
      const size_t qs = valid ? q : 0;
      int i = 0, j = 0, kq = 0;
      decode_q(qs, i, j, kq);
      const size_t c0 = 4 * qs;
      const int k0 = 4 * kq;
      /* own quad */
      Cg1Q own;
      load_q(own, qs);
      const float4 dg = __ldg(d4p + qs), pf = __ldg(pf4 + qs);
      const float4 po = (init || first) ? zero : p4[qs];
      const float4 xo = init ? zero : __ldcg(x4 + qs); /* phase 0a wrote x by another map */
      /* i/j neighbour quads */
      const bool has[4] = {i + 1 < n, i > 0, j + 1 < n, j > 0};
      const long off[4] = {(long)qplane, -(long)qplane, (long)qrow, -(long)qrow};
      Cg1Q nbq[4];
#pragma unroll
      for (int d = 0; d < 4; d++) {
        if (has[d]) {
          load_q(nbq[d], (size_t)((long)qs + off[d]));
        } else {
          nbq[d].A = make_uchar4(0, 0, 0, 0);
          nbq[d].u = nbq[d].w = nbq[d].s = zero;
        }
      }
      /* the k neighbour across the chunk's ends: cell c0-1 for lane 0, c0+4
       * for lane 31 (inside the chunk the shuffles below carry it) */
      const bool edge = (lane == 0 && k0 > 0) || (lane == 31 && k0 + 4 < n);
      const size_t ce = lane == 0 ? c0 - 1 : c0 + 4;
      unsigned char eA = 0;
      float eu0 = 0.0f, ew = 0.0f, es = 0.0f;
      if (edge) {
        eA = a.A[ce];
        eu0 = __ldcg(Uo + ce);
        if (!init) {
          ew = __ldcg(Wo + ce);
          if (!first) es = __ldcg(So + ce);
        }
      }
      const uchar4 A4 = own.A;
      const float4 un = u_of(own);
      const bool any = fl(A4.x) || fl(A4.y) || fl(A4.z) || fl(A4.w);
      /* k neighbours across quads */
      float left = __shfl_up_sync(FULL, un.w, 1);
      int left_fl = __shfl_up_sync(FULL, (int)fl(A4.w), 1);
      float right = __shfl_down_sync(FULL, un.x, 1);
      int right_fl = __shfl_down_sync(FULL, (int)fl(A4.x), 1);
      if (!valid || !any) continue;
      const float eu = edge ? u1(eA, eu0, ew, es) : 0.0f;
      if (k0 == 0) {
        left_fl = 0;
      } else if (lane == 0) {
        left = eu;
        left_fl = fl(eA);
      }
      if (k0 + 4 >= n) {
        right_fl = 0;
      } else if (lane == 31) {
        right = eu;
        right_fl = fl(eA);
      }
      float acc[4] = {dg.x * un.x, dg.y * un.y, dg.z * un.z, dg.w * un.w};
#pragma unroll
      for (int d = 0; d < 4; d++) {
        const float4 v = u_of(nbq[d]);
        acc[0] -= v.x;
        acc[1] -= v.y;
        acc[2] -= v.z;
        acc[3] -= v.w;
      }
      const bool fv[4] = {fl(A4.x), fl(A4.y), fl(A4.z), fl(A4.w)};
      const float uv[4] = {un.x, un.y, un.z, un.w};
      acc[0] -= (fv[1] ? uv[1] : 0.0f) + (left_fl ? left : 0.0f);
      acc[1] -= (fv[0] ? uv[0] : 0.0f) + (fv[2] ? uv[2] : 0.0f);
      acc[2] -= (fv[1] ? uv[1] : 0.0f) + (fv[3] ? uv[3] : 0.0f);
      acc[3] -= (fv[2] ? uv[2] : 0.0f) + (right_fl ? right : 0.0f);
      const float PF[4] = {pf.x, pf.y, pf.z, pf.w}, DG[4] = {dg.x, dg.y, dg.z, dg.w};
      float wn[4], wt[4];
#pragma unroll
      for (int t2 = 0; t2 < 4; t2++) {
        wn[t2] = fv[t2] ? acc[t2] * hs : 0.0f;
        wt[t2] = PF[t2] * wn[t2];
      }
      reinterpret_cast<float4 *>(Wn)[q] = make_float4(wt[0], wt[1], wt[2], wt[3]);
      if (init) {
#pragma unroll
        for (int t2 = 0; t2 < 4; t2++)
          if (fv[t2]) ff_add_prod(pd, wn[t2], uv[t2]);
        /* U[cur^1] mirrors U[cur] so the first sweep reads the same U */
        reinterpret_cast<float4 *>(Un)[q] = own.u;
        continue;
      }
      /* own updates: p, St, x, U (= u') */
      const float Uv[4] = {own.u.x, own.u.y, own.u.z, own.u.w};
      const float Wv[4] = {own.w.x, own.w.y, own.w.z, own.w.w};
      const float Sv[4] = {own.s.x, own.s.y, own.s.z, own.s.w};
      const float Pv[4] = {po.x, po.y, po.z, po.w}, Xv[4] = {xo.x, xo.y, xo.z, xo.w};
      float pn[4], stn[4], xn[4];
#pragma unroll
      for (int t2 = 0; t2 < 4; t2++) {
        if (fv[t2]) {
          pn[t2] = first ? Uv[t2] : Uv[t2] + beta * Pv[t2];
          stn[t2] = first ? Wv[t2] : Wv[t2] + beta * Sv[t2];
          xn[t2] = Xv[t2] + alpha * pn[t2];
          const float rn = DG[t2] * uv[t2]; /* r' = diag u' */
          ff_add_prod(pg, rn, uv[t2]);
          ff_add_prod(pd, wn[t2], uv[t2]);
          ff_add_prod(pr, rn, rn);
        } else {
          pn[t2] = stn[t2] = xn[t2] = 0.0f;
        }
      }
      p4[q] = make_float4(pn[0], pn[1], pn[2], pn[3]);
      x4[q] = make_float4(xn[0], xn[1], xn[2], xn[3]);
      reinterpret_cast<float4 *>(Sn)[q] = make_float4(stn[0], stn[1], stn[2], stn[3]);
      reinterpret_cast<float4 *>(Un)[q] = un;
    }
  };

  /* phase 0b: Wt0 = M^-1 A U0 (into W[1]); delta0 = w.u */
  {
    FF pg = ff_zero(), pd = ff_zero(), pr = ff_zero();
    sweep(0, 0.0f, 0.0f, std::true_type{}, std::true_type{}, pg, pd, pr);
    FF v[1] = {pd};
    store_partials<1, BLOCK>(a.part, 3, nb, v);
  }
  if (!count_barrier(a.bar, epoch, a.iflags)) return;
  double alpha = 0.0, beta = 0.0;
  if (threadIdx.x < 32) {
    double t[1];
    warp_sum_partials<1>(a.part, 3, nb, t);
    if (threadIdx.x == 0) {
      alpha = gamma / t[0];
      if (!(alpha == alpha) || !(t[0] > 0.0)) done = done ? done : 2;
      s_alpha = (float)alpha;
      s_done = done;
    }
  }
  __syncthreads();
  float alpha_f = s_alpha, beta_f = 0.0f;
  done = s_done;
  int cur = 1; /* U[1] = U0, W[1] = Wt0 */
  bool first = true;
  int set = 0;
  while (!done) {
    FF v[3] = {ff_zero(), ff_zero(), ff_zero()};
    if (first)
      sweep(cur, alpha_f, beta_f, std::true_type{}, std::false_type{}, v[0], v[1], v[2]);
    else
      sweep(cur, alpha_f, beta_f, std::false_type{}, std::false_type{}, v[0], v[1], v[2]);
    const int k0 = set ? 3 : 0;
    store_partials<3, BLOCK>(a.part, k0, nb, v);
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    set ^= 1;
    cur ^= 1;
    first = false;
    iters++;
    if (threadIdx.x < 32) {
      double t[3];
      warp_sum_partials<3>(a.part, k0, nb, t);
      if (threadIdx.x == 0) {
        const double gn = t[0], dn = t[1];
        e2 = t[2];
        if (e2 <= eps) done = 1;
        else if (!(e2 == e2)) done = 2;
        else if (iters >= a.max_iters) done = 3;
        const double bnext = gn / gamma;
        const double den = dn - bnext * gn / alpha;
        alpha = gn / den;
        beta = bnext;
        gamma = gn;
        if (!done && !(alpha == alpha && den > 0.0)) done = 2;
        s_alpha = (float)alpha;
        s_beta = (float)beta;
        s_done = done;
      }
    }
    __syncthreads();
    alpha_f = s_alpha;
    beta_f = s_beta;
    done = s_done;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iflags[IF_DONE] = done;
    a.iflags[IF_ITERS] = iters;
    a.iflags[IF_NAN] = done == 2;
    a.scal[SC_ERR2] = e2;
    a.scal[SC_B2] = b2;
    a.scal[SC_EPS] = eps;
  }
}

/* ------------------------------------------ multigrid-preconditioned CG */

/* MG-PCG (FAST mode, n % 4 == 0): PCG whose preconditioner is one symmetric
 * V-cycle of geometric multigrid, the structure of McAdams, Sifakis and
 * Teran ("A parallel multigrid Poisson solver for fluids simulation on large
 * grids", SCA 2010):
 *   - smoothing: red-black Gauss-Seidel, nu red-then-black sweeps before
 *     the coarse correction and as many black-then-red sweeps after it
 *     (red: i+j+k even), starting from a zero correction;
 *   - restriction: the average of the 8 children's residuals; prolongation:
 *     the coarse correction added to its 8 children;
 *   - coarser operators: the 7-point Laplacian rediscretised on the
 *     coarsened flags (a coarse cell is liquid if a child is, else air if a
 *     child is, else wall; air is a zero Dirichlet value, wall a zero flux);
 *   - the coarsest level (at most 4^3 cells): coarse_sweeps red-black
 *     sweeps, then as many black-red ones.
 * Every count is fixed and the post-smoothing mirrors the pre-smoothing, so
 * the V-cycle is a fixed symmetric operator, as PCG needs. One persistent
 * cooperative launch per solve: level 0 runs on quads over the liquid
 * chunks, the middle levels on cells grid-wide, and the levels of at most
 * 16^3 cells inside block 0's shared memory; counting barriers separate the
 * phases. x is 0 off the liquid on every level, so neighbour sums need no
 * flags. */
constexpr int MGU = 4;            /* cells per thread and round, loads first */
constexpr unsigned MG_BLOCK_CELLS = 4096; /* levels this small run in block 0 */

template <bool GLOBAL> __device__ __forceinline__ float mg_ld(const float *p) {
  if (GLOBAL) return __ldcg(p);
  return *p;
}

__device__ __forceinline__ void mg_decode(unsigned c, unsigned m, int &i, int &j, int &k) {
  const unsigned row = c / m;
  k = (int)(c - row * m);
  i = (int)(row / m);
  j = (int)(row - (unsigned)i * m);
}

/* the same with shifts when m = 2^lg (lg >= 0) */
__device__ __forceinline__ void mg_decode(unsigned c, unsigned m, int lg, int &i, int &j,
                                          int &k) {
  if (lg >= 0) {
    k = (int)(c & (m - 1));
    j = (int)((c >> lg) & (m - 1));
    i = (int)(c >> (2 * lg));
  } else {
    mg_decode(c, m, i, j, k);
  }
}

template <bool GLOBAL>
__device__ __forceinline__ float mg_nbsum(const float *x, int m, int i, int j, int k, unsigned c) {
  const unsigned mm = (unsigned)m * m;
  float s = 0.0f;
  if (i > 0) s += mg_ld<GLOBAL>(x + c - mm);
  if (i + 1 < m) s += mg_ld<GLOBAL>(x + c + mm);
  if (j > 0) s += mg_ld<GLOBAL>(x + c - m);
  if (j + 1 < m) s += mg_ld<GLOBAL>(x + c + m);
  if (k > 0) s += mg_ld<GLOBAL>(x + c - 1);
  if (k + 1 < m) s += mg_ld<GLOBAL>(x + c + 1);
  return s;
}

/* red-black half sweep: liquid cells of `color` take
 * x = (b / hs + sum of the neighbours' x) / diag */
template <bool GLOBAL>
__device__ void mg_gs(const MgLevel &L, int color, unsigned start, unsigned stride) {
  const unsigned m = (unsigned)L.m, tot = m * m * m;
  if (L.lgm >= 1) {
    /* m = 2^lg: enumerate the cells of the colour only (k = 2 kk + parity) */
    const int lg = L.lgm;
    const unsigned half = tot >> 1, hm = m >> 1;
    for (unsigned h0 = start; h0 < half; h0 += stride * MGU) {
      float nbs[MGU], bv[MGU], dv[MGU];
      unsigned cc[MGU];
      bool upd[MGU];
#pragma unroll
      for (int u = 0; u < MGU; u++) {
        const unsigned h = h0 + (unsigned)u * stride;
        upd[u] = false;
        nbs[u] = bv[u] = 0.0f;
        dv[u] = 1.0f;
        cc[u] = 0;
        if (h < half) {
          const unsigned row = h >> (lg - 1);
          const int j = (int)(row & (m - 1)), i = (int)(row >> lg);
          const int k = 2 * (int)(h & (hm - 1)) + ((i + j + color) & 1);
          const unsigned c = (row << lg) + (unsigned)k;
          cc[u] = c;
          upd[u] = L.flags[c] == CELL_FLUID;
          bv[u] = mg_ld<GLOBAL>(L.b + c);
          dv[u] = L.diag[c];
          nbs[u] = mg_nbsum<GLOBAL>(L.x, (int)m, i, j, k, c);
        }
      }
#pragma unroll
      for (int u = 0; u < MGU; u++)
        if (upd[u]) L.x[cc[u]] = __fdividef(bv[u] * L.ihs + nbs[u], dv[u]);
    }
    return;
  }
  for (unsigned c0 = start; c0 < tot; c0 += stride * MGU) {
    float nbs[MGU], bv[MGU], dv[MGU];
    bool upd[MGU];
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      upd[u] = false;
      nbs[u] = bv[u] = 0.0f;
      dv[u] = 1.0f;
      if (c < tot) {
        int i, j, k;
        mg_decode(c, m, L.lgm, i, j, k);
        if (((i + j + k) & 1) == color) {
          upd[u] = L.flags[c] == CELL_FLUID;
          bv[u] = mg_ld<GLOBAL>(L.b + c);
          dv[u] = L.diag[c];
          nbs[u] = mg_nbsum<GLOBAL>(L.x, (int)m, i, j, k, c);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < MGU; u++)
      if (upd[u]) L.x[c0 + (unsigned)u * stride] = __fdividef(bv[u] * L.ihs + nbs[u], dv[u]);
  }
}

/* res = b - A x on the liquid, 0 elsewhere */
template <bool GLOBAL>
__device__ void mg_residual(const MgLevel &L, unsigned start, unsigned stride) {
  const unsigned m = (unsigned)L.m, tot = m * m * m;
  for (unsigned c0 = start; c0 < tot; c0 += stride * MGU) {
    float nbs[MGU], bv[MGU], dv[MGU], xv[MGU];
    bool fl_[MGU];
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      fl_[u] = false;
      nbs[u] = bv[u] = dv[u] = xv[u] = 0.0f;
      if (c < tot) {
        int i, j, k;
        mg_decode(c, m, L.lgm, i, j, k);
        fl_[u] = L.flags[c] == CELL_FLUID;
        bv[u] = mg_ld<GLOBAL>(L.b + c);
        dv[u] = L.diag[c];
        xv[u] = mg_ld<GLOBAL>(L.x + c);
        nbs[u] = mg_nbsum<GLOBAL>(L.x, (int)m, i, j, k, c);
      }
    }
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      if (c < tot) L.res[c] = fl_[u] ? bv[u] - L.hs * (dv[u] * xv[u] - nbs[u]) : 0.0f;
    }
  }
}

/* coarse b = mean of the 8 children's residuals; coarse x = its first red
 * half sweep from zero (b / (hs diag) on red liquid cells, 0 elsewhere) */
template <bool GF, bool GC>
__device__ void mg_restrict(const MgLevel &F, const MgLevel &Cl, unsigned start, unsigned stride) {
  const unsigned mc = (unsigned)Cl.m, totc = mc * mc * mc, mf = (unsigned)F.m;
  for (unsigned c0 = start; c0 < totc; c0 += stride * MGU) {
    float sum[MGU];
    bool red[MGU], fl_[MGU];
    float dv[MGU];
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      sum[u] = 0.0f;
      red[u] = fl_[u] = false;
      dv[u] = 1.0f;
      if (c < totc) {
        int I, J, K;
        mg_decode(c, mc, Cl.lgm, I, J, K);
        red[u] = ((I + J + K) & 1) == 0;
        fl_[u] = Cl.flags[c] == CELL_FLUID;
        dv[u] = Cl.diag[c];
        if ((mf & 1u) == 0) { /* the k pair as one aligned float2 */
#pragma unroll
          for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++) {
              const unsigned i = 2u * I + a, j = 2u * J + b;
              const float2 *pp =
                  reinterpret_cast<const float2 *>(F.res + (i * mf + j) * mf + 2u * K);
              const float2 v = GF ? __ldcg(pp) : *pp;
              sum[u] += v.x;
              sum[u] += v.y;
            }
        } else {
#pragma unroll
          for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
              for (int d = 0; d < 2; d++) {
                const unsigned i = 2u * I + a, j = 2u * J + b, k = 2u * K + d;
                if (i < mf && j < mf && k < mf)
                  sum[u] += mg_ld<GF>(F.res + (i * mf + j) * mf + k);
              }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      if (c >= totc) continue;
      const float bc = sum[u] * 0.125f;
      Cl.b[c] = bc;
      Cl.x[c] = (red[u] && fl_[u]) ? __fdividef(bc * Cl.ihs, dv[u]) : 0.0f;
    }
  }
}

/* x += the parent's correction on the liquid */
template <bool GF, bool GC>
__device__ void mg_prolong(const MgLevel &F, const MgLevel &Cl, unsigned start, unsigned stride) {
  const unsigned mf = (unsigned)F.m, tot = mf * mf * mf, mc = (unsigned)Cl.m;
  for (unsigned c0 = start; c0 < tot; c0 += stride * MGU) {
    float xv[MGU], ev[MGU];
    bool fl_[MGU];
#pragma unroll
    for (int u = 0; u < MGU; u++) {
      const unsigned c = c0 + (unsigned)u * stride;
      fl_[u] = false;
      xv[u] = ev[u] = 0.0f;
      if (c < tot) {
        int i, j, k;
        mg_decode(c, mf, F.lgm, i, j, k);
        const unsigned pc =
            (((unsigned)i >> 1) * mc + ((unsigned)j >> 1)) * mc + ((unsigned)k >> 1);
        fl_[u] = F.flags[c] == CELL_FLUID;
        xv[u] = mg_ld<GF>(F.x + c);
        ev[u] = mg_ld<GC>(Cl.x + pc);
      }
    }
#pragma unroll
    for (int u = 0; u < MGU; u++)
      if (fl_[u]) F.x[c0 + (unsigned)u * stride] = xv[u] + ev[u];
  }
}

/* The levels lb.. in block 0's shared memory: V-cycle from level lb's b and
 * first half sweep (in global memory, from the restriction) to level lb's
 * corrected x (written back to global memory). */
__device__ void mg_block_levels(const MgArgs &mg, MgLevel *sl) {
  const unsigned t = threadIdx.x, S = blockDim.x;
  const int lb = mg.lb, last = mg.nlev - 1;
  const MgLevel &G = mg.lv[lb];
  const unsigned m0 = (unsigned)G.m, tot0 = m0 * m0 * m0;
  for (unsigned c0 = t; c0 < tot0; c0 += S * 8) {
    float bv[8], xv[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const unsigned c = c0 + (unsigned)u * S;
      bv[u] = c < tot0 ? __ldcg(G.b + c) : 0.0f;
      xv[u] = c < tot0 ? __ldcg(G.x + c) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const unsigned c = c0 + (unsigned)u * S;
      if (c < tot0) {
        sl[lb].b[c] = bv[u];
        sl[lb].x[c] = xv[u];
      }
    }
  }
  __syncthreads();
  for (int l = lb; l < last; l++) {
    mg_gs<false>(sl[l], 1, t, S);
    __syncthreads();
    for (int sw = 1; sw < mg.nu; sw++) {
      mg_gs<false>(sl[l], 0, t, S);
      __syncthreads();
      mg_gs<false>(sl[l], 1, t, S);
      __syncthreads();
    }
    mg_residual<false>(sl[l], t, S);
    __syncthreads();
    mg_restrict<false, false>(sl[l], sl[l + 1], t, S);
    __syncthreads();
  }
  /* coarsest: the restriction did the first red half sweep */
  mg_gs<false>(sl[last], 1, t, S);
  __syncthreads();
  for (int it = 1; it < mg.coarse_sweeps; it++) {
    mg_gs<false>(sl[last], 0, t, S);
    __syncthreads();
    mg_gs<false>(sl[last], 1, t, S);
    __syncthreads();
  }
  for (int it = 0; it < mg.coarse_sweeps; it++) {
    mg_gs<false>(sl[last], 1, t, S);
    __syncthreads();
    mg_gs<false>(sl[last], 0, t, S);
    __syncthreads();
  }
  for (int l = last - 1; l >= lb; l--) {
    mg_prolong<false, false>(sl[l], sl[l + 1], t, S);
    __syncthreads();
    for (int sw = 0; sw < mg.nu; sw++) {
      mg_gs<false>(sl[l], 1, t, S);
      __syncthreads();
      mg_gs<false>(sl[l], 0, t, S);
      __syncthreads();
    }
  }
  for (unsigned c = t; c < tot0; c += S) G.x[c] = sl[lb].x[c];
}

/* Shared-memory bytes of block 0's levels (flags, diag, x, b, res). */
__host__ __device__ inline size_t mg_block_bytes(const int *m, int lb, int nlev) {
  size_t b = 0;
  for (int l = lb; l < nlev; l++) {
    const size_t c = (size_t)m[l] * m[l] * m[l];
    b += (c + 15) / 16 * 16 + 4 * 4 * c;
  }
  return b;
}

/* Level-0 phases on quads of the liquid chunks. */
/* MG_BLACK_PROLONG: the black half sweep after the coarse correction, with
 * the prolongation folded in: every value is read as z plus the parent's
 * correction, and only the black cells are written (the red cells keep
 * their uncorrected z, which the neighbours of this phase read and correct
 * themselves; the red half sweep that follows overwrites every red cell). */
enum MgPhase { MG_MATVEC, MG_UPDATE, MG_BLACK, MG_RES, MG_RED_DOT, MG_BLACK_PROLONG, MG_RED };

template <int PH, int BLOCK>
__device__ __forceinline__ void mg_quads(const CgArgs &a, float alpha, float beta, const float *pold,
                                         float *pnew, FF &acc0) {
  const int n = a.s.n, qrow = n / 4;
  const size_t qplane = (size_t)qrow * n, nq = a.nc / 4;
  const size_t warps = (size_t)gridDim.x * (BLOCK / 32);
  const size_t wid = (size_t)blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const MgLevel &L0 = a.mg.lv[0];
  const float hs = L0.hs, ihs = L0.ihs;
  const uchar4 *A4p = reinterpret_cast<const uchar4 *>(a.A);
  const float4 *d4p = reinterpret_cast<const float4 *>(a.diag);
  float *zf = L0.x, *rf = a.r;
  const float4 zero = make_float4(0, 0, 0, 0);
  const unsigned nact = __ldcg(a.chunk_count);
  unsigned cnext = wid < nact ? __ldg(a.chunk_list + wid) : 0u;
  for (size_t t = wid; t < nact; t += warps) {
    const size_t q = (size_t)cnext * 32 + lane;
    if (t + warps < nact) cnext = __ldg(a.chunk_list + t + warps);
    const bool valid = q < nq;
    const size_t qs = valid ? q : 0;
    const unsigned q32 = (unsigned)qs, row = q32 / (unsigned)qrow;
    const int kq = (int)(q32 - row * (unsigned)qrow);
    const int i = (int)(row / (unsigned)n), j = (int)(row - (unsigned)i * (unsigned)n);
    const int k0 = 4 * kq;
    const size_t c0 = 4 * qs;
    const uchar4 A4 = A4p[qs];
    const bool fv[4] = {fl(A4.x), fl(A4.y), fl(A4.z), fl(A4.w)};
    const int par0 = (i + j + k0) & 1; /* colour of the quad's first cell */
    constexpr bool NB = PH == MG_MATVEC || PH == MG_BLACK || PH == MG_RES || PH == MG_RED_DOT ||
                        PH == MG_BLACK_PROLONG || PH == MG_RED;
    /* the field whose neighbours are summed: p' = z + beta p (MATVEC) or z */
    float4 own = zero, own0 = zero; /* own0: as loaded, before any correction */
    float4 nbq[4] = {zero, zero, zero, zero};
    float edge = 0.0f;
    const bool has[4] = {i + 1 < n, i > 0, j + 1 < n, j > 0};
    const long off[4] = {(long)qplane, -(long)qplane, (long)qrow, -(long)qrow};
    const bool ed = (lane == 0 && k0 > 0) || (lane == 31 && k0 + 4 < n);
    const size_t ce = lane == 0 ? c0 - 1 : c0 + 4;
    if (PH == MG_MATVEC) {
      const float4 z4 = __ldcg(reinterpret_cast<const float4 *>(zf) + qs);
      const float4 p4 = __ldcg(reinterpret_cast<const float4 *>(pold) + qs);
      own = make_float4(z4.x + beta * p4.x, z4.y + beta * p4.y, z4.z + beta * p4.z,
                        z4.w + beta * p4.w);
#pragma unroll
      for (int d = 0; d < 4; d++)
        if (has[d]) {
          const size_t qq = (size_t)((long)qs + off[d]);
          const float4 zn = __ldcg(reinterpret_cast<const float4 *>(zf) + qq);
          const float4 pn = __ldcg(reinterpret_cast<const float4 *>(pold) + qq);
          nbq[d] = make_float4(zn.x + beta * pn.x, zn.y + beta * pn.y, zn.z + beta * pn.z,
                               zn.w + beta * pn.w);
        }
      if (ed) edge = __ldcg(zf + ce) + beta * __ldcg(pold + ce);
    } else {
      if (NB) own = __ldcg(reinterpret_cast<const float4 *>(zf) + qs);
      own0 = own;
      if (NB) {
#pragma unroll
        for (int d = 0; d < 4; d++)
          if (has[d])
            nbq[d] = __ldcg(reinterpret_cast<const float4 *>(zf) + (size_t)((long)qs + off[d]));
        if (ed) edge = __ldcg(zf + ce);
      }
      if (PH == MG_BLACK_PROLONG) {
        /* add the parents' corrections on the liquid (level 1 holds them) */
        const MgLevel &L1 = a.mg.lv[1];
        const unsigned m1 = (unsigned)L1.m;
        auto par2 = [&](int ii, int jj) {
          const unsigned idx = (((unsigned)ii >> 1) * m1 + ((unsigned)jj >> 1)) * m1 +
                               (unsigned)(k0 >> 1);
          return __ldcg(reinterpret_cast<const float2 *>(L1.x + idx));
        };
        auto add = [](float4 &v, uchar4 f, float2 e) {
          v.x += fl(f.x) ? e.x : 0.0f;
          v.y += fl(f.y) ? e.x : 0.0f;
          v.z += fl(f.z) ? e.y : 0.0f;
          v.w += fl(f.w) ? e.y : 0.0f;
        };
        const int di[4] = {1, -1, 0, 0}, dj[4] = {0, 0, 1, -1};
        add(own, A4, par2(i, j));
#pragma unroll
        for (int d = 0; d < 4; d++)
          if (has[d]) add(nbq[d], A4p[(size_t)((long)qs + off[d])], par2(i + di[d], j + dj[d]));
        if (ed) {
          const int ke = lane == 0 ? k0 - 1 : k0 + 4;
          const unsigned idx =
              (((unsigned)i >> 1) * m1 + ((unsigned)j >> 1)) * m1 + (unsigned)(ke >> 1);
          if (fl(a.A[ce])) edge += __ldcg(L1.x + idx);
        }
      }
    }
    /* k neighbours across quads */
    float left = __shfl_up_sync(FULL, own.w, 1);
    float right = __shfl_down_sync(FULL, own.x, 1);
    if (k0 == 0) left = 0.0f;
    else if (lane == 0) left = edge;
    if (k0 + 4 >= n) right = 0.0f;
    else if (lane == 31) right = edge;
    if (!valid || !(fv[0] || fv[1] || fv[2] || fv[3])) continue;
    const float ov[4] = {own.x, own.y, own.z, own.w};
    float nbs[4];
    if (NB) {
      const float kl[4] = {left, ov[0], ov[1], ov[2]}, kr[4] = {ov[1], ov[2], ov[3], right};
      const float n0[4] = {nbq[0].x, nbq[0].y, nbq[0].z, nbq[0].w};
      const float n1[4] = {nbq[1].x, nbq[1].y, nbq[1].z, nbq[1].w};
      const float n2[4] = {nbq[2].x, nbq[2].y, nbq[2].z, nbq[2].w};
      const float n3[4] = {nbq[3].x, nbq[3].y, nbq[3].z, nbq[3].w};
#pragma unroll
      for (int u = 0; u < 4; u++) nbs[u] = ((((n0[u] + n1[u]) + n2[u]) + n3[u]) + kl[u]) + kr[u];
    }
    if (PH == MG_MATVEC) {
      const float4 dg = __ldg(d4p + qs);
      const float dv[4] = {dg.x, dg.y, dg.z, dg.w};
      float qv[4], pv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        pv[u] = fv[u] ? ov[u] : 0.0f;
        qv[u] = fv[u] ? hs * (dv[u] * ov[u] - nbs[u]) : 0.0f;
        if (fv[u]) ff_add_prod(acc0, pv[u], qv[u]);
      }
      reinterpret_cast<float4 *>(pnew)[q] = make_float4(pv[0], pv[1], pv[2], pv[3]);
      reinterpret_cast<float4 *>(a.q)[q] = make_float4(qv[0], qv[1], qv[2], qv[3]);
    } else if (PH == MG_UPDATE) {
      /* x += alpha p', r -= alpha q; r.r; z: first red half sweep from 0 */
      const float4 x4 = __ldcg(reinterpret_cast<const float4 *>(a.x) + q);
      const float4 r4 = __ldcg(reinterpret_cast<const float4 *>(rf) + q);
      const float4 p4 = __ldcg(reinterpret_cast<const float4 *>(pnew) + q);
      const float4 q4 = __ldcg(reinterpret_cast<const float4 *>(a.q) + q);
      const float4 dg = __ldg(d4p + qs);
      const float xv[4] = {x4.x, x4.y, x4.z, x4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w};
      const float pv[4] = {p4.x, p4.y, p4.z, p4.w}, qv[4] = {q4.x, q4.y, q4.z, q4.w};
      const float dv[4] = {dg.x, dg.y, dg.z, dg.w};
      float xn[4], rn[4], zn[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (fv[u]) {
          xn[u] = xv[u] + alpha * pv[u];
          rn[u] = rv[u] - alpha * qv[u];
          ff_add_prod(acc0, rn[u], rn[u]);
          zn[u] = ((par0 + u) & 1) == 0 ? __fdividef(rn[u] * ihs, dv[u]) : 0.0f;
        } else {
          xn[u] = xv[u];
          rn[u] = zn[u] = 0.0f;
        }
      }
      reinterpret_cast<float4 *>(a.x)[q] = make_float4(xn[0], xn[1], xn[2], xn[3]);
      reinterpret_cast<float4 *>(rf)[q] = make_float4(rn[0], rn[1], rn[2], rn[3]);
      reinterpret_cast<float4 *>(zf)[q] = make_float4(zn[0], zn[1], zn[2], zn[3]);
    } else if (PH == MG_RES) {
      const float4 r4 = __ldcg(reinterpret_cast<const float4 *>(rf) + q);
      const float4 dg = __ldg(d4p + qs);
      const float rv[4] = {r4.x, r4.y, r4.z, r4.w}, dv[4] = {dg.x, dg.y, dg.z, dg.w};
      float res[4];
#pragma unroll
      for (int u = 0; u < 4; u++) res[u] = fv[u] ? rv[u] - hs * (dv[u] * ov[u] - nbs[u]) : 0.0f;
      reinterpret_cast<float4 *>(L0.res)[q] = make_float4(res[0], res[1], res[2], res[3]);
    } else { /* MG_BLACK, MG_BLACK_PROLONG, MG_RED, MG_RED_DOT: half sweep of one colour */
      const int color = (PH == MG_RED_DOT || PH == MG_RED) ? 0 : 1;
      const float4 r4 = __ldcg(reinterpret_cast<const float4 *>(rf) + q);
      const float4 dg = __ldg(d4p + qs);
      const float rv[4] = {r4.x, r4.y, r4.z, r4.w}, dv[4] = {dg.x, dg.y, dg.z, dg.w};
      const float o0[4] = {own0.x, own0.y, own0.z, own0.w};
      float zn[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        zn[u] = o0[u];
        if (fv[u] && ((par0 + u) & 1) == color) zn[u] = __fdividef(rv[u] * ihs + nbs[u], dv[u]);
        if (PH == MG_RED_DOT && fv[u]) ff_add_prod(acc0, rv[u], zn[u]);
      }
      reinterpret_cast<float4 *>(zf)[q] = make_float4(zn[0], zn[1], zn[2], zn[3]);
    }
  }
}

template <int BLOCK> __global__ void __launch_bounds__(BLOCK, 1) k_cg_mg(CgArgs a) {
  if (ir_skipped(a)) return;
  const unsigned nb = gridDim.x;
  const int n = a.s.n;
  const int qrow = n / 4;
  const size_t qplane = (size_t)qrow * n;
  const size_t nq = a.nc / 4;
  const size_t warps = (size_t)nb * (BLOCK / 32);
  const size_t wid = (size_t)blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  float4 *x4 = reinterpret_cast<float4 *>(a.x);
  const float4 *b4 = reinterpret_cast<const float4 *>(a.b);
  const MgArgs &mg = a.mg;
  const unsigned gt = blockIdx.x * BLOCK + threadIdx.x, gs = nb * BLOCK;
  unsigned epoch = 0;
  __shared__ float s_alpha, s_beta;
  __shared__ int s_done;
  extern __shared__ __align__(16) unsigned char mg_smem[];

  /* block 0: its levels' flags and diagonals into shared memory (fixed
   * during the solve) */
  MgLevel sl[MG_MAX_LEVELS];
  if (blockIdx.x == 0) {
    unsigned char *pp = mg_smem;
    for (int l = mg.lb; l < mg.nlev; l++) {
      const unsigned m = (unsigned)mg.lv[l].m, c = m * m * m;
      sl[l] = mg.lv[l];
      uint8_t *fl8 = pp;
      pp += (c + 15) / 16 * 16;
      float *dg = reinterpret_cast<float *>(pp);
      sl[l].x = dg + c;
      sl[l].b = dg + 2 * c;
      sl[l].res = dg + 3 * c;
      pp += 4 * 4 * (size_t)c;
      for (unsigned e = threadIdx.x; e < c; e += BLOCK) {
        fl8[e] = mg.lv[l].flags[e];
        dg[e] = mg.lv[l].diag[e];
      }
      sl[l].flags = fl8;
      sl[l].diag = dg;
    }
  }

  /* phase 0: r = b - A x on the liquid (x zeroed elsewhere); b.b, r.r */
  FF pbb = ff_zero(), prr = ff_zero();
  for (size_t base = wid * 32; base < nq; base += warps * 32) {
    size_t q = base + lane;
    bool valid = q < nq;
    int i = 0, j = 0, kq = 0;
    if (valid) {
      const unsigned q32 = (unsigned)q, row = q32 / (unsigned)qrow;
      kq = (int)(q32 - row * (unsigned)qrow);
      i = (int)(row / (unsigned)n);
      j = (int)(row - (unsigned)i * (unsigned)n);
    }
    float4 xs, ax;
    uchar4 A4;
    quad_matvec(a, valid ? q : 0, valid, qrow, qplane, i, j, kq, a.x, a.x, 0.0f, true, xs, ax, A4);
    if (!valid) continue;
    const float4 bv = b4[q];
    const bool fv[4] = {fl(A4.x), fl(A4.y), fl(A4.z), fl(A4.w)};
    const float bb[4] = {bv.x, bv.y, bv.z, bv.w}, av[4] = {ax.x, ax.y, ax.z, ax.w};
    const float4 xo = x4[q];
    const float xov[4] = {xo.x, xo.y, xo.z, xo.w};
    float rv[4], xv[4];
#pragma unroll
    for (int t = 0; t < 4; t++) {
      if (fv[t]) {
        ff_add_prod(pbb, bb[t], bb[t]);
        rv[t] = bb[t] - av[t];
        ff_add_prod(prr, rv[t], rv[t]);
        xv[t] = xov[t];
      } else {
        rv[t] = xv[t] = 0.0f;
      }
    }
    reinterpret_cast<float4 *>(a.r)[q] = make_float4(rv[0], rv[1], rv[2], rv[3]);
    x4[q] = make_float4(xv[0], xv[1], xv[2], xv[3]);
  }
  {
    FF v[2] = {pbb, prr};
    store_partials<2, BLOCK>(a.part, 0, nb, v);
  }
  if (!count_barrier(a.bar, epoch, a.iflags)) return;
  double b2 = 0.0, eps = 0.0, e2 = 0.0, rz = 0.0, alpha = 0.0, beta = 0.0;
  int done = 0, iters = 0;
  if (threadIdx.x < 32) {
    double t[2];
    warp_sum_partials<2>(a.part, 0, nb, t);
    if (threadIdx.x == 0) {
      b2 = t[0];
      e2 = t[1];
      const double rt = cg_rel_tol(a);
      eps = rt * rt * b2;
      s_done = e2 <= eps ? 1 : 0;
    }
  }
  __syncthreads();
  done = s_done;

  /* z = V-cycle(r) after the level-0 first red half sweep (MG_UPDATE);
   * the final red half sweep accumulates r.z */
  auto vcycle_rest = [&](FF &prz) -> bool {
    FF none = ff_zero();
    mg_quads<MG_BLACK, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
    if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    for (int sw = 1; sw < mg.nu; sw++) {
      mg_quads<MG_RED, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      mg_quads<MG_BLACK, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    }
    mg_quads<MG_RES, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
    if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    mg_restrict<true, true>(mg.lv[0], mg.lv[1], gt, gs);
    if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    for (int l = 1; l < mg.lb; l++) {
      mg_gs<true>(mg.lv[l], 1, gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      for (int sw = 1; sw < mg.nu; sw++) {
        mg_gs<true>(mg.lv[l], 0, gt, gs);
        if (!count_barrier(a.bar, epoch, a.iflags)) return false;
        mg_gs<true>(mg.lv[l], 1, gt, gs);
        if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      }
      mg_residual<true>(mg.lv[l], gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      mg_restrict<true, true>(mg.lv[l], mg.lv[l + 1], gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    }
    if (blockIdx.x == 0) mg_block_levels(mg, sl);
    if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    for (int l = mg.lb - 1; l >= 1; l--) {
      mg_prolong<true, true>(mg.lv[l], mg.lv[l + 1], gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      mg_gs<true>(mg.lv[l], 1, gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      mg_gs<true>(mg.lv[l], 0, gt, gs);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      for (int sw = 1; sw < mg.nu; sw++) {
        mg_gs<true>(mg.lv[l], 1, gt, gs);
        if (!count_barrier(a.bar, epoch, a.iflags)) return false;
        mg_gs<true>(mg.lv[l], 0, gt, gs);
        if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      }
    }
    mg_quads<MG_BLACK_PROLONG, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
    if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    for (int sw = 1; sw < mg.nu; sw++) {
      mg_quads<MG_RED, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
      mg_quads<MG_BLACK, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, none);
      if (!count_barrier(a.bar, epoch, a.iflags)) return false;
    }
    mg_quads<MG_RED_DOT, BLOCK>(a, 0.0f, 0.0f, nullptr, nullptr, prz);
    return true;
  };

  float *P[2] = {a.p, a.p2};
  int pc = 0; /* P[pc]: the previous direction (zero before the first) */
  if (!done) {
    FF none = ff_zero(), prz = ff_zero();
    /* with alpha = 0 the update pass only starts the V-cycle (P and q are
     * zero on entry) */
    mg_quads<MG_UPDATE, BLOCK>(a, 0.0f, 0.0f, P[0], P[1], none);
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    if (!vcycle_rest(prz)) return;
    {
      FF v[1] = {prz};
      store_partials<1, BLOCK>(a.part, 2, nb, v);
    }
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    if (threadIdx.x < 32) {
      double t[1];
      warp_sum_partials<1>(a.part, 2, nb, t);
      if (threadIdx.x == 0) {
        rz = t[0];
        if (!(rz == rz) || !(rz > 0.0)) done = 2;
        s_done = done;
      }
    }
    __syncthreads();
    done = s_done;
  }
  float beta_f = 0.0f;
  while (!done) {
    /* p' = z + beta p, q = A p', p'.q */
    FF ppq = ff_zero();
    mg_quads<MG_MATVEC, BLOCK>(a, 0.0f, beta_f, P[pc], P[pc ^ 1], ppq);
    {
      FF v[1] = {ppq};
      store_partials<1, BLOCK>(a.part, 3, nb, v);
    }
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    if (threadIdx.x < 32) {
      double t[1];
      warp_sum_partials<1>(a.part, 3, nb, t);
      if (threadIdx.x == 0) {
        alpha = rz / t[0];
        if (!(alpha == alpha) || !(t[0] > 0.0)) done = 2;
        s_alpha = (float)alpha;
        s_done = done;
      }
    }
    __syncthreads();
    done = s_done;
    if (done) break;
    /* x += alpha p', r -= alpha q, r.r; the V-cycle's first half sweep */
    FF prr2 = ff_zero();
    mg_quads<MG_UPDATE, BLOCK>(a, s_alpha, 0.0f, P[pc], P[pc ^ 1], prr2);
    {
      FF v[1] = {prr2};
      store_partials<1, BLOCK>(a.part, 4, nb, v);
    }
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    iters++;
    if (threadIdx.x < 32) {
      double t[1];
      warp_sum_partials<1>(a.part, 4, nb, t);
      if (threadIdx.x == 0) {
        e2 = t[0];
        if (e2 <= eps) done = 1;
        else if (!(e2 == e2)) done = 2;
        else if (iters >= a.max_iters) done = 3;
        s_done = done;
      }
    }
    __syncthreads();
    done = s_done;
    if (done) break;
    FF prz = ff_zero();
    if (!vcycle_rest(prz)) return;
    {
      FF v[1] = {prz};
      store_partials<1, BLOCK>(a.part, 5, nb, v);
    }
    if (!count_barrier(a.bar, epoch, a.iflags)) return;
    if (threadIdx.x < 32) {
      double t[1];
      warp_sum_partials<1>(a.part, 5, nb, t);
      if (threadIdx.x == 0) {
        const double rzn = t[0];
        beta = rzn / rz;
        rz = rzn;
        if (!(beta == beta)) done = 2;
        s_beta = (float)beta;
        s_done = done;
      }
    }
    __syncthreads();
    beta_f = s_beta;
    done = s_done;
    pc ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iflags[IF_DONE] = done;
    a.iflags[IF_ITERS] = iters;
    a.iflags[IF_NAN] = done == 2;
    a.scal[SC_ERR2] = e2;
    a.scal[SC_B2] = b2;
    a.scal[SC_EPS] = eps;
  }
}

/* coarse flags: liquid if a child is, else air if a child is, else wall */
__global__ void __launch_bounds__(BLK) k_mg_coarsen(const uint8_t *__restrict__ ff, int mf,
                                                    uint8_t *__restrict__ cf, int mc) {
  const unsigned c = blockIdx.x * BLK + threadIdx.x, tot = (unsigned)mc * mc * mc;
  if (c >= tot) return;
  int I, J, K;
  mg_decode(c, (unsigned)mc, I, J, K);
  bool anyf = false, anya = false;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int d = 0; d < 2; d++) {
        const int i = 2 * I + a, j = 2 * J + b, k = 2 * K + d;
        if (i < mf && j < mf && k < mf) {
          const uint8_t f = ff[((size_t)i * mf + j) * mf + k];
          anyf |= f == CELL_FLUID;
          anya |= f == CELL_AIR;
        }
      }
  cf[c] = anyf ? CELL_FLUID : (anya ? CELL_AIR : CELL_WALL);
}

/* coarse diagonal: the liquid cell's neighbours that are not wall (cells
 * outside the grid are wall; at least 1) */
__global__ void __launch_bounds__(BLK) k_mg_diag(const uint8_t *__restrict__ cf, int m,
                                                 float *__restrict__ diag) {
  const unsigned c = blockIdx.x * BLK + threadIdx.x, tot = (unsigned)m * m * m;
  if (c >= tot) return;
  if (cf[c] != CELL_FLUID) {
    diag[c] = 0.0f;
    return;
  }
  int i, j, k;
  mg_decode(c, (unsigned)m, i, j, k);
  const unsigned mm = (unsigned)m * m;
  int d = 0;
  d += i > 0 && cf[c - mm] != CELL_WALL;
  d += i + 1 < m && cf[c + mm] != CELL_WALL;
  d += j > 0 && cf[c - m] != CELL_WALL;
  d += j + 1 < m && cf[c + m] != CELL_WALL;
  d += k > 0 && cf[c - 1] != CELL_WALL;
  d += k + 1 < m && cf[c + 1] != CELL_WALL;
  diag[c] = (float)(d > 0 ? d : 1); /* a liquid cell walled in on all sides */
}

/* ------------------------------------------ IC(0)/MIC(0) as line wavefronts */

/* The lexicographic incomplete-Cholesky factor of the reference's
 * buildPreconditioner (src/solver.cpp:125-139), with the neighbour test on
 * the cell flag instead of the value, plus the MIC(0) modification weighted
 * by tau, and its triangular solves (src/solver.cpp:141-180). Cell (i,j,k)
 * depends on its -x/-y/-z neighbours (factor, forward solve) or its
 * +x/+y/+z neighbours (backward solve), so the cells of a plane i+j+k are
 * independent and a sweep is 3n-2 planes deep.
 *
 * Line wavefront: a warp owns a line, one i and 32 consecutive j (one per
 * lane), and walks k; lane l runs l steps behind lane 0, so at step s it
 * computes k = s - l (mirrored for the backward solve), taking its
 * j-neighbour from lane l-1's previous step (a shuffle) and its k-neighbour
 * from its own previous step. A task is IC_W lines, i = IC_W I .. IC_W I +
 * IC_W - 1 (one warp each) at one 32-j block; warp w takes its i-neighbour
 * from warp w-1 of the task at the same step through a shared-memory ring
 * guarded by mbarriers (full / empty per slot). Tasks go to whole CTAs by an atomic ticket in
 * wavefront order, so every dependency has a smaller ticket and runs.
 * Across tasks, values pass through skewed line buffers of 64-bit words
 * that carry the value and the tag of the sweep that wrote it: the reader
 * polls the word until the tag is its sweep's (bounded), so no flag, fence
 * or barrier sits between a producer and a consumer in different CTAs.
 *
 * Skewed layout: line (i, jb) holds n + 31 rows of 32 words, row s slot l =
 * cell (i, 32 jb + l, s - l), what the line's forward warp touches at step
 * s: every warp step reads or writes one contiguous row, and the backward
 * warp walks the rows in reverse with its lanes reversed. Each warp's reads
 * of its line's rows, of its neighbour lines and of r (natural layout) are
 * issued IC_D steps ahead, IC_G steps at a time, with cp.async (16 bytes,
 * L2 only) into per-warp shared rings.
 *
 * Lines and tasks without liquid are skipped; neighbours treat them as
 * non-liquid. Every cell is computed from the same neighbours in the same
 * order as the sequential sweeps (neighbours i, j, k in that order), so the
 * tiling does not change a value. The preconditioned residual's dot z.r
 * equals q.q for z = L^-T q, q = L^-1 r: it is summed in the forward solve. */
constexpr int IC_BLOCK = 512;         /* threads of the IC kernel: 16 lines per task */
constexpr int IC_W = IC_BLOCK / 32;
constexpr int IC_D = 16;
constexpr int IC_RING = 8;
constexpr int IC_RQ = 32;
constexpr int IC_G = 4;           /* steps per copy group */
constexpr unsigned IC_SPIN_LIMIT = 1u << 22;
constexpr unsigned IC_TAG_WRAP = 0xf0000000u; /* tags left: > 2^28 */
constexpr int IC_MAX_ITERS = 1 << 26;        /* 2^27 + 2 tags per launch at most */
enum { IC_FACTOR = 0, IC_FORWARD = 1, IC_BACKWARD = 2 };

struct IcWarp {
  float pf[IC_D][32];               /* own line: factor rows (solves) */
  union {
    unsigned long long qv[IC_D][32]; /* own line: tagged q rows (backward) */
    float rn[32][IC_RQ];             /* r per lane, natural k order (forward) */
  };
  float2 ring[IC_RING][32];         /* (factor, value) for the next warp's line */
  float jp[IC_D][4];                /* lane 0's j-neighbour: 16-byte factor chunk */
  unsigned long long jv[IC_D][2];   /* ... and its tagged value chunk */
};
struct IcSmem {
  IcWarp w[IC_W];
  float ip[IC_D][32];               /* warp 0's i-neighbour line: factor rows */
  unsigned long long iv[IC_D][32];  /* ... tagged value rows */
  /* ring slot s % IC_RING of warp w: full (written for step s) and empty
   * (read by warp w+1) barriers, 32 arrivals each */
  unsigned long long full[IC_W][IC_RING], empty[IC_W][IC_RING];
  FF part[IC_W];
  unsigned ticket;
  int stop;
};

__device__ __forceinline__ unsigned long long ic_word(float v, unsigned tag) {
  return ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ float ic_val(unsigned long long w) {
  return __uint_as_float((unsigned)w);
}
__device__ __forceinline__ unsigned ic_tagof(unsigned long long w) { return (unsigned)(w >> 32); }

/* The copies are issued without a compiler memory barrier: their shared
 * destinations are read only after cp.async.wait_group (which has one) and
 * a __syncwarp. */
__device__ __forceinline__ void cpa16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;"); }
template <int N> __device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ unsigned long long ld_cg_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.global.cg.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

/* The word at p once it carries `tag` (w: a copy read earlier). Bounded:
 * gives up with FLIPGPU_ETIMEOUT (value 0), or at once when another wait
 * has already timed out. */
__device__ __forceinline__ unsigned long long ic_poll(const unsigned long long *p,
                                                   unsigned long long w, unsigned tag,
                                                   int *iflags) {
  unsigned spins = 0;
  while (ic_tagof(w) != tag) {
    if ((++spins & 255u) == 0 &&
        (spins > IC_SPIN_LIMIT || *(volatile int *)(iflags + IF_TIMEOUT) != 0)) {
      atomicExch(iflags + IF_TIMEOUT, 1);
      return (unsigned long long)tag << 32;
    }
    if (spins > 32) __nanosleep(64);
    w = ld_cg_u64(p);
  }
  return w;
}

/* Shared-memory barriers of the rings between a task's warps. */
__device__ __forceinline__ unsigned icb_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void icb_init(unsigned long long *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(icb_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void icb_inval(unsigned long long *b) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(icb_addr(b)) : "memory");
}
__device__ __forceinline__ void icb_arrive(unsigned long long *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(icb_addr(b)) : "memory");
}
__device__ __forceinline__ bool icb_test(unsigned long long *b, unsigned parity) {
  unsigned done;
  asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
               "selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(done)
               : "r"(icb_addr(b)), "r"(parity)
               : "memory");
  return done != 0;
}
/* Wait for the barrier's phase of this parity: polled (the neighbour warp
 * is usually a step ahead), napping after a while. Bounded: gives up with
 * FLIPGPU_ETIMEOUT, or at once when another wait has already timed out. */
__device__ __forceinline__ void icb_wait(unsigned long long *b, unsigned parity, int *iflags) {
  for (unsigned spin = 0;; spin++) {
    if (icb_test(b, parity)) return;
    if (spin > 64) __nanosleep(32);
    if ((spin & 255u) == 255u &&
        (spin > IC_SPIN_LIMIT || *(volatile int *)(iflags + IF_TIMEOUT) != 0)) {
      atomicExch(iflags + IF_TIMEOUT, 1);
      return;
    }
  }
}

/* One line of a task: the factor (KIND = IC_FACTOR, writes the factor's
 * plain and tagged rows), the forward solve (reads r, writes tagged q and
 * adds q.q to qq) or the backward solve (reads tagged q, writes z in the
 * natural layout and tagged). tag: this sweep's; tagq: the forward solve's
 * (backward only). Every per-step address is a per-lane pointer advanced by
 * a fixed stride; each shared word is read once per step. */
template <int KIND>
__device__ void ic_line(const CgArgs &a, IcSmem &sm, int I, int jb, unsigned tag, unsigned tagq,
                        FF &qq) {
  constexpr bool MIR = KIND == IC_BACKWARD;
  constexpr bool SOLVE = KIND != IC_FACTOR;
  const unsigned FULL = 0xffffffffu;
  const int n = a.s.n, njb = a.ic_njb, sl = n + 31;
  const int lane = threadIdx.x & 31, rho = threadIdx.x >> 5;
  const int i = MIR ? I * IC_W + (IC_W - 1 - rho) : I * IC_W + rho;
  if (i >= n || !__ldg(a.ic_line + (size_t)i * njb + jb)) return;
  IcWarp &ws = sm.w[rho];
  const int J0 = 32 * jb;
  const int j = MIR ? J0 + 31 - lane : J0 + lane;
  const int lf = MIR ? 31 - lane : lane; /* slot in the skewed rows */
  const bool jon = j < n;
  const size_t lsize = (size_t)sl * 32;
  const size_t lbase = ((size_t)i * njb + jb) * lsize;
  /* i-neighbour line: the previous warp's (ring) or another task's (warp 0) */
  const int ip = MIR ? i + 1 : i - 1;
  const bool ipon = ip >= 0 && ip < n && __ldg(a.ic_line + (size_t)ip * njb + jb);
  const bool iglob = rho == 0 && ipon;
  const size_t ibase = ((size_t)(ipon ? ip : 0) * njb + jb) * lsize;
  /* lane 0's j-neighbour: slot 31 (forward) or 0 (backward) of the
   * neighbouring block's line, row s + 31 or n - 1 - s */
  const int jbn = MIR ? jb + 1 : jb - 1, jn = MIR ? J0 + 32 : J0 - 1, jlf = MIR ? 0 : 31;
  const bool jpon = jn >= 0 && jn < n && __ldg(a.ic_line + (size_t)i * njb + jbn);
  const size_t jbase = ((size_t)i * njb + (jpon ? jbn : 0)) * lsize;
  /* the next warp's line takes this line's values through the ring */
  const int inext = MIR ? i - 1 : i + 1;
  const bool cons = rho + 1 < IC_W && inext >= 0 && inext < n &&
                    __ldg(a.ic_line + (size_t)inext * njb + jb);
  const unsigned long long *vsrc =
      KIND == IC_FACTOR ? a.ic_psk : (KIND == IC_FORWARD ? a.ic_qsk : a.ic_zsk);
  unsigned long long *vdst =
      KIND == IC_FACTOR ? a.ic_psk : (KIND == IC_FORWARD ? a.ic_qsk : a.ic_zsk);
  const bool natvec = (n & 3) == 0; /* 16-byte rows of r and z */
  const size_t rowbase = ((size_t)i * n + (jon ? j : 0)) * n;
  const float tau = a.mic_tau;
  /* skewed rows advance by dstep words per step (backward: row n + 30 - s) */
  const long dstep = MIR ? -32 : 32;
  const size_t row0 = MIR ? (size_t)(n + 30) * 32 : 0;

  /* Copies go in groups of IC_G steps: a group's rows of a line are one
   * contiguous block (512 bytes of factor, 1 KB of tagged words), copied by
   * all 32 lanes at once, IC_D steps ahead. Lane l takes 16-byte chunk l
   * (factor) or chunks l and l + 32 (words) of the block; memory row m of a
   * group is step t0 + m (forward) or t0 + 3 - m (backward). */
  constexpr int G = IC_G, GD = IC_D / IC_G;
  const long gstep = MIR ? -32 * G : 32 * G; /* floats or words per group */
  const int mr = lane >> 3, col = 4 * (lane & 7);
  const int ta_of = MIR ? G - 1 - mr : mr;
  const size_t mrow = MIR ? (size_t)(n + 31 - G + mr) * 32 : (size_t)mr * 32;
  const float *pfg = a.ic_pf + lbase + mrow + col;
  const float *ipg = a.ic_pf + ibase + mrow + col;
  const int qc = 2 * (lane & 15), qm0 = lane >> 4, qm1 = qm0 + 2;
  const int tq0 = MIR ? G - 1 - qm0 : qm0, tq1 = MIR ? G - 1 - qm1 : qm1;
  const size_t qrow0 = MIR ? (size_t)(n + 31 - G + qm0) * 32 : (size_t)qm0 * 32;
  const size_t qrow1 = MIR ? (size_t)(n + 31 - G + qm1) * 32 : (size_t)qm1 * 32;
  const unsigned long long *qg0 = a.ic_qsk + lbase + qrow0 + qc;
  const unsigned long long *qg1 = a.ic_qsk + lbase + qrow1 + qc;
  const unsigned long long *ig0 = vsrc + ibase + qrow0 + qc;
  const unsigned long long *ig1 = vsrc + ibase + qrow1 + qc;
  /* lane 0's j-neighbour row at step t: t + 31 (forward) or n - 1 - t */
  const long jstep = MIR ? -32 : 32;
  const size_t jrow0 = MIR ? (size_t)(n - 1) * 32 : (size_t)31 * 32;
  const float *r_row = a.r + rowbase;

  auto prefetch = [&](int g) {
    const int t0 = G * g;
    if (t0 < sl) {
      const long og = (long)g * gstep;
      const int ta = t0 + ta_of, t1 = t0 + tq0, t2 = t0 + tq1;
      if (SOLVE && ta < sl) {
        cpa16(&ws.pf[ta & (IC_D - 1)][col], pfg + og);
        if (iglob) cpa16(&sm.ip[ta & (IC_D - 1)][col], ipg + og);
      }
      if (KIND == IC_BACKWARD) {
        if (t1 < sl) cpa16(&ws.qv[t1 & (IC_D - 1)][qc], qg0 + og);
        if (t2 < sl) cpa16(&ws.qv[t2 & (IC_D - 1)][qc], qg1 + og);
      }
      if (iglob) {
        if (t1 < sl) cpa16(&sm.iv[t1 & (IC_D - 1)][qc], ig0 + og);
        if (t2 < sl) cpa16(&sm.iv[t2 & (IC_D - 1)][qc], ig1 + og);
      }
      if (jpon && lane < 2 * G) {
        const int tj = t0 + (lane & (G - 1));
        if (tj < n) {
          const size_t rj = jbase + jrow0 + (long)tj * jstep;
          if (lane < G) {
            if (SOLVE) cpa16(&ws.jp[tj & (IC_D - 1)][0], a.ic_pf + rj + (jlf & ~3));
          } else {
            cpa16(&ws.jv[tj & (IC_D - 1)][0], vsrc + rj + (jlf & ~1));
          }
        }
      }
      if (KIND == IC_FORWARD && natvec && jon) {
        /* the one chunk of 4 cells whose first cell this lane reaches in
         * the group */
        const int kc = (t0 + G - 1 - lane) & ~3;
        if (kc >= 0 && kc < n) cpa16(&ws.rn[lane][kc & (IC_RQ - 1)], r_row + kc);
      }
    }
    cpa_commit();
  };

#pragma unroll 1
  for (int g = 0; g < GD; g++) prefetch(g);
  float2 last = make_float2(0.0f, 0.0f);
  float4 zq = make_float4(0.0f, 0.0f, 0.0f, 0.0f); /* backward: z of k .. k+3 */
  const IcWarp &wprev = sm.w[rho > 0 ? rho - 1 : 0];
  const int rprev = rho > 0 ? rho - 1 : 0;
  /* this lane's output word and factor at step 0 (valid steps only) */
  unsigned long long *out = vdst + lbase + row0 + lf;
  float *pf_out = a.ic_pf + lbase + row0 + lf;
  const int ngroups = (sl + G - 1) / G;
#pragma unroll 1
  for (int g = 0; g < ngroups; g++) {
    /* the group's copies have landed (issued IC_D steps ago) */
    cpa_wait<GD - 1>();
    __syncwarp();
#pragma unroll
    for (int u = 0; u < G; u++) {
      const int s = G * g + u;
      if (s >= sl) break;
      const int slot = s & (IC_D - 1);
      const int kk = s - lane;
      const bool valid = jon && kk >= 0 && kk < n;
      const int k = MIR ? n - 1 - kk : kk;
      const long os = (long)s * dstep;
      /* i-neighbour at this step */
      float pi = 0.0f, vi = 0.0f;
      if (ipon) {
        if (rho > 0) {
          /* the previous warp's step s; hand the slot back */
          icb_wait(&sm.full[rprev][s & (IC_RING - 1)], (unsigned)(s / IC_RING) & 1u, a.iflags);
          const float2 e = wprev.ring[s & (IC_RING - 1)][lane];
          icb_arrive(&sm.empty[rprev][s & (IC_RING - 1)]);
          pi = e.x;
          vi = e.y;
        } else if (valid) {
          /* a copy taken before its producer wrote it: read it again */
          unsigned long long wi = sm.iv[slot][lf];
          if (ic_tagof(wi) != tag) wi = ic_poll(vsrc + ibase + row0 + os + lf, wi, tag, a.iflags);
          if (KIND == IC_FACTOR) {
            pi = ic_val(wi);
          } else {
            pi = sm.ip[slot][lf];
            vi = ic_val(wi);
          }
        }
      }
      /* j-neighbour: lane l-1's previous step; lane 0: the neighbouring line */
      float pj = __shfl_up_sync(FULL, last.x, 1), vj = __shfl_up_sync(FULL, last.y, 1);
      if (lane == 0) {
        pj = vj = 0.0f;
        if (jpon && valid) {
          unsigned long long wj = ws.jv[slot][jlf & 1];
          if (ic_tagof(wj) != tag)
            wj = ic_poll(vsrc + jbase + jrow0 + (long)s * jstep + jlf, wj, tag, a.iflags);
          if (KIND == IC_FACTOR) {
            pj = ic_val(wj);
          } else {
            pj = ws.jp[slot][jlf & 3];
            vj = ic_val(wj);
          }
        }
      }
      /* k-neighbour: this lane's previous step */
      const float pk = last.x, vk = last.y;
      float p = 0.0f, v = 0.0f;
      if (valid) {
        const size_t c = rowbase + k;
        if (KIND == IC_FACTOR) {
          const unsigned cf = __ldg(a.ic_cf + c);
          if (cf & 1u) {
            const float diag = __ldg(a.diag + c);
            float ev = diag;
            const float pm[3] = {pi, pj, pk};
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
              if (pm[ax] == 0.0f) continue;
              ev -= pm[ax] * pm[ax];
              if (tau != 0.0f) ev -= tau * (float)((cf >> (1 + 2 * ax)) & 3u) * pm[ax] * pm[ax];
            }
            if (ev < 0.25f * diag) ev = diag;
            p = 1.0f / sqrtf(ev);
          }
          pf_out[os] = p;
          out[os] = ic_word(p, tag);
        } else {
          p = ws.pf[slot][lf];
          if (KIND == IC_FORWARD) {
            if (p != 0.0f) {
              float t = natvec ? ws.rn[lane][kk & (IC_RQ - 1)] : __ldcg(a.r + c);
              if (pi != 0.0f) t += pi * vi;
              if (pj != 0.0f) t += pj * vj;
              if (pk != 0.0f) t += pk * vk;
              v = t * p;
              ff_add_prod(qq, v, v);
            }
          } else {
            unsigned long long wq = ws.qv[slot][lf];
            if (ic_tagof(wq) != tagq)
              wq = ic_poll(a.ic_qsk + lbase + row0 + os + lf, wq, tagq, a.iflags);
            if (p != 0.0f) {
              float t = 0.0f;
              if (pi != 0.0f) t += vi;
              if (pj != 0.0f) t += vj;
              if (pk != 0.0f) t += vk;
              v = (ic_val(wq) + p * t) * p;
            }
            if (natvec) {
              zq = make_float4(v, zq.x, zq.y, zq.z);
              if ((k & 3) == 0) *reinterpret_cast<float4 *>(a.z + c) = zq;
            } else {
              a.z[c] = v;
            }
          }
          out[os] = ic_word(v, tag);
        }
      }
      last = valid ? make_float2(p, v) : make_float2(0.0f, 0.0f);
      if (cons) {
        /* the slot's previous value (step s - IC_RING) has been taken */
        if (s >= IC_RING)
          icb_wait(&sm.empty[rho][s & (IC_RING - 1)], (unsigned)(s / IC_RING - 1) & 1u, a.iflags);
        ws.ring[s & (IC_RING - 1)][lane] = last;
        icb_arrive(&sm.full[rho][s & (IC_RING - 1)]);
      }
    }
    /* every lane has read the group's slots: refill them IC_D steps ahead */
    __syncwarp();
    prefetch(g + GD);
  }
  cpa_wait<0>();
  __syncwarp();
}

/* One task: IC_W lines at one 32-j block; the forward solve leaves the
 * task's q.q in ic_part[task]. */
template <int KIND>
__device__ void ic_task(const CgArgs &a, IcSmem &sm, int task, unsigned tag, unsigned tagq) {
  const int I = task / a.ic_njb, jb = task - I * a.ic_njb;
  unsigned long long *bars = &sm.full[0][0];
  constexpr int NB = 2 * IC_W * IC_RING; /* full then empty, contiguous */
  for (int b = threadIdx.x; b < NB; b += IC_BLOCK) icb_init(bars + b, 32);
  __syncthreads();
  FF qq = ff_zero();
  ic_line<KIND>(a, sm, I, jb, tag, tagq, qq);
  if (KIND == IC_FORWARD) {
    for (int o = 16; o > 0; o >>= 1) qq = ff_merge(qq, ff_shfl_down(qq, o));
    if ((threadIdx.x & 31) == 0) sm.part[threadIdx.x >> 5] = qq;
  }
  __syncthreads();
  /* the next task initialises them afresh */
  for (int b = threadIdx.x; b < NB; b += IC_BLOCK) icb_inval(bars + b);
  if (KIND == IC_FORWARD && threadIdx.x == 0) {
    FF t = sm.part[0];
    for (int w = 1; w < IC_W; w++) t = ff_merge(t, sm.part[w]);
    a.ic_part[task] = make_float2(t.hi, t.lo);
  }
}

/* The factor (tasks = ic_tasks) or one preconditioner application, forward
 * then backward (2 ic_tasks), over the ticket counter. */
__device__ void ic_sweeps(const CgArgs &a, IcSmem &sm, bool factor, unsigned tag_f,
                          unsigned tag_b) {
  const unsigned T = (unsigned)a.ic_tasks, tasks = factor ? T : 2u * T;
  while (true) {
    if (threadIdx.x == 0) {
      sm.ticket = atomicAdd(a.ticket, 1u);
      sm.stop = *(volatile int *)(a.iflags + IF_TIMEOUT);
    }
    __syncthreads();
    const unsigned t = sm.ticket;
    const int stop = sm.stop;
    __syncthreads(); /* every thread has the ticket before the next one overwrites it */
    if (t >= tasks || stop) break;
    if (factor)
      ic_task<IC_FACTOR>(a, sm, (int)__ldg(a.ic_order + t), tag_f, 0u);
    else if (t < T)
      ic_task<IC_FORWARD>(a, sm, (int)__ldg(a.ic_order + t), tag_f, 0u);
    else
      ic_task<IC_BACKWARD>(a, sm, (int)__ldg(a.ic_order + (2u * T - 1u - t)), tag_b, tag_f);
  }
}

/* z.r (as q.q) from the per-task partials in task order (identical in every block). */
__device__ __forceinline__ double ic_sum_parts(const CgArgs &a) {
  FF v = ff_zero();
  for (int b = threadIdx.x; b < a.ic_tasks; b += IC_BLOCK) {
    const float2 p = __ldcg(a.ic_part + b);
    v = ff_merge(v, FF{p.x, p.y});
  }
  return ff_to_double(block_sum_ff<IC_BLOCK>(v));
}

/* Per cell: bit 0 liquid; bits 1-2, 3-4, 5-6: how many of the -x, -y, -z
 * neighbour's two other + neighbours are liquid (the MIC(0) terms of the
 * factor); per line (i, 32-j block): whether it holds liquid (ic_line zeroed
 * before). */
__global__ void __launch_bounds__(BLK) k_ic_prep(int n, int njb, const uint8_t *__restrict__ A,
                                                 uint8_t *__restrict__ cf,
                                                 unsigned *__restrict__ line) {
  const size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  if (c >= (size_t)n * n * n) return;
  int i, j, k;
  decode_index(c, n, n, i, j, k);
  auto liq = [&](int x, int y, int z) -> unsigned {
    return x >= 0 && x < n && y >= 0 && y < n && z >= 0 && z < n &&
           A[((size_t)x * n + y) * n + z] == CELL_FLUID;
  };
  unsigned v = 0;
  if (A[c] == CELL_FLUID) {
    v = 1u;
    v |= (liq(i - 1, j + 1, k) + liq(i - 1, j, k + 1)) << 1;
    v |= (liq(i + 1, j - 1, k) + liq(i, j - 1, k + 1)) << 3;
    v |= (liq(i + 1, j, k - 1) + liq(i, j + 1, k - 1)) << 5;
    line[(size_t)i * njb + (j >> 5)] = 1u;
  }
  cf[c] = (uint8_t)v;
}

/* FAST-mode PCG with the wavefront IC(0)/MIC(0) preconditioner. */
__global__ void __launch_bounds__(IC_BLOCK, 1) k_cg_ic(CgArgs a) {
  if (ir_skipped(a)) return;
  extern __shared__ __align__(16) unsigned char dyn[];
  IcSmem &sm = *reinterpret_cast<IcSmem *>(dyn);
  const unsigned nb = gridDim.x;
  const size_t stride = (size_t)nb * IC_BLOCK;
  const size_t t0 = (size_t)blockIdx.x * IC_BLOCK + threadIdx.x;
  const int n = a.s.n;
  const size_t nc = a.nc;
  constexpr int M = FLIPGPU_SOLVE_FAST;
  unsigned apply = 0; /* preconditioner applications so far */
  /* this launch's tags: base + 1 (factor), base + 2a, base + 2a + 1
   * (application a); the counter moves past them when the launch ends */
  unsigned base = *(volatile const unsigned *)a.ic_ctr;
  auto leave = [&]() {
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.ic_ctr = base + 2u * apply + 2u;
  };
  if (base > IC_TAG_WRAP) {
    /* near the end of the tag space: clear every word, start again at 0 */
    const size_t words = (size_t)a.s.n * a.ic_njb * (size_t)(a.s.n + 31) * 32;
    for (size_t e = t0; e < words; e += stride) a.ic_psk[e] = a.ic_qsk[e] = a.ic_zsk[e] = 0ull;
    base = 0;
    if (!grid_barrier(a.bar, a.iflags)) return leave();
  }

  /* factor (the refinement's later passes keep the first pass's: A and
   * the diagonal are fixed during a solve) */
  if (a.ic_factor) {
    ic_sweeps(a, sm, true, base + 1u, 0u);
    if (!grid_barrier(a.bar, a.iflags, a.ticket)) return leave();
  }

  /* r = b - A x; b.b, r.r */
  FF pbb = ff_zero(), prr = ff_zero();
  for (size_t c = t0; c < nc; c += stride) {
    float rv = 0.0f;
    if (a.A[c] == CELL_FLUID) {
      int i, j, k;
      decode(c, n, i, j, k);
      float bc = a.b[c];
      ff_add_prod(pbb, bc, bc);
      float ax = cg_matvec<M>(a, c, i, j, k, a.x[c], a.x, a.x, 0.0f, true);
      rv = bc - ax;
      ff_add_prod(prr, rv, rv);
    } else {
      a.x[c] = 0.0f;
    }
    a.r[c] = rv;
  }
  store_partial<IC_BLOCK>(a.part, 0, nb, pbb);
  store_partial<IC_BLOCK>(a.part, 1, nb, prr);
  if (!grid_barrier(a.bar, a.iflags)) return leave();
  double b2, rr, unused;
  sum_partials<IC_BLOCK>(a.part, 0, 1, nb, b2, rr);
  const double rt = cg_rel_tol(a);
  const double eps = rt * rt * b2;
  int done = rr <= eps ? 1 : 0, iters = 0;
  double e2 = rr, azr = 0.0;
  if (!done) {
    apply++;
    ic_sweeps(a, sm, false, base + 2u * apply, base + 2u * apply + 1u);
    if (!grid_barrier(a.bar, a.iflags, a.ticket)) return leave();
    azr = ic_sum_parts(a);
  }
  float *so = a.s0, *sn = a.s1;
  float beta_f = 0.0f;
  bool first = true;
  __shared__ float s_bcast;
  while (!done) {
    /* phase A: s = z + beta s, w = A s; w.s */
    FF pws = ff_zero();
    for (size_t c = t0; c < nc; c += stride) {
      if (a.A[c] != CELL_FLUID) continue;
      int i, j, k;
      decode(c, n, i, j, k);
      float zc = __ldcg(a.z + c);
      float snv = first ? zc : zc + beta_f * so[c];
      float wv = cg_matvec<M>(a, c, i, j, k, snv, a.z, so, beta_f, first);
      ff_add_prod(pws, wv, snv);
      sn[c] = snv;
      a.w[c] = wv;
    }
    store_partial<IC_BLOCK>(a.part, 3, nb, pws);
    if (!grid_barrier(a.bar, a.iflags)) return leave();
    double ws;
    sum_partials<IC_BLOCK>(a.part, 3, -1, nb, ws, unused);
    if (threadIdx.x == 0) s_bcast = (float)(azr / ws); /* one FP64 division per block */
    __syncthreads();
    const float alpha_f = s_bcast;
    /* phase B: x += alpha s, r -= alpha w; r.r */
    FF prr2 = ff_zero();
    for (size_t c = t0; c < nc; c += stride) {
      if (a.A[c] != CELL_FLUID) continue;
      a.x[c] = fmaf(alpha_f, sn[c], a.x[c]);
      float rv = fmaf(-alpha_f, a.w[c], a.r[c]);
      a.r[c] = rv;
      ff_add_prod(prr2, rv, rv);
    }
    store_partial<IC_BLOCK>(a.part, 4, nb, prr2);
    if (!grid_barrier(a.bar, a.iflags)) return leave();
    sum_partials<IC_BLOCK>(a.part, 4, -1, nb, rr, unused);
    iters++;
    e2 = rr;
    if (e2 <= eps) { done = 1; break; }
    if (!(e2 == e2)) { done = 2; break; }
    if (iters >= a.max_iters) { done = 3; break; }
    /* z = M^-1 r by the two wavefront sweeps; z.r = q.q per task */
    apply++;
    ic_sweeps(a, sm, false, base + 2u * apply, base + 2u * apply + 1u);
    if (!grid_barrier(a.bar, a.iflags, a.ticket)) return leave();
    const double zr = ic_sum_parts(a);
    __syncthreads();
    if (threadIdx.x == 0) s_bcast = (float)(zr / azr);
    __syncthreads();
    beta_f = s_bcast;
    azr = zr;
    first = false;
    float *t = so;
    so = sn;
    sn = t;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iflags[IF_DONE] = done;
    a.iflags[IF_ITERS] = iters;
    a.iflags[IF_NAN] = done == 2;
    a.scal[SC_ERR2] = e2;
    a.scal[SC_B2] = b2;
    a.scal[SC_EPS] = eps;
  }
  leave();
}

} // namespace

size_t ic_smem_bytes();

/* FP64 r.r of the true residual b - A x of the FAST-mode matrix (the FP32
 * coefficients, evaluated in double): the check of the outer refinement. */
__global__ void __launch_bounds__(BLK) k_true_r2(SolveArgs s, const uint8_t *__restrict__ A,
                                                 const float *__restrict__ diag,
                                                 const float *__restrict__ b,
                                                 const float *__restrict__ x,
                                                 double *__restrict__ part) {
  __shared__ double sh[BLK];
  const int n = s.n;
  const size_t nc = (size_t)n * n * n;
  double acc2 = 0.0;
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK) {
    if (A[c] != CELL_FLUID) continue;
    int i, j, k;
    decode(c, n, i, j, k);
    double acc = (double)diag[c] * (double)x[c];
    const size_t sj = n, si = (size_t)n * n;
    if (i + 1 < n && A[c + si] == CELL_FLUID) acc -= (double)x[c + si];
    if (i > 0 && A[c - si] == CELL_FLUID) acc -= (double)x[c - si];
    if (j + 1 < n && A[c + sj] == CELL_FLUID) acc -= (double)x[c + sj];
    if (j > 0 && A[c - sj] == CELL_FLUID) acc -= (double)x[c - sj];
    if (k + 1 < n && A[c + 1] == CELL_FLUID) acc -= (double)x[c + 1];
    if (k > 0 && A[c - 1] == CELL_FLUID) acc -= (double)x[c - 1];
    const double r = (double)b[c] - acc * (double)s.inv_h2_f;
    acc2 += r * r;
  }
  sh[threadIdx.x] = acc2;
  __syncthreads();
  for (int w = BLK / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

/* one block of RED_BLOCKS threads: a fixed tree over the block partials */
__global__ void k_true_r2_sum(const double *__restrict__ part, double *__restrict__ scal) {
  __shared__ double sh[RED_BLOCKS];
  sh[threadIdx.x] = part[threadIdx.x];
  __syncthreads();
  for (int w = RED_BLOCKS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) scal[SC_TRUE2] = sh[0];
}

/* ------------------------------------------ mixed-precision refinement */

/* The FAST solve refines: the iterate x = xhi + xlo is a double-float pair
 * (about 48 significant bits), its residual r = b - A x is evaluated with
 * error-free FP32 transforms, and each pass solves A e = r with the FP32
 * PCG (any preconditioner) to a loose relative tolerance, then adds e to the
 * pair. Stopping is on the residual of the pair, ||r|| <= rel_tol ||b||. With
 * x stored in FP32 alone, b - A x levels off near the FP32 rounding of A x
 * (about 1e-4 of ||b|| at n = 128), which no restart can move. GB300's FP64
 * rate is about 1/64 of its FP32 rate, so the FP64-class arithmetic runs on
 * the FP32 pipe; only per-block partials and scalars are doubles. */

/* x + y for a double-float x and a float y (TwoSum, then renormalise) */
__device__ __forceinline__ FF df_add_f(FF x, float y) {
  float s, e;
  refmath::two_sum(x.hi, y, s, e);
  e += x.lo;
  const float hi = s + e;
  return FF{hi, e - (hi - s)};
}

/* x * y for a double-float x and a float y (exact product of the high
 * word by FMA) */
__device__ __forceinline__ FF df_mul_f(FF x, float y) {
  const float p = x.hi * y;
  float pe = fmaf(x.hi, y, -p);
  pe = fmaf(x.lo, y, pe);
  const float hi = p + pe;
  return FF{hi, pe - (hi - p)};
}

constexpr double IR_INNER_FLOOR = 1e-3; /* tightest inner tolerance asked for:
                                           the FP32 inner solve's true residual
                                           follows its recursive one to about
                                           there (FLIPGPU_IR_FLOOR overrides) */

constexpr int IR_BLOCKS = 4 * RED_BLOCKS; /* residual blocks (partials: 2 x IR_BLOCKS <= 8192) */

/* r = b - A (xhi + xlo) on the liquid, rb = float(r), e = 0, and the block
 * partials of r.r (and, on the first pass, b.b). The first pass starts from
 * xlo = 0 and zeroes x off the liquid, as every FAST solve leaves it. */
template <bool FIRST>
__global__ void __launch_bounds__(BLK)
k_ir_residual(SolveArgs s, const uint8_t *__restrict__ A, const float *__restrict__ diag,
              const float *__restrict__ b, float *__restrict__ xhi, float *__restrict__ xlo,
              float *__restrict__ rb, float *__restrict__ e, const int *__restrict__ iflags,
              double *__restrict__ part) {
  if (!FIRST && *(volatile const int *)(iflags + IF_IR_DONE)) return;
  const int n = s.n;
  const size_t nc = (size_t)n * n * n;
  const size_t sj = n, si = (size_t)n * n;
  FF rr = ff_zero(), bb = ff_zero();
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK) {
    if (A[c] != CELL_FLUID) {
      rb[c] = 0.0f;
      e[c] = 0.0f;
      if (FIRST) {
        xhi[c] = 0.0f;
        xlo[c] = 0.0f;
      }
      continue;
    }
    int i, j, k;
    decode(c, n, i, j, k);
    const float d = diag[c], hc = xhi[c];
    const float p = d * hc;
    FF S{p, fmaf(d, hc, -p)}; /* diag * xhi exactly */
    float T = FIRST ? 0.0f : d * xlo[c];
    auto nb = [&](size_t q) {
      S = df_add_f(S, -xhi[q]);
      if (!FIRST) T -= xlo[q];
    };
    if (i + 1 < n && A[c + si] == CELL_FLUID) nb(c + si);
    if (i > 0 && A[c - si] == CELL_FLUID) nb(c - si);
    if (j + 1 < n && A[c + sj] == CELL_FLUID) nb(c + sj);
    if (j > 0 && A[c - sj] == CELL_FLUID) nb(c - sj);
    if (k + 1 < n && A[c + 1] == CELL_FLUID) nb(c + 1);
    if (k > 0 && A[c - 1] == CELL_FLUID) nb(c - 1);
    S = df_add_f(S, T);
    const FF ax = df_mul_f(S, s.inv_h2_f);
    const float bc = b[c];
    const FF r = df_add_f(FF{-ax.hi, -ax.lo}, bc);
    const float r32 = r.hi + r.lo;
    rb[c] = r32;
    e[c] = 0.0f;
    if (FIRST) {
      xlo[c] = 0.0f;
      ff_add_prod(bb, bc, bc);
    }
    ff_add_prod(rr, r32, r32);
  }
  const FF t = block_sum_ff<BLK>(rr);
  if (threadIdx.x == 0) part[blockIdx.x] = ff_to_double(t);
  if (FIRST) {
    const FF t2 = block_sum_ff<BLK>(bb);
    if (threadIdx.x == 0) part[IR_BLOCKS + blockIdx.x] = ff_to_double(t2);
  }
}

/* One block of RED_BLOCKS threads: the true r.r (and b.b) in a fixed tree,
 * then the outer loop's decision: converged, failed, or the next inner
 * solve's relative tolerance, aimed at half the remaining reduction and no
 * tighter than IR_INNER_FLOOR. */
__global__ void __launch_bounds__(RED_BLOCKS)
k_ir_check(int first, double rel_tol, int max_passes, double floor_tol,
           const double *__restrict__ part, double *__restrict__ scal, int *__restrict__ iflags) {
  __shared__ double sh[RED_BLOCKS], sb[RED_BLOCKS];
  if (!first && iflags[IF_IR_DONE]) return;
  /* each thread first adds IR_BLOCKS / RED_BLOCKS partials in order */
  double a = 0.0, bsum = 0.0;
  for (int q = 0; q < IR_BLOCKS / RED_BLOCKS; q++) {
    a += part[threadIdx.x * (IR_BLOCKS / RED_BLOCKS) + q];
    if (first) bsum += part[IR_BLOCKS + threadIdx.x * (IR_BLOCKS / RED_BLOCKS) + q];
  }
  sh[threadIdx.x] = a;
  sb[threadIdx.x] = bsum;
  __syncthreads();
  for (int w = RED_BLOCKS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sh[threadIdx.x] += sh[threadIdx.x + w];
      sb[threadIdx.x] += sb[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double rr = sh[0];
  if (first) scal[SC_IR_B2] = sb[0];
  const double b2 = scal[SC_IR_B2];
  scal[SC_TRUE2] = rr;
  const int pass = iflags[IF_IR_PASS];
  int done = 0;
  if (!(rr == rr) || !(b2 == b2)) done = 2;
  else if (b2 == 0.0) done = 4;
  else if (rr <= rel_tol * rel_tol * b2) done = 1;
  else if (pass >= max_passes) done = 3;
  else if (pass > 0 && rr > 0.81 * scal[SC_IR_PREV]) done = 3; /* < 10 % per pass: stalled */
  if (done) {
    iflags[IF_IR_DONE] = done;
    return;
  }
  double t = 0.5 * rel_tol * sqrt(b2 / rr);
  t = t < floor_tol ? floor_tol : (t > 0.5 ? 0.5 : t);
  scal[SC_IR_TOL] = t;
  scal[SC_IR_PREV] = rr;
}

/* x += e after an inner solve (double-float add), unless the inner solve
 * failed; a zero right-hand side sets x = 0. Block 0 books the pass. */
__global__ void __launch_bounds__(BLK)
k_ir_update(size_t nc, const uint8_t *__restrict__ A, const float *__restrict__ e,
            float *__restrict__ xhi, float *__restrict__ xlo, int *__restrict__ iflags) {
  const int ir = *(volatile const int *)(iflags + IF_IR_DONE);
  if (ir != 0 && ir != 4) return;
  const int inner = iflags[IF_DONE];
  const bool failed = iflags[IF_TIMEOUT] != 0 || inner == 2;
  if (ir == 0 && failed) {
    if (blockIdx.x == 0 && threadIdx.x == 0) iflags[IF_IR_DONE] = 2;
    return;
  }
  for (size_t c = (size_t)blockIdx.x * BLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * BLK) {
    if (A[c] != CELL_FLUID) continue;
    if (ir == 4) {
      xhi[c] = 0.0f;
      xlo[c] = 0.0f;
      continue;
    }
    float s, err;
    refmath::two_sum(xhi[c], e[c], s, err);
    err += xlo[c];
    const float hi = s + err;
    xhi[c] = hi;
    xlo[c] = err - (hi - s);
  }
  if (ir == 0 && blockIdx.x == 0 && threadIdx.x == 0) {
    iflags[IF_IR_ITERS] += iflags[IF_ITERS];
    iflags[IF_IR_PASS] += 1;
    /* an inner solve that hit its iteration cap still improved x; the next
     * check decides whether the outer loop goes on */
  }
}

/* xhi + xlo as double (flipgpu_get_pressure) */
__global__ void __launch_bounds__(BLK)
k_pressure_double(size_t nc, const float *__restrict__ xhi, const float *__restrict__ xlo,
                  double *__restrict__ out) {
  const size_t c = (size_t)blockIdx.x * BLK + threadIdx.x;
  if (c < nc) out[c] = (double)xhi[c] + (xlo ? (double)xlo[c] : 0.0);
}

/* Statistics and status of the last solve from the device slots. A refined
 * solve (IF_IR_PASS > 0 or a decision in IF_IR_DONE) reports its passes,
 * the inner iterations of all of them and the true residual of the
 * double-float iterate as r2; its status is that of the outer loop. */
static void stats_from(const double *sc, const int *fl, FlipGpuSolveStats *st) {
  *st = FlipGpuSolveStats();
  const bool refined = fl[IF_IR_DONE] != 0 || fl[IF_IR_PASS] > 0;
  st->b2 = sc[SC_B2];
  st->r2 = sc[SC_ERR2];
  st->r2_true = sc[SC_TRUE2];
  if (refined) {
    st->iterations = fl[IF_IR_ITERS];
    st->refine_passes = fl[IF_IR_PASS];
    st->b2 = sc[SC_IR_B2];
    st->r2 = sc[SC_TRUE2];
    const int ir = fl[IF_IR_DONE];
    st->status = fl[IF_TIMEOUT] ? FLIPGPU_ETIMEOUT
                 : ir == 2      ? FLIPGPU_ENAN
                 : (ir == 1 || ir == 4) ? FLIPGPU_OK
                                        : FLIPGPU_ENOCONV;
  } else {
    st->iterations = fl[IF_ITERS];
    st->status = fl[IF_TIMEOUT] ? FLIPGPU_ETIMEOUT
                 : fl[IF_NAN]   ? FLIPGPU_ENAN
                 : fl[IF_DONE] == 3 ? FLIPGPU_ENOCONV
                                    : FLIPGPU_OK;
  }
}

int read_solve_stats(FlipGpu *h, FlipGpuSolveStats *st) {
  double sc[SC_COUNT];
  int fl[IF_COUNT];
  cudaMemcpyAsync(sc, h->scal, sizeof(sc), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(fl, h->iflags, sizeof(fl), cudaMemcpyDeviceToHost, h->stream);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return FLIPGPU_ECUDA;
  stats_from(sc, fl, st);
  return FLIPGPU_OK;
}

static int finish_stats(FlipGpu *h, FlipGpuSolveStats *st, int mode) {
  double sc[SC_COUNT];
  int host_flags[IF_COUNT];
  cudaMemcpyAsync(sc, h->scal, sizeof(sc), cudaMemcpyDeviceToHost, h->stream);
  cudaMemcpyAsync(host_flags, h->iflags, sizeof(host_flags), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    snprintf(h->err, sizeof h->err, "solve: %s", cudaGetErrorString(e));
    return FLIPGPU_ECUDA;
  }
  FlipGpuSolveStats one;
  stats_from(sc, host_flags, &one);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  one.ms = ms;
  if (st) *st = one;
  const int status = one.status;
  if (status == FLIPGPU_ETIMEOUT) {
    snprintf(h->err, sizeof h->err, "solve: a grid barrier wait expired");
    return status;
  }
  if (status == FLIPGPU_ENAN) {
    snprintf(h->err, sizeof h->err, "solve: non-finite residual");
    return status;
  }
  /* the reference stops silently at its cap */
  if (status == FLIPGPU_ENOCONV && mode != FLIPGPU_SOLVE_REF) {
    if (one.refine_passes > 0)
      snprintf(h->err, sizeof h->err,
               "solve: true residual %.3g of ||b|| after %d refinement passes (%d iterations)",
               one.b2 > 0.0 ? sqrt(one.r2 / one.b2) : 0.0, one.refine_passes, one.iterations);
    else
      snprintf(h->err, sizeof h->err, "solve: no convergence in %d iterations", one.iterations);
    return status;
  }
  return FLIPGPU_OK;
}

constexpr int MG_COARSE_SWEEPS = 2; /* the iteration count does not depend on it */
constexpr int MG_SWEEPS_DEFAULT = 2; /* measured: 1 -> 2 sweeps cut the solve 11 % at
                                          n=128 and 35 % at n=256; 3 gain nothing */
constexpr int CG_MG_BLOCK = 512;
constexpr size_t MG_SMEM_MAX = 96 * 1024; /* block 0's levels: <= 16^3 + 8^3 + 4^3 cells */

/* threads per block of a persistent CG kernel */
static int cg_block_of(const void *kern) {
  if (kern == (const void *)k_cg_cg1<CG1_BLOCK_SMALL>) return CG1_BLOCK_SMALL;
  if (kern == (const void *)k_cg_cg1<CG1_BLOCK_LARGE>) return CG1_BLOCK_LARGE;
  if (kern == (const void *)k_cg_mg<CG_MG_BLOCK>) return CG_MG_BLOCK;
  if (kern == (const void *)k_cg_ic) return IC_BLOCK;
  return CG_BLOCK;
}

/* The level sizes (n, ceil(n/2), ... down to at most 4 per axis), the first
 * level solved in block 0 (at most 16^3 cells) and the buffers of levels
 * 1.. plus the level-0 scratch (residual, second direction, A p). */
int mg_alloc(FlipGpu *h) {
  if (h->mg_nlev > 0) return FLIPGPU_OK;
  int m = h->n, nlev = 0;
  int lv[MG_MAX_LEVELS];
  lv[nlev++] = m;
  while (m > 4 && nlev < MG_MAX_LEVELS) {
    m = (m + 1) / 2;
    lv[nlev++] = m;
  }
  if (nlev < 2 || lv[nlev - 1] > 4) return FLIPGPU_EINVAL;
  int lb = 1;
  while (lb < nlev - 1 && (size_t)lv[lb] * lv[lb] * lv[lb] > MG_BLOCK_CELLS) lb++;
  if (mg_block_bytes(lv, lb, nlev) > MG_SMEM_MAX) return FLIPGPU_EINVAL;
  const size_t nc = h->nc;
  bool ok = cudaMalloc(&h->mg_res[0], nc * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&h->mg_p2, nc * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&h->mg_q, nc * sizeof(float)) == cudaSuccess;
  for (int l = 1; ok && l < nlev; l++) {
    const size_t c = (size_t)lv[l] * lv[l] * lv[l];
    ok = cudaMalloc(&h->mg_flags[l], c) == cudaSuccess &&
         cudaMalloc(&h->mg_diag[l], c * sizeof(float)) == cudaSuccess &&
         cudaMalloc(&h->mg_x[l], c * sizeof(float)) == cudaSuccess &&
         cudaMalloc(&h->mg_b[l], c * sizeof(float)) == cudaSuccess &&
         cudaMalloc(&h->mg_res[l], c * sizeof(float)) == cudaSuccess;
  }
  if (!ok) {
    mg_free(h);
    return FLIPGPU_ENOMEM;
  }
  for (int l = 0; l < nlev; l++) h->mg_m[l] = lv[l];
  h->mg_lb = lb;
  h->mg_nlev = nlev;
  return FLIPGPU_OK;
}

void mg_free(FlipGpu *h) {
  for (int l = 0; l < MG_MAX_LEVELS; l++) {
    if (h->mg_flags[l]) cudaFree(h->mg_flags[l]);
    if (h->mg_diag[l]) cudaFree(h->mg_diag[l]);
    if (h->mg_x[l]) cudaFree(h->mg_x[l]);
    if (h->mg_b[l]) cudaFree(h->mg_b[l]);
    if (h->mg_res[l]) cudaFree(h->mg_res[l]);
    h->mg_flags[l] = nullptr;
    h->mg_diag[l] = h->mg_x[l] = h->mg_b[l] = h->mg_res[l] = nullptr;
  }
  if (h->mg_p2) cudaFree(h->mg_p2);
  if (h->mg_q) cudaFree(h->mg_q);
  h->mg_p2 = h->mg_q = nullptr;
  h->mg_nlev = 0;
}

/* Buffers of the IC(0)/MIC(0) line wavefront (FAST mode). */
int ic_alloc(FlipGpu *h) {
  if (h->ic_tasks > 0) return FLIPGPU_OK;
  const int n = h->n, njb = (n + 31) / 32, nis = (n + IC_W - 1) / IC_W;
  const size_t lines = (size_t)n * njb, words = lines * (size_t)(n + 31) * 32;
  const int tasks = nis * njb;
  bool ok = cudaMalloc(&h->ic_order, tasks * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&h->ic_line, lines * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&h->ic_cf, h->nc) == cudaSuccess &&
            cudaMalloc(&h->ic_pf, words * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&h->ic_psk, words * 8) == cudaSuccess &&
            cudaMalloc(&h->ic_qsk, words * 8) == cudaSuccess &&
            cudaMalloc(&h->ic_zsk, words * 8) == cudaSuccess &&
            cudaMalloc(&h->ic_part, tasks * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&h->ic_ctr, sizeof(unsigned)) == cudaSuccess;
  if (ok) {
    /* tasks by increasing i block + j block: every task's dependencies
     * (i block - 1, j block - 1) come earlier */
    std::vector<unsigned> order;
    for (int d = 0; d <= nis + njb - 2; d++)
      for (int I = 0; I < nis; I++) {
        const int jb = d - I;
        if (jb >= 0 && jb < njb) order.push_back((unsigned)(I * njb + jb));
      }
    ok = cudaMemcpy(h->ic_order, order.data(), order.size() * sizeof(unsigned),
                    cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(h->ic_psk, 0, words * 8) == cudaSuccess &&
         cudaMemset(h->ic_qsk, 0, words * 8) == cudaSuccess &&
         cudaMemset(h->ic_zsk, 0, words * 8) == cudaSuccess &&
         cudaMemset(h->ic_ctr, 0, sizeof(unsigned)) == cudaSuccess;
  }
  if (!ok) {
    ic_free(h);
    return FLIPGPU_ENOMEM;
  }
  h->ic_njb = njb;
  h->ic_tasks = tasks;
  return FLIPGPU_OK;
}

void ic_free(FlipGpu *h) {
  void *ptrs[] = {h->ic_order, h->ic_line, h->ic_cf, h->ic_pf, h->ic_psk,
                  h->ic_qsk,   h->ic_zsk,  h->ic_part, h->ic_ctr};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  h->ic_order = h->ic_line = h->ic_ctr = nullptr;
  h->ic_cf = nullptr;
  h->ic_pf = nullptr;
  h->ic_psk = h->ic_qsk = h->ic_zsk = nullptr;
  h->ic_part = nullptr;
  h->ic_tasks = 0;
}

/* the persistent solve kernel's name in the per-kernel profile */
static const char *solve_kernel_name(const void *kern) {
  if (kern == (const void *)k_cg_mg<CG_MG_BLOCK>) return "k_cg_mg";
  if (kern == (const void *)k_cg_ic) return "k_cg_ic";
  if (kern == (const void *)k_cg_cg1<CG1_BLOCK_SMALL> ||
      kern == (const void *)k_cg_cg1<CG1_BLOCK_LARGE>)
    return "k_cg_cg1";
  return "k_cg";
}

int run_solve(FlipGpu *h, FlipGpuSolveStats *st) {
  const int n = h->n;
  const size_t nc = h->nc;
  const int mode = h->prm.solve_mode;
  int precond = h->prm.precond;
  if (mode == FLIPGPU_SOLVE_REF) precond = FLIPGPU_PRECOND_REF;
  if (mode == FLIPGPU_SOLVE_FAST && precond == FLIPGPU_PRECOND_REF) precond = FLIPGPU_PRECOND_JACOBI;
  SolveArgs sa;
  sa.n = n;
  sa.subcell = h->prm.subcell;
  sa.pow2 = (n & (n - 1)) == 0;
  float h2f = (float)(1.0 / ((double)n * n));
  sa.h2 = (double)h2f;
  sa.inv_h2 = 1.0 / (double)h2f;
  sa.inv_h2_f = (float)sa.inv_h2;
  const double ref_eps = 1.0e-2 * ((double)n * n * n);
  long cap = h->prm.max_iters > 0 ? h->prm.max_iters : (long)nc;
  /* a multigrid solve that needs more than this has failed: stop early */
  if (h->prm.max_iters <= 0 && h->prm.precond == FLIPGPU_PRECOND_MG && cap > 1000) cap = 1000;
  const int max_iters = cap > 0x7fffffff ? 0x7fffffff : (int)cap;
  cudaStream_t S = h->stream;
  const unsigned G = grid_for(nc, BLK);
  auto scalar = [&](int what) {
    k_scalar<<<1, SPINE, 0, S>>>(what, mode, RED_BLOCKS, h->partial, h->scal, h->iflags,
                                 h->prm.eps_abs, h->prm.rel_tol, ref_eps, max_iters);
    FG_LAUNCHED(h, 1);
  };
  if (!h->async_mode) cudaEventRecord(h->ev0, S);
  cudaMemsetAsync(h->iflags, 0, IF_COUNT * sizeof(int), S);
  /* setup: flip b, preconditioner / diagonal */
  k_setup<<<G, BLK, 0, S>>>(sa, mode, h->A, h->L, h->div,
                            mode == FLIPGPU_SOLVE_REF ? h->P : nullptr,
                            mode == FLIPGPU_SOLVE_REF ? nullptr : h->diag,
                            precond == FLIPGPU_PRECOND_JACOBI ? h->Pf : nullptr, h->iflags);
  FG_LAUNCHED(h, 1);
  /* the system as posed (b negated as the reference does), for training data */
  if (h->capture && h->cap_b) {
    cudaMemcpyAsync(h->cap_b, h->div, nc * sizeof(float), cudaMemcpyDeviceToDevice, S);
    cudaMemcpyAsync(h->cap_x0, h->press, nc * sizeof(float), cudaMemcpyDeviceToDevice, S);
    if (mode == FLIPGPU_SOLVE_FAST) launch_residual(h, sa.inv_h2_f, h->press, h->cap_r0);
    else cudaMemsetAsync(h->cap_r0, 0, nc * sizeof(float), S);
  }
  /* learned warm start: x0 += g d before CG (FAST mode) */
  double wres[3] = {0.0, 0.0, 0.0};
  float wms = 0.0f;
  const int warm = h->warm && mode == FLIPGPU_SOLVE_FAST;
  if (warm) {
    int wr = warm_start_apply(h, sa.inv_h2_f, wres, &wms);
    if (wr != FLIPGPU_OK) return wr;
  }
  auto warm_stats = [&](FlipGpuSolveStats *o) {
    if (!o) return;
    o->warm = warm;
    o->r2_prev = wres[0];
    o->r2_guess = warm ? wres[1] : 0.0;
    o->gamma = wres[2];
    o->warm_ms = wms;
  };
  /* persistent single-launch CG unless the REF preconditioner has an entry
   * equal to 1.0 (then its neighbour terms act and it runs sequentially) */
  bool persistent = precond != FLIPGPU_PRECOND_NONE && h->cg_grid[0] > 0;
  if (precond == FLIPGPU_PRECOND_MG) {
    if (mode != FLIPGPU_SOLVE_FAST || n % 4 != 0 || n < 8 || h->cg_grid[5] <= 0 ||
        nc / 4 >= (size_t)1 << 31) {
      snprintf(h->err, sizeof h->err, "solve: the MG preconditioner needs FAST mode, n %% 4 == 0, "
                                      "n >= 8 and a cooperative launch");
      return FLIPGPU_EINVAL;
    }
    const int r = mg_alloc(h);
    if (r != FLIPGPU_OK) {
      snprintf(h->err, sizeof h->err, "solve: multigrid buffers (%d)", r);
      return r;
    }
  }
  if (precond == FLIPGPU_PRECOND_IC && (mode != FLIPGPU_SOLVE_FAST || h->cg_grid[3] <= 0)) {
    snprintf(h->err, sizeof h->err, "solve: the IC preconditioner needs FAST mode and a "
                                    "cooperative launch");
    return FLIPGPU_EINVAL;
  }
  if (precond == FLIPGPU_PRECOND_IC) {
    const int r = ic_alloc(h);
    if (r != FLIPGPU_OK) {
      snprintf(h->err, sizeof h->err, "solve: wavefront buffers (%d)", r);
      return r;
    }
  }
  if (persistent && mode == FLIPGPU_SOLVE_REF) {
    int exotic = 0;
    cudaMemcpyAsync(&exotic, h->iflags + IF_EXOTIC, sizeof(int), cudaMemcpyDeviceToHost, S);
    cudaStreamSynchronize(S);
    persistent = exotic == 0;
  }
  if (persistent) {
    CgArgs a;
    a.s = sa;
    a.nc = nc;
    a.A = h->A;
    a.L = h->L;
    a.b = h->div;
    a.x = h->press;
    a.r = h->r;
    a.z = h->z;
    a.s0 = h->s;
    a.s1 = h->s1;
    a.w = h->w;
    a.w1 = h->w1;
    a.p = h->pdir;
    a.P = h->P;
    a.diag = h->diag;
    a.Pf = h->Pf;
    a.part = (float2 *)h->partial;
    a.bar = h->bar;
    a.iflags = h->iflags;
    a.scal = h->scal;
    a.eps_abs = h->prm.eps_abs;
    a.rel_tol = h->prm.rel_tol;
    a.ref_eps = ref_eps;
    a.max_iters = max_iters;
    a.mic_tau = (float)h->prm.mic_tau;
    a.ticket = h->ticket;
    a.ic_njb = h->ic_njb;
    a.ic_tasks = h->ic_tasks;
    a.ic_order = h->ic_order;
    a.ic_line = h->ic_line;
    a.ic_cf = h->ic_cf;
    a.ic_pf = h->ic_pf;
    a.ic_psk = h->ic_psk;
    a.ic_qsk = h->ic_qsk;
    a.ic_zsk = h->ic_zsk;
    a.ic_part = h->ic_part;
    a.ic_ctr = h->ic_ctr;
    a.ic_factor = 1;
    cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), S);
    void *kargs[] = {&a};
    const void *kern = mode == FLIPGPU_SOLVE_REF ? (const void *)k_cg<FLIPGPU_SOLVE_REF>
                                                 : (const void *)k_cg<FLIPGPU_SOLVE_FAST>;
    int grid = h->cg_grid[mode == FLIPGPU_SOLVE_REF ? 0 : 1];
    size_t smem = 0;
    a.chunk_list = nullptr;
    a.chunk_count = nullptr;
    a.p2 = a.q = nullptr;
    std::memset(&a.mg, 0, sizeof a.mg);
    /* the 32-quad chunks holding liquid (A is fixed during the solve) */
    auto chunk_list = [&]() -> cudaError_t {
      const size_t nq = nc / 4, nch = (nq + 31) / 32;
      k_cg1_chunk_flags<<<grid_for((nch + 1) * 32, BLK), BLK, 0, S>>>(
          nq, reinterpret_cast<const uchar4 *>(h->A), h->chunk_off);
      FG_LAUNCHED(h, 1);
      cudaError_t e = scan_exclusive(h, h->chunk_off, h->chunk_off, nch + 1);
      if (e == cudaSuccess) {
        k_cg1_chunk_scatter<<<grid_for(nch, BLK), BLK, 0, S>>>(nch, h->chunk_off, h->chunk_list);
        FG_LAUNCHED(h, 1);
        e = cudaGetLastError();
      }
      a.chunk_list = h->chunk_list;
      a.chunk_count = h->chunk_off + nch;
      return e;
    };
    if (mode == FLIPGPU_SOLVE_FAST && precond == FLIPGPU_PRECOND_JACOBI && n % 4 == 0 &&
        nc / 4 < (size_t)1 << 31) {
      const bool large = n >= CG1_LARGE_N;
      kern = large ? (const void *)k_cg_cg1<CG1_BLOCK_LARGE> : (const void *)k_cg_cg1<CG1_BLOCK_SMALL>;
      grid = h->cg_grid[large ? 4 : 2];
      cudaError_t e = chunk_list();
      if (e != cudaSuccess) {
        snprintf(h->err, sizeof h->err, "solve: chunk list: %s", cudaGetErrorString(e));
        return FLIPGPU_ECUDA;
      }
    }
    if (precond == FLIPGPU_PRECOND_MG) {
      kern = (const void *)k_cg_mg<CG_MG_BLOCK>;
      grid = h->cg_grid[5];
      smem = mg_block_bytes(h->mg_m, h->mg_lb, h->mg_nlev);
      cudaError_t e = chunk_list();
      /* levels: 0 = the solver's grid (z the correction, r its right-hand
       * side); coarser ones from the coarsened flags */
      MgArgs &mg = a.mg;
      mg.nlev = h->mg_nlev;
      mg.lb = h->mg_lb;
      mg.coarse_sweeps = MG_COARSE_SWEEPS;
      mg.nu = h->prm.mg_sweeps > 0 ? h->prm.mg_sweeps : MG_SWEEPS_DEFAULT;
      float hs = sa.inv_h2_f;
      for (int l = 0; l < mg.nlev; l++) {
        MgLevel &L = mg.lv[l];
        L.m = h->mg_m[l];
        L.flags = l == 0 ? h->A : h->mg_flags[l];
        L.diag = l == 0 ? h->diag : h->mg_diag[l];
        L.x = l == 0 ? h->z : h->mg_x[l];
        L.b = l == 0 ? h->r : h->mg_b[l];
        L.res = h->mg_res[l];
        L.hs = hs;
        L.ihs = 1.0f / hs;
        L.lgm = (L.m & (L.m - 1)) == 0 ? __builtin_ctz((unsigned)L.m) : -1;
        hs *= 0.25f;
      }
      for (int l = 1; e == cudaSuccess && l < mg.nlev; l++) {
        const size_t c = (size_t)h->mg_m[l] * h->mg_m[l] * h->mg_m[l];
        k_mg_coarsen<<<grid_for(c, BLK), BLK, 0, S>>>(mg.lv[l - 1].flags, h->mg_m[l - 1],
                                                      h->mg_flags[l], h->mg_m[l]);
        k_mg_diag<<<grid_for(c, BLK), BLK, 0, S>>>(h->mg_flags[l], h->mg_m[l], h->mg_diag[l]);
        FG_LAUNCHED(h, 2);
        e = cudaGetLastError();
      }
      a.p2 = h->mg_p2;
      a.q = h->mg_q;
      /* zero off the liquid chunks (the sweeps only write inside them) and
       * finite direction buffers for the first iteration */
      float *zero_bufs[5] = {h->z, h->mg_res[0], h->pdir, h->mg_p2, h->mg_q};
      for (float *zb : zero_bufs)
        if (e == cudaSuccess) e = cudaMemsetAsync(zb, 0, nc * sizeof(float), S);
      if (e != cudaSuccess) {
        snprintf(h->err, sizeof h->err, "solve: multigrid setup: %s", cudaGetErrorString(e));
        return FLIPGPU_ECUDA;
      }
    }
    /* no more blocks than the grid has work for (about two quads or eight
     * cells per thread): small grids keep short barriers and leave the rest
     * of the GPU to other simulations */
    if (precond != FLIPGPU_PRECOND_IC) {
      h->solve_capacity = grid;
      const size_t per_block = (size_t)cg_block_of(kern) * 8;
      const size_t want = (nc + per_block - 1) / per_block;
      if (want < (size_t)grid) grid = want > 0 ? (int)want : 1;
      /* the caller's share of the GPU (flipgpu_set_solve_blocks) */
      if (h->solve_blocks > 0 && h->solve_blocks < grid) grid = h->solve_blocks;
    }
    if (mode == FLIPGPU_SOLVE_FAST && precond == FLIPGPU_PRECOND_IC) {
      kern = (const void *)k_cg_ic;
      grid = h->cg_grid[3];
      smem = ic_smem_bytes();
      if (a.max_iters > IC_MAX_ITERS) a.max_iters = IC_MAX_ITERS;
      /* liquid flags, MIC(0) counts and liquid lines (A is fixed during
       * the solve) */
      cudaMemsetAsync(h->ic_line, 0, (size_t)n * h->ic_njb * sizeof(unsigned), S);
      k_ic_prep<<<grid_for(nc, BLK), BLK, 0, S>>>(n, h->ic_njb, h->A, h->ic_cf, h->ic_line);
      FG_LAUNCHED(h, 1);
      cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), S);
    }
    a.ir_skip = nullptr;
    a.ir_tol = nullptr;
    const int block = cg_block_of(kern);
    auto reset_flags = [&]() {
      cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), S);
      if (precond == FLIPGPU_PRECOND_IC) cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), S);
    };
    if (mode == FLIPGPU_SOLVE_FAST && h->prm.refine_steps > 0) {
      /* mixed-precision iterative refinement: the iterate is the
       * double-float pair (press, press_lo); each pass solves A e = b - A x
       * in FP32 from e = 0 to the tolerance the outer loop sets and adds e.
       * The passes are launched up front and the kernels of passes that are
       * no longer needed return at once, so nothing waits for the host. */
      const int passes = h->prm.refine_steps;
      a.b = h->ir_b;
      a.x = h->ir_e;
      a.ir_skip = h->iflags + IF_IR_DONE;
      a.ir_tol = h->scal + SC_IR_TOL;
      const unsigned ug = grid_for(nc, BLK) < 4096 ? grid_for(nc, BLK) : 4096;
      double floor_tol = IR_INNER_FLOOR;
      if (const char *ev = getenv("FLIPGPU_IR_FLOOR")) {
        const double v = atof(ev);
        if (v > 0.0 && v < 1.0) floor_tol = v;
      }
      k_ir_residual<true><<<IR_BLOCKS, BLK, 0, S>>>(sa, h->A, h->diag, h->div, h->press,
                                                      h->press_lo, h->ir_b, h->ir_e, h->iflags,
                                                      h->partial);
      k_ir_check<<<1, RED_BLOCKS, 0, S>>>(1, h->prm.rel_tol, passes, floor_tol, h->partial,
                                          h->scal, h->iflags);
      FG_LAUNCHED(h, 2);
      for (int pass = 0; pass < passes; pass++) {
        if (pass > 0) reset_flags();
        a.ic_factor = pass == 0;
        ktime_begin(h, solve_kernel_name(kern));
        cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(block), kargs, smem, S);
        ktime_end(h);
        FG_LAUNCHED(h, 1);
        if (e != cudaSuccess) {
          snprintf(h->err, sizeof h->err, "solve: cooperative launch: %s", cudaGetErrorString(e));
          return FLIPGPU_ECUDA;
        }
        k_ir_update<<<ug, BLK, 0, S>>>(nc, h->A, h->ir_e, h->press, h->press_lo, h->iflags);
        k_ir_residual<false><<<IR_BLOCKS, BLK, 0, S>>>(sa, h->A, h->diag, h->div, h->press,
                                                         h->press_lo, h->ir_b, h->ir_e,
                                                         h->iflags, h->partial);
        k_ir_check<<<1, RED_BLOCKS, 0, S>>>(0, h->prm.rel_tol, passes, floor_tol, h->partial,
                                            h->scal, h->iflags);
        FG_LAUNCHED(h, 3);
      }
      h->press_lo_valid = 1;
      if (h->async_mode) return FLIPGPU_OK; /* stats stay on the device (read_solve_stats) */
      cudaEventRecord(h->ev1, S);
      FlipGpuSolveStats one;
      const int rc = finish_stats(h, &one, mode);
      if (st) *st = one;
      warm_stats(st);
      return rc;
    }
    /* FAST mode without refinement: CG stops on its recursive residual with
     * x in FP32, and the true residual b - A x is evaluated in FP64 after */
    ktime_begin(h, solve_kernel_name(kern));
    cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(block), kargs, smem, S);
    ktime_end(h);
    FG_LAUNCHED(h, 1);
    if (e != cudaSuccess) {
      snprintf(h->err, sizeof h->err, "solve: cooperative launch: %s", cudaGetErrorString(e));
      return FLIPGPU_ECUDA;
    }
    if (mode == FLIPGPU_SOLVE_FAST) {
      k_true_r2<<<RED_BLOCKS, BLK, 0, S>>>(sa, h->A, h->diag, h->div, h->press, h->partial);
      k_true_r2_sum<<<1, RED_BLOCKS, 0, S>>>(h->partial, h->scal);
      FG_LAUNCHED(h, 2);
      h->press_lo_valid = 0;
    }
    if (h->async_mode) return FLIPGPU_OK;
    cudaEventRecord(h->ev1, S);
    const int rc = finish_stats(h, st, mode);
    warm_stats(st);
    return rc;
  }
  if (mode == FLIPGPU_SOLVE_REF) {
    k_build_ref_seq<<<1, 1, 0, S>>>(n, h->A, h->P, nullptr, h->iflags, h->L, h->prm.subcell);
    FG_LAUNCHED(h, 1);
  }
  /* b.b and the stop bound */
  k_dot<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, 0, h->A, h->div, h->div, h->partial);
  FG_LAUNCHED(h, 1);
  scalar(ST_B2);

  auto matvec = [&](const float *x, float *out) {
    if (mode == FLIPGPU_SOLVE_REF)
      k_matvec_ref<<<G, BLK, 0, S>>>(sa, h->iflags, h->A, h->L, x, out);
    else
      k_matvec_fast<<<G, BLK, 0, S>>>(sa, h->iflags, h->A, h->diag, x, out);
    FG_LAUNCHED(h, 1);
  };
  auto apply = [&](const float *r, float *z) {
    if (precond == FLIPGPU_PRECOND_REF) {
      k_apply_ref_diag<<<G, BLK, 0, S>>>(sa, h->iflags, h->A, h->P, r, z);
      k_apply_ref_seq<<<1, 1, 0, S>>>(n, h->iflags, h->A, h->P, r, z, h->P + nc);
      FG_LAUNCHED(h, 2);
    } else if (precond == FLIPGPU_PRECOND_JACOBI) {
      k_apply_jacobi<<<G, BLK, 0, S>>>(sa, h->iflags, h->A, h->Pf, r, z);
      FG_LAUNCHED(h, 1);
    } else {
      cudaMemcpyAsync(z, r, nc * sizeof(float), cudaMemcpyDeviceToDevice, S);
    }
  };

  /* z = A x; r = b - z; z = M^-1 r; s = z; a = z.r */
  matvec(h->press, h->z);
  k_residual<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->A, h->div, h->z, h->r, h->partial);
  FG_LAUNCHED(h, 1);
  scalar(ST_ERR0);
  apply(h->r, h->z);
  cudaMemcpyAsync(h->s, h->z, nc * sizeof(float), cudaMemcpyDeviceToDevice, S);
  k_dot<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, 0, h->A, h->z, h->r, h->partial);
  FG_LAUNCHED(h, 1);
  scalar(ST_A0);

  const int CHUNK = 8;
  int done = 0;
  int host_flags[IF_COUNT];
  for (long it = 0; it < max_iters && !done; it += CHUNK) {
    for (int u = 0; u < CHUNK; u++) {
      matvec(h->s, h->z);
      k_dot<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, 1, h->A, h->z, h->s, h->partial);
      FG_LAUNCHED(h, 1);
      scalar(ST_ALPHA);
      k_update_xr<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, h->scal, h->A, h->press, h->r,
                                             h->s, h->z, h->partial);
      FG_LAUNCHED(h, 1);
      scalar(ST_CHECK);
      apply(h->r, h->z);
      k_dot<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, 1, h->A, h->z, h->r, h->partial);
      FG_LAUNCHED(h, 1);
      scalar(ST_BETA);
      k_update_s<<<RED_BLOCKS, BLK, 0, S>>>(nc, h->iflags, h->scal, h->A, h->z, h->s);
      FG_LAUNCHED(h, 1);
    }
    cudaError_t e = cudaMemcpyAsync(host_flags, h->iflags, sizeof(host_flags),
                                    cudaMemcpyDeviceToHost, S);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S);
    if (e != cudaSuccess) {
      snprintf(h->err, sizeof h->err, "solve: %s", cudaGetErrorString(e));
      return FLIPGPU_ECUDA;
    }
    done = host_flags[IF_DONE];
  }
  cudaEventRecord(h->ev1, S);
  double sc[SC_COUNT];
  cudaMemcpyAsync(sc, h->scal, sizeof(sc), cudaMemcpyDeviceToHost, S);
  cudaMemcpyAsync(host_flags, h->iflags, sizeof(host_flags), cudaMemcpyDeviceToHost, S);
  cudaError_t e = cudaStreamSynchronize(S);
  if (e != cudaSuccess) {
    snprintf(h->err, sizeof h->err, "solve: %s", cudaGetErrorString(e));
    return FLIPGPU_ECUDA;
  }
  int status = FLIPGPU_OK;
  if (host_flags[IF_NAN]) status = FLIPGPU_ENAN;
  else if (host_flags[IF_DONE] == 3 || (!host_flags[IF_DONE] && mode != FLIPGPU_SOLVE_REF))
    status = FLIPGPU_ENOCONV;
  if (st) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    st->iterations = host_flags[IF_ITERS];
    st->status = status;
    st->r2 = sc[SC_ERR2];
    st->b2 = sc[SC_B2];
    st->ms = ms;
    warm_stats(st);
  }
  /* The reference stops silently at its cap; only non-finite residuals are
   * errors in REF mode. */
  if (status == FLIPGPU_ENAN) {
    snprintf(h->err, sizeof h->err, "solve: non-finite residual");
    return status;
  }
  if (status == FLIPGPU_ENOCONV && mode != FLIPGPU_SOLVE_REF) {
    snprintf(h->err, sizeof h->err, "solve: no convergence in %d iterations", host_flags[IF_ITERS]);
    return status;
  }
  return FLIPGPU_OK;
}

size_t ic_smem_bytes() { return sizeof(IcSmem); }

void launch_pressure_double(FlipGpu *h, double *out) {
  k_pressure_double<<<grid_for(h->nc, BLK), BLK, 0, h->stream>>>(
      h->nc, h->press, h->press_lo_valid ? h->press_lo : nullptr, out);
  FG_LAUNCHED(h, 1);
}

/* Dynamic shared memory limits of the IC and MG kernels, once per device. */
int ic_init_device() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  if (cudaFuncSetAttribute(k_cg_ic, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)ic_smem_bytes()) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(k_cg_mg<CG_MG_BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)MG_SMEM_MAX) != cudaSuccess)
    return -1;
  done[dev] = true;
  return 0;
}

/* Cooperative grid of each CG variant (REF, FAST, single-reduction with
 * small blocks, IC, single-reduction with large blocks, MG): SMs x resident
 * blocks (at most 4). */
int cg_grid_size(int *out) {
  int dev = 0, sms = 0, coop = 0;
  for (int v = 0; v < CG_VARIANTS; v++) out[v] = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop) return 0;
  if (ic_init_device() != 0) return -1;
  const void *k[CG_VARIANTS] = {(const void *)k_cg<FLIPGPU_SOLVE_REF>,
                                (const void *)k_cg<FLIPGPU_SOLVE_FAST>,
                                (const void *)k_cg_cg1<CG1_BLOCK_SMALL>, (const void *)k_cg_ic,
                                (const void *)k_cg_cg1<CG1_BLOCK_LARGE>,
                                (const void *)k_cg_mg<CG_MG_BLOCK>};
  for (int v = 0; v < CG_VARIANTS; v++) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k[v], cg_block_of(k[v]), v == 3 ? ic_smem_bytes() : v == 5 ? MG_SMEM_MAX : 0);
    if (per_sm > 4) per_sm = 4;
    out[v] = sms * per_sm;
    if (out[v] * 6 > 8192) out[v] = 8192 / 6;
  }
  return 0;
}
