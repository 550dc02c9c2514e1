/*
 * k_grid.cu — the driver's grid stages on the MAC grid.
 *
 *   k_mark_water        sorter::markWater + sorter::levelset per cell
 *   k_divergence        project(): divergence of FLUID cells
 *   k_gradient_enforce  project(): subcell pressure gradient, then the
 *                       second enforce_boundary
 *   k_extrap_delta      extrapolate_velocity, then subtract_grid
 */
#include "devcommon.cuh"

using namespace refmath;

namespace {

constexpr int BLK = 256;

/* sorter::markWater (src/sorter.cpp:83-93) and sorter::levelset
 * (src/sorter.cpp:70-81) from the sorted cell lists. */
__global__ void __launch_bounds__(BLK)
k_mark_water(SimConst c, const uint32_t *__restrict__ cs, const float4 *__restrict__ spos,
             const float *__restrict__ sdens, uint8_t *__restrict__ A, float *__restrict__ L) {
  size_t cidx = (size_t)blockIdx.x * BLK + threadIdx.x;
  const size_t nc = (size_t)c.n * c.n * c.n;
  if (cidx >= nc) return;
  uint32_t s = cs[cidx], e = cs[cidx + 1];
  bool wall = false, nonfluid = false;
  float accm = 0.0f;
  for (uint32_t a = s; a < e; a++) {
    int t = unpack_type(spos[a].w);
    if (t == CELL_WALL) wall = true;
    if (!nonfluid) {
      if (t == CELL_FLUID)
        accm += sdens[a];
      else
        nonfluid = true;
    }
  }
  /* return 0.2*n0 - accm (double), or 1.0 at the first non-fluid particle */
  float l = nonfluid ? 1.0f : add_fd(-accm, c.l0h, c.l0l, c.l0);
  L[cidx] = l;
  A[cidx] = wall ? CELL_WALL : (l < 0.0f ? CELL_FLUID : CELL_AIR);
}

/* Divergence of FLUID cells (src/flip3D.cpp:814-821); other cells keep
 * their previous contents, as the reference's static array does. */
__global__ void __launch_bounds__(BLK)
k_divergence(SimConst c, const uint8_t *__restrict__ A, const float *__restrict__ u0,
             const float *__restrict__ u1, const float *__restrict__ u2,
             float *__restrict__ div) {
  size_t cidx = (size_t)blockIdx.x * BLK + threadIdx.x;
  const int n = c.n;
  const size_t nc = (size_t)n * n * n;
  if (cidx >= nc || A[cidx] != CELL_FLUID) return;
  int i, j, k;
  decode_index(cidx, n, n, i, j, k);
  float d = u0[((size_t)(i + 1) * n + j) * n + k] - u0[((size_t)i * n + j) * n + k] +
            u1[((size_t)i * (n + 1) + j + 1) * n + k] - u1[((size_t)i * (n + 1) + j) * n + k] +
            u2[((size_t)i * n + j) * (n + 1) + k + 1] - u2[((size_t)i * n + j) * (n + 1) + k];
  div[cidx] = d / c.h;
}

/* Subtract the pressure gradient with the subcell ghost values
 * (src/flip3D.cpp:832-867), then enforce_boundary (src/flip3D.cpp:783-805,
 * called again at :1067). */
__global__ void __launch_bounds__(BLK)
k_gradient_enforce(SimConst c, int subcell, int enforce, const uint8_t *__restrict__ A,
                   const float *__restrict__ L, const float *__restrict__ press,
                   const float *__restrict__ press_lo, float *__restrict__ u0,
                   float *__restrict__ u1, float *__restrict__ u2) {
  const int n = c.n;
  const int comp = blockIdx.y;
  size_t f = (size_t)blockIdx.x * BLK + threadIdx.x;
  const size_t nf = (size_t)(n + 1) * n * n;
  if (f >= nf) return;
  const int ex[3] = {comp == 0 ? n + 1 : n, comp == 1 ? n + 1 : n, comp == 2 ? n + 1 : n};
  int i, j, k;
  decode_index(f, ex[1], ex[2], i, j, k);
  int a = comp == 0 ? i : (comp == 1 ? j : k);
  float *u = comp == 0 ? u0 : (comp == 1 ? u1 : u2);
  if (a == 0 || a == n) {
    if (enforce) u[f] = 0.0f;
    return;
  }
  size_t cf = cell_id(n, i, j, k);
  size_t cb = comp == 0 ? cell_id(n, i - 1, j, k)
                        : (comp == 1 ? cell_id(n, i, j - 1, k) : cell_id(n, i, j, k - 1));
  /* with a refined solve the pressure is the pair press + press_lo */
  float pf = press[cf], pb = press[cb];
  const float lof = press_lo ? press_lo[cf] : 0.0f, lob = press_lo ? press_lo[cb] : 0.0f;
  float lf = lof, lb = lob;
  float Lf = L[cf], Lb = L[cb];
  if (subcell && Lf * Lb < 0.0f) {
    if (Lf >= 0.0f) {
      pf = (float)((double)Lf / fmin(1.0e-3, (double)Lb) * ((double)press[cb] + (double)lob));
      lf = 0.0f;
    }
    if (Lb >= 0.0f) {
      pb = (float)((double)Lb / fmin(1.0e-6, (double)Lf) * ((double)press[cf] + (double)lof));
      lb = 0.0f;
    }
  }
  const float dp = press_lo ? (pf - pb) + (lf - lb) : pf - pb;
  float val = u[f] - dp / c.h;
  if (enforce && (A[cf] == CELL_WALL) != (A[cb] == CELL_WALL)) val = 0.0f;
  u[f] = val;
}

/* mark / wall_mark of a face (src/flip3D.cpp:1016-1029). */
__device__ __forceinline__ void face_marks(const uint8_t *__restrict__ A, int n, int comp, int i,
                                           int j, int k, bool &mark, bool &wall_mark) {
  int a = comp == 0 ? i : (comp == 1 ? j : k);
  bool has_minus = a > 0, has_plus = a < n;
  uint8_t am = CELL_WALL, ap = CELL_WALL;
  if (has_minus) {
    int mi = i - (comp == 0), mj = j - (comp == 1), mk = k - (comp == 2);
    am = A[cell_id(n, mi, mj, mk)];
  }
  if (has_plus) ap = A[cell_id(n, i, j, k)];
  mark = (has_minus && am == CELL_FLUID) || (has_plus && ap == CELL_FLUID);
  wall_mark = (!has_minus || am == CELL_WALL) && (!has_plus || ap == CELL_WALL);
}

/* extrapolate_velocity (src/flip3D.cpp:1031-1053): wall faces next to no
 * fluid take the mean of their marked face neighbours; only unmarked faces
 * are written and only marked faces are read. Then subtract_grid
 * (src/flip3D.cpp:985-997): us = u - us. */
__global__ void __launch_bounds__(BLK)
k_extrap_delta(SimConst c, const uint8_t *__restrict__ A, float *__restrict__ u0,
               float *__restrict__ u1, float *__restrict__ u2, float *__restrict__ us0,
               float *__restrict__ us1, float *__restrict__ us2) {
  const int n = c.n;
  const int comp = blockIdx.y;
  size_t f = (size_t)blockIdx.x * BLK + threadIdx.x;
  const size_t nf = (size_t)(n + 1) * n * n;
  if (f >= nf) return;
  const int ex[3] = {comp == 0 ? n + 1 : n, comp == 1 ? n + 1 : n, comp == 2 ? n + 1 : n};
  int i, j, k;
  decode_index(f, ex[1], ex[2], i, j, k);
  float *u = comp == 0 ? u0 : (comp == 1 ? u1 : u2);
  float *us = comp == 0 ? us0 : (comp == 1 ? us1 : us2);
  bool mark, wmark;
  face_marks(A, n, comp, i, j, k, mark, wmark);
  float val = u[f];
  if (!mark && wmark) {
    int wsum = 0;
    float sum = 0.0f;
    const int q[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                         {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
#pragma unroll
    for (int s = 0; s < 6; s++) {
      int qi = q[s][0], qj = q[s][1], qk = q[s][2];
      if (qi < 0 || qi >= ex[0] || qj < 0 || qj >= ex[1] || qk < 0 || qk >= ex[2]) continue;
      bool m2, w2;
      face_marks(A, n, comp, qi, qj, qk, m2, w2);
      if (m2) {
        wsum++;
        sum += u[((size_t)qi * ex[1] + qj) * ex[2] + qk];
      }
    }
    if (wsum) {
      val = sum / (float)wsum;
      u[f] = val;
    }
  }
  us[f] = val - us[f];
}

} // namespace

cudaError_t launch_mark_water(FlipGpu *h) {
  SimConst c = make_const(h);
  k_mark_water<<<grid_for(h->nc, BLK), BLK, 0, h->stream>>>(c, h->cell_start, h->spos,
                                                            h->sdens, h->A, h->L);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_divergence(FlipGpu *h) {
  SimConst c = make_const(h);
  k_divergence<<<grid_for(h->nc, BLK), BLK, 0, h->stream>>>(c, h->A, h->u[0], h->u[1],
                                                            h->u[2], h->div);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_gradient_enforce(FlipGpu *h, int enforce) {
  SimConst c = make_const(h);
  dim3 grid(grid_for(h->nf, BLK), 3);
  k_gradient_enforce<<<grid, BLK, 0, h->stream>>>(
      c, h->prm.subcell, enforce, h->A, h->L, h->press, h->press_lo_valid ? h->press_lo : nullptr,
      h->u[0], h->u[1], h->u[2]);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_extrapolate_delta(FlipGpu *h) {
  SimConst c = make_const(h);
  dim3 grid(grid_for(h->nf, BLK), 3);
  k_extrap_delta<<<grid, BLK, 0, h->stream>>>(c, h->A, h->u[0], h->u[1], h->u[2], h->us[0],
                                              h->us[1], h->us[2]);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}
