/*
 * k_particles.cu — particle stages of the FLIP step.
 *
 * Gathers run one thread per sorted slot, so a warp works on particles of
 * the same few cells and re-reads the same neighbour runs from L1. A
 * neighbourhood of cells [i0,i1]x[j0,j1]x[k0,k1] is visited as in
 * sorter::getNeigboringParticles_* (src/sorter.cpp:42-64): si, then sj,
 * then sk, each cell in particle order; for fixed (si,sj) the k-range is one
 * contiguous run of slots. Every float expression follows the reference's
 * evaluation order and promotions (nvcc -fmad=false; refmath.h for the
 * double-promoted ones), so the results are the reference's bit for bit.
 *
 * The gathers and the per-particle updates are templated on an arithmetic
 * policy: RefArith reproduces those expressions (the default), FastArith
 * evaluates the same formulas in native FP32 with fused multiply-adds and
 * the fast division intrinsic (FLIPGPU_ARITH_FAST).
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "autotune.h"
#include "devcommon.cuh"

using namespace refmath;

namespace {

constexpr int BLK = 256;

/* The reference's expressions, bit for bit (refmath.h). */
struct RefArith {
  static __device__ __forceinline__ float hypot2(float a, float b, float c) {
    return hypot2_ref(a, b, c);
  }
  static __device__ __forceinline__ float length(float a, float b, float c) {
    return length_ref(a, b, c);
  }
  static __device__ __forceinline__ float sharp(float r2, float hh, float r2_floor, float small) {
    return sharp_ref(r2, hh, r2_floor, small);
  }
  static __device__ __forceinline__ float smooth_density(const SimConst &c, float r2) {
    return c.kd_rcp != 0.0f ? smooth_ref_pow2(r2, c.kd_rcp) : smooth_ref(r2, c.kd_hh);
  }
  static __device__ __forceinline__ float smooth_corr(const SimConst &c, float r2) {
    return c.corr_rcp != 0.0f ? smooth_ref_pow2(r2, c.corr_rcp) : smooth_ref(r2, c.re_corr_hh);
  }
  static __device__ __forceinline__ float blend(const SimConst &c, float pic, float flip) {
    return blend_ref(pic, flip, c.c1h, c.c1l, c.c2h, c.c2l, c.c1, c.c2);
  }
  static __device__ __forceinline__ float euler(const SimConst &c, float p, float v) {
    return axpy_fd(p, v, c.dt_h, c.dt_l, c.dt);
  }
  /* the wall push p + (push_re - dist) n, in double as the reference has it */
  static __device__ __forceinline__ float push(const SimConst &c, float p, float dist, float nq) {
    return (float)((double)p + (c.push_re - (double)dist) * (double)nq);
  }
  /* w dx / dist re, left to right */
  static __device__ __forceinline__ float spring_term(float w, float d, float dist, float re) {
    return w * d / dist * re;
  }
};

/* The same formulas in native FP32. */
struct FastArith {
  static __device__ __forceinline__ float hypot2(float a, float b, float c) {
    return fmaf(a, a, fmaf(b, b, c * c));
  }
  static __device__ __forceinline__ float length(float a, float b, float c) {
    return sqrtf(hypot2(a, b, c));
  }
  static __device__ __forceinline__ float sharp(float r2, float hh, float, float) {
    return r2 < hh ? fmaxf(__fdividef(hh, fmaxf(r2, 1.0e-5f)) - 1.0f, 0.0f) : 0.0f;
  }
  static __device__ __forceinline__ float smooth_density(const SimConst &c, float r2) {
    return fmaxf(fmaf(-r2, c.kd_inv, 1.0f), 0.0f);
  }
  static __device__ __forceinline__ float smooth_corr(const SimConst &c, float r2) {
    return fmaxf(fmaf(-r2, c.corr_inv, 1.0f), 0.0f);
  }
  static __device__ __forceinline__ float blend(const SimConst &c, float pic, float flip) {
    return fmaf((float)c.c2, flip, (float)c.c1 * pic);
  }
  static __device__ __forceinline__ float euler(const SimConst &c, float p, float v) {
    return fmaf(v, (float)c.dt, p);
  }
  static __device__ __forceinline__ float push(const SimConst &c, float p, float dist, float nq) {
    return fmaf((float)c.push_re - dist, nq, p);
  }
  static __device__ __forceinline__ float spring_term(float w, float d, float dist, float re) {
    return __fdividef(w * re, dist) * d;
  }
};

constexpr int REPO_GRID = 152 * 4; /* grid-stride launches over the stuck list */
constexpr int REPO_ROUNDS = 16;    /* parallel resample rounds before the ordered tail */

/* Visit the slots of cells [i0,i1]x[j0,j1]x[k0,k1] (clipped to the grid) in
 * the reference's order; f(slot). */
template <class F>
__device__ __forceinline__ void visit_cells(int n, const uint32_t *__restrict__ cs, int i0,
                                            int i1, int j0, int j1, int k0, int k1, F f) {
  i0 = max(i0, 0);
  i1 = min(i1, n - 1);
  j0 = max(j0, 0);
  j1 = min(j1, n - 1);
  k0 = max(k0, 0);
  k1 = min(k1, n - 1);
  if (k0 > k1) return;
  for (int si = i0; si <= i1; si++)
    for (int sj = j0; sj <= j1; sj++) {
      size_t base = ((size_t)si * n + sj) * n;
      uint32_t s = __ldg(cs + base + k0), e = __ldg(cs + base + k1 + 1);
      for (uint32_t b = s; b < e; b++) f(b);
    }
}

/* visit_cells restricted to a ball of radius sqrt(r2) around (px, py, pz):
 * rows (si, sj) whose cells lie wholly outside the ball are skipped and
 * each row's k-range is trimmed to the cells the ball reaches. A cell's
 * particles lie in its interval [s h, (s+1) h) of each axis, except the
 * first and last cells, which also hold the clamped particles outside the
 * grid (their interval is open on that side). With mid (the lists of
 * FAST arithmetic, each cell's lower z half first), a row's run also
 * starts at the first cell's upper half, or stops before the last cell's
 * upper half, when the ball's z-extent lies wholly on the other side of
 * that cell's mid-plane (k + 0.5) h: the sort placed the particles by an
 * exact compare with that plane. Callers pass r2 a little above their own
 * cut-off (the corrector's reach), so every particle that passes their
 * exact distance test is visited, in the same order. */
template <class F>
__device__ __forceinline__ void visit_ball(int n, float fn, float h, const uint32_t *__restrict__ cs,
                                           const uint32_t *__restrict__ mid, float px, float py,
                                           float pz, float r2, int i0, int i1, int j0, int j1,
                                           int k0, int k1, F f) {
  i0 = max(i0, 0);
  i1 = min(i1, n - 1);
  j0 = max(j0, 0);
  j1 = min(j1, n - 1);
  k0 = max(k0, 0);
  k1 = min(k1, n - 1);
  if (k0 > k1) return;
  auto gap = [&](float p, int s) -> float {
    const float lo = s == 0 ? -INFINITY : (float)s * h;
    const float hi = s == n - 1 ? INFINITY : (float)(s + 1) * h;
    return fmaxf(0.0f, fmaxf(lo - p, p - hi));
  };
  for (int si = i0; si <= i1; si++) {
    const float gx = gap(px, si), gx2 = gx * gx;
    if (gx2 > r2) continue;
    for (int sj = j0; sj <= j1; sj++) {
      const float gy = gap(py, sj), g2 = gx2 + gy * gy;
      if (g2 > r2) continue;
      const float rem = sqrtf(r2 - g2);
      const int ka = max(k0, (int)floorf(fn * (pz - rem))), kb = min(k1, (int)floorf(fn * (pz + rem)));
      if (ka > kb) continue;
      const size_t base = ((size_t)si * n + sj) * n;
      uint32_t s = __ldg(cs + base + ka), e = __ldg(cs + base + kb + 1);
      if (mid) {
        if (pz - rem >= ((float)ka + 0.5f) * h) s = __ldg(mid + base + ka);
        if (pz + rem < ((float)kb + 0.5f) * h) e = __ldg(mid + base + kb);
      }
      for (uint32_t b = s; b < e; b++) f(b);
    }
  }
}

/* linear() (src/mapper.cpp:96-106) with the k clamp of the reference (h-2);
 * k+1 is kept inside the row where the reference reads one past it. */
__device__ __forceinline__ float linear(const float *__restrict__ q, float x, float y, float z,
                                        int w, int h, int d) {
  x = fmaxf(0.0f, fminf((float)w, x));
  y = fmaxf(0.0f, fminf((float)h, y));
  z = fmaxf(0.0f, fminf((float)d, z));
  int i = (int)((x > (float)(w - 2)) ? (float)(w - 2) : x);
  int j = (int)((y > (float)(h - 2)) ? (float)(h - 2) : y);
  int k = (int)((z > (float)(h - 2)) ? (float)(h - 2) : z);
  int k1 = min(k + 1, d - 1);
  auto Q = [&](int a, int b, int c) { return __ldg(q + ((size_t)a * h + b) * d + c); };
  float fx0 = (float)(i + 1) - x, fx1 = x - (float)i;
  float fy0 = (float)(j + 1) - y, fy1 = y - (float)j;
  float fz0 = (float)(k + 1) - z, fz1 = z - (float)k;
  return fz0 * ((fx0 * Q(i, j, k) + fx1 * Q(i + 1, j, k)) * fy0 +
                (fx0 * Q(i, j + 1, k) + fx1 * Q(i + 1, j + 1, k)) * fy1) +
         fz1 * ((fx0 * Q(i, j, k1) + fx1 * Q(i + 1, j, k1)) * fy0 +
                (fx0 * Q(i, j + 1, k1) + fx1 * Q(i + 1, j + 1, k1)) * fy1);
}

/* mapper::fetchVelocity (src/mapper.cpp:108-112). gy - 0.5 is exact in
 * double, so one float subtraction rounds it as the reference does. */
__device__ __forceinline__ void fetch_velocity(int n, float fn, const float *__restrict__ u0,
                                               const float *__restrict__ u1,
                                               const float *__restrict__ u2, float x, float y,
                                               float z, float out[3]) {
  float gx = fn * x, gy = fn * y, gz = fn * z;
  out[0] = linear(u0, gx, gy - 0.5f, gz - 0.5f, n + 1, n, n);
  out[1] = linear(u1, gx - 0.5f, gy, gz - 0.5f, n, n + 1, n);
  out[2] = linear(u2, gx - 0.5f, gy - 0.5f, gz, n, n, n + 1);
}

/* ------------------------------------------------------ computeDensity */

template <class AR, int B = BLK>
__global__ void __launch_bounds__(B)
k_density(SimConst c, const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
          const float4 *__restrict__ spos, float *__restrict__ dens,
          float *__restrict__ sdens) {
  int a = blockIdx.x * B + threadIdx.x;
  if (a >= c.np) return;
  float4 P = spos[a];
  uint32_t p = perm[a];
  if (unpack_type(P.w) == CELL_WALL) {
    dens[p] = 1.0f;
    sdens[a] = 1.0f;
    return;
  }
  int ci = cell_clamp(P.x, c.fn, c.n), cj = cell_clamp(P.y, c.fn, c.n),
      ck = cell_clamp(P.z, c.fn, c.n);
  float wsum = 0.0f;
  visit_cells(c.n, cs, ci - 1, ci + 1, cj - 1, cj + 1, ck - 1, ck + 1, [&](uint32_t b) {
    float4 Q = __ldg(spos + b);
    if (unpack_type(Q.w) == CELL_WALL) return;
    float d2 = AR::hypot2(Q.x - P.x, Q.y - P.y, Q.z - P.z);
    wsum += AR::smooth_density(c, d2);
  });
  float d = wsum / c.max_dens;
  dens[p] = d;
  sdens[a] = d;
}

/* ------------------------------------------------------------ mapP2G */

/* One MAC face per thread (src/mapper.cpp:17-88). The reference gathers
 * cells [i-1,i] along the normal and [j-2,j+1] along each tangent; the
 * tangent cell j-2 lies at least 1.5 cells from the face centre, beyond the
 * kernel radius RE=1.4, so its weights are exactly 0 and it is skipped.
 * Writes the saved grid (save_grid) and the boundary-enforced grid
 * (enforce_boundary, src/flip3D.cpp:783-805) in one pass. */
template <class AR>
__global__ void __launch_bounds__(BLK)
k_p2g(SimConst c, int enforce, const uint32_t *__restrict__ cs, const float4 *__restrict__ spg,
      const float4 *__restrict__ svel, const uint8_t *__restrict__ A, float *__restrict__ u0,
      float *__restrict__ u1, float *__restrict__ u2, float *__restrict__ us0,
      float *__restrict__ us1, float *__restrict__ us2) {
  const int n = c.n;
  /* consecutive blocks take the three components of the same face range,
   * so the particles of a region are read from DRAM once and reused from L2
   * by all three (one component after another re-read them per component) */
  const int comp = (int)(blockIdx.x % 3u);
  size_t f = (size_t)(blockIdx.x / 3u) * BLK + threadIdx.x;
  const size_t nf = (size_t)(n + 1) * n * n;
  if (f >= nf) return;
  const int ex[3] = {comp == 0 ? n + 1 : n, comp == 1 ? n + 1 : n, comp == 2 ? n + 1 : n};
  int i, j, k;
  decode_index(f, ex[1], ex[2], i, j, k);
  float fp[3] = {(float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f};
  int lo[3] = {i - 1, j - 1, k - 1}, hi[3] = {i + 1, j + 1, k + 1};
  if (comp == 0) { fp[0] = (float)i; hi[0] = i; }
  if (comp == 1) { fp[1] = (float)j; hi[1] = j; }
  if (comp == 2) { fp[2] = (float)k; hi[2] = k; }
  const float hh = c.re_p2g_hh;
  float sumw = 0.0f, sumx = 0.0f;
  visit_cells(n, cs, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], [&](uint32_t b) {
    float4 Q = __ldg(spg + b);
    if (unpack_type(Q.w) != CELL_FLUID) return;
    float r2 = AR::hypot2(Q.x - fp[0], Q.y - fp[1], Q.z - fp[2]);
    if (!(r2 < hh)) return; /* weight exactly 0 */
    float w = AR::sharp(r2, hh, c.r2_floor, c.sharp_small_p2g);
    float4 V = __ldg(svel + b);
    float vc = comp == 0 ? V.x : (comp == 1 ? V.y : V.z);
    sumx += w * vc;
    sumw += w;
  });
  float val = (sumw != 0.0f) ? sumx / sumw : 0.0f;
  /* enforce_boundary */
  int a = comp == 0 ? i : (comp == 1 ? j : k);
  float out = val;
  if (!enforce) {
  } else if (a == 0 || a == n) {
    out = 0.0f;
  } else {
    size_t c1 = cell_id(n, i, j, k);
    size_t c0 = comp == 0 ? cell_id(n, i - 1, j, k)
                          : (comp == 1 ? cell_id(n, i, j - 1, k) : cell_id(n, i, j, k - 1));
    bool w1 = A[c1] == CELL_WALL, w0 = A[c0] == CELL_WALL;
    if (w1 != w0) out = 0.0f;
  }
  float *u = comp == 0 ? u0 : (comp == 1 ? u1 : u2);
  float *us = comp == 0 ? us0 : (comp == 1 ? us1 : us2);
  us[f] = val;
  u[f] = out;
}

/* ----------------------------------------------------- mapG2P / FLIP */

/* mapper::mapG2P (src/mapper.cpp:90-94) for every particle, walls included,
 * as the reference does (the step itself skips walls: no stage reads their
 * velocity). */
__global__ void __launch_bounds__(BLK)
k_g2p(SimConst c, const float *__restrict__ px, const float *__restrict__ py,
      const float *__restrict__ pz, const uint8_t *__restrict__ type,
      const float *__restrict__ u0, const float *__restrict__ u1,
      const float *__restrict__ u2, float *__restrict__ vx, float *__restrict__ vy,
      float *__restrict__ vz) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= c.np) return;
  (void)type;
  float v[3];
  fetch_velocity(c.n, c.fn, u0, u1, u2, px[p], py[p], pz[p], v);
  vx[p] = v[0];
  vy[p] = v[1];
  vz[p] = v[2];
}

/* The FLIP block of solve_picflip (src/flip3D.cpp:1071-1097): sample the
 * grid change and the new grid, then u = (1-ALPHA)*pic + ALPHA*(u + du). */
template <class AR>
__global__ void __launch_bounds__(BLK)
k_flip_blend(SimConst c, const float *__restrict__ px, const float *__restrict__ py,
             const float *__restrict__ pz, const uint8_t *__restrict__ type,
             const float *__restrict__ u0, const float *__restrict__ u1,
             const float *__restrict__ u2, const float *__restrict__ d0,
             const float *__restrict__ d1, const float *__restrict__ d2,
             float *__restrict__ vx, float *__restrict__ vy, float *__restrict__ vz) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= c.np || type[p] != CELL_FLUID) return;
  float x = px[p], y = py[p], z = pz[p];
  float du[3], pic[3];
  fetch_velocity(c.n, c.fn, d0, d1, d2, x, y, z, du);
  fetch_velocity(c.n, c.fn, u0, u1, u2, x, y, z, pic);
  float v[3] = {vx[p], vy[p], vz[p]};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    float flip = du[q] + v[q];
    v[q] = AR::blend(c, pic[q], flip);
  }
  vx[p] = v[0];
  vy[p] = v[1];
  vz[p] = v[2];
}

/* ----------------------------------------------------- advect_particle */

/* advect_particle (src/flip3D.cpp:877-969) for one fluid particle: Euler
 * step through the grid velocity vg sampled at pp, clamp inside the walls,
 * push out of wall particles closer than 1.5*DENSITY/N and drop the normal
 * component of the particle velocity uu, then flag it if it is stuck. Each
 * particle only reads itself and the (static) wall particles, so the
 * reference's serial loop is order-independent. */
template <class AR>
__device__ __forceinline__ void advect_one(const SimConst &c, int p, float pp[3], const float vg[3],
                                           float uu[3], float *__restrict__ px,
                                           float *__restrict__ py, float *__restrict__ pz,
                                           float *__restrict__ vx, float *__restrict__ vy,
                                           float *__restrict__ vz, const float *__restrict__ dens,
                                           const uint8_t *__restrict__ A,
                                           const uint32_t *__restrict__ wall_start,
                                           const float4 *__restrict__ wall_pos,
                                           const float4 *__restrict__ wall_nrm,
                                           uint8_t *__restrict__ stuck) {
  const int n = c.n;
#pragma unroll
  for (int q = 0; q < 3; q++) pp[q] = AR::euler(c, pp[q], vg[q]);
  /* p = fmax(r, fmin(1.0-r, p)) */
#pragma unroll
  for (int q = 0; q < 3; q++) {
    float t = pp[q];
    if (t != t || t > c.wall_hi_thr) t = c.wall_hi;
    if (t < c.wall_r) t = c.wall_r;
    pp[q] = t;
  }
  int i = cell_clamp_minmax(pp[0], c.fn, n), j = cell_clamp_minmax(pp[1], c.fn, n),
      k = cell_clamp_minmax(pp[2], c.fn, n);
  visit_cells(n, wall_start, i - 1, i + 1, j - 1, j + 1, k - 1, k + 1, [&](uint32_t w) {
    float4 Q = __ldg(wall_pos + w);
    float dist = AR::length(pp[0] - Q.x, pp[1] - Q.y, pp[2] - Q.z);
    if (!(dist <= c.push_re_thr)) return; /* (double)dist < 1.5*DENSITY/N */
    float4 Nw = __ldg(wall_nrm + w);
    float nrm[3] = {Nw.x, Nw.y, Nw.z};
    if (nrm[0] == 0.0f && nrm[1] == 0.0f && nrm[2] == 0.0f && dist != 0.0f) {
      nrm[0] = (pp[0] - Q.x) / dist;
      nrm[1] = (pp[1] - Q.y) / dist;
      nrm[2] = (pp[2] - Q.z) / dist;
    }
#pragma unroll
    for (int q = 0; q < 3; q++) pp[q] = AR::push(c, pp[q], dist, nrm[q]);
    float dot = uu[0] * nrm[0] + uu[1] * nrm[1] + uu[2] * nrm[2];
#pragma unroll
    for (int q = 0; q < 3; q++) uu[q] -= dot * nrm[q];
  });
  px[p] = pp[0];
  py[p] = pp[1];
  pz[p] = pp[2];
  vx[p] = uu[0];
  vy[p] = uu[1];
  vz[p] = uu[2];
  /* stuck detection (src/flip3D.cpp:933-955) */
  uint8_t s = 0;
  int ai = cell_clamp_minmax(pp[0], c.fn, n), aj = cell_clamp_minmax(pp[1], c.fn, n),
      ak = cell_clamp_minmax(pp[2], c.fn, n);
  if (A[cell_id(n, ai, aj, ak)] == CELL_WALL) s = 1;
  int si = (int)fminf((float)(n - 3), fmaxf(2.0f, pp[0] * c.fn));
  int sj = (int)fminf((float)(n - 3), fmaxf(2.0f, pp[1] * c.fn));
  int sk = (int)fminf((float)(n - 3), fmaxf(2.0f, pp[2] * c.fn));
  if ((double)dens[p] < 0.04 && (A[cell_id(n, si, max(0, sj - 1), sk)] == CELL_WALL ||
                                 A[cell_id(n, si, min(n - 1, sj + 1), sk)] == CELL_WALL))
    s = 1;
  stuck[p] = s;
}

template <class AR>
__global__ void __launch_bounds__(BLK)
k_advect(SimConst c, float *__restrict__ px, float *__restrict__ py, float *__restrict__ pz,
         float *__restrict__ vx, float *__restrict__ vy, float *__restrict__ vz,
         const uint8_t *__restrict__ type, const float *__restrict__ dens,
         const float *__restrict__ u0, const float *__restrict__ u1,
         const float *__restrict__ u2, const uint8_t *__restrict__ A,
         const uint32_t *__restrict__ wall_start, const float4 *__restrict__ wall_pos,
         const float4 *__restrict__ wall_nrm, uint8_t *__restrict__ stuck) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= c.np) return;
  if (type[p] != CELL_FLUID) {
    stuck[p] = 0;
    return;
  }
  float pp[3] = {px[p], py[p], pz[p]};
  float v[3];
  fetch_velocity(c.n, c.fn, u0, u1, u2, pp[0], pp[1], pp[2], v);
  float uu[3] = {vx[p], vy[p], vz[p]};
  advect_one<AR>(c, p, pp, v, uu, px, py, pz, vx, vy, vz, dens, A, wall_start, wall_pos,
                 wall_nrm, stuck);
}

/* The FLIP blend of solve_picflip (src/flip3D.cpp:1071-1097) fused with
 * advect_particle (src/flip3D.cpp:877-969): both sample the new grid at the
 * particle's position before it moves, so one sample serves the PIC term of
 * the blend and the Euler step. The results equal k_flip_blend followed by
 * k_advect. */
template <class AR>
__global__ void __launch_bounds__(BLK)
k_flip_advect(SimConst c, float *__restrict__ px, float *__restrict__ py, float *__restrict__ pz,
              float *__restrict__ vx, float *__restrict__ vy, float *__restrict__ vz,
              const uint8_t *__restrict__ type, const float *__restrict__ dens,
              const float *__restrict__ u0, const float *__restrict__ u1,
              const float *__restrict__ u2, const float *__restrict__ d0,
              const float *__restrict__ d1, const float *__restrict__ d2,
              const uint8_t *__restrict__ A, const uint32_t *__restrict__ wall_start,
              const float4 *__restrict__ wall_pos, const float4 *__restrict__ wall_nrm,
              uint8_t *__restrict__ stuck) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= c.np) return;
  if (type[p] != CELL_FLUID) {
    stuck[p] = 0;
    return;
  }
  float pp[3] = {px[p], py[p], pz[p]};
  float du[3], pic[3];
  fetch_velocity(c.n, c.fn, d0, d1, d2, pp[0], pp[1], pp[2], du);
  fetch_velocity(c.n, c.fn, u0, u1, u2, pp[0], pp[1], pp[2], pic);
  float uu[3] = {vx[p], vy[p], vz[p]};
#pragma unroll
  for (int q = 0; q < 3; q++) uu[q] = AR::blend(c, pic[q], du[q] + uu[q]);
  advect_one<AR>(c, p, pp, pic, uu, px, py, pz, vx, vy, vz, dens, A, wall_start, wall_pos,
                 wall_nrm, stuck);
}

/* ------------------------------------------------------------ reposition */

/* Deep-water cells: FLUID with every in-range face neighbour FLUID
 * (src/flip3D.cpp:412-421). */
/* cnt[0 .. m] = 0 for the m stuck particles (the shuffle's live counts) */
__global__ void k_zero_live(const int *__restrict__ m, uint32_t *__restrict__ cnt) {
  const int e = *m;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= e; q += gridDim.x * blockDim.x)
    cnt[q] = 0u;
}

/* reposition (src/flip3D.cpp:405-441): the first m deep-water cells in cell
 * order (repeated when there are fewer), shuffled by my_rand_shuffle
 * (src/utility.cpp:28-30) — here the keyed Fisher-Yates: for i = m-1 .. 1
 * swap(a[i], a[j_i]) with j_i = draw(i) % (i+1).
 *
 * The swaps run in parallel. Step i is the last to touch position i, so
 * a[i] ends with whatever position j_i held just before step i; that value
 * was put there by the most recent earlier step s > i with j_s = j_i (the
 * smallest such s), which took it from position s just before step s, and
 * so on back to an untouched original entry. lists[p] holds the steps s with
 * j_s = p in ascending order; each output follows its chain of lookups. */
__global__ void k_shuffle_draws(SimConst c, const int *__restrict__ counts,
                                uint32_t *__restrict__ draw, uint32_t *__restrict__ cnt) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  for (int q = 1 + blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    uint32_t r = flip_rand31(c.seed, flip_stream(FLIP_RNG_SHUFFLE, (uint64_t)*c.dstep, 0),
                             (uint64_t)q, 0);
    uint32_t j = r % (uint32_t)(q + 1);
    draw[q] = j;
    atomicAdd(cnt + j, 1u);
  }
}

__global__ void k_shuffle_fill(const int *__restrict__ counts, const uint32_t *__restrict__ draw,
                               const uint32_t *__restrict__ start, uint32_t *__restrict__ cnt,
                               uint32_t *__restrict__ list) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  for (int q = 1 + blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    const uint32_t j = draw[q];
    list[start[j] + atomicSub(cnt + j, 1u) - 1u] = (uint32_t)q;
  }
}

/* each list ascending (lists are short: about ln(m/p) entries) */
__global__ void k_shuffle_sort(const int *__restrict__ counts, const uint32_t *__restrict__ start,
                               uint32_t *__restrict__ list) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
    const uint32_t s = start[p], e = start[p + 1];
    for (uint32_t a = s + 1; a < e; a++) {
      const uint32_t v = list[a];
      uint32_t b = a;
      while (b > s && list[b - 1] > v) {
        list[b] = list[b - 1];
        b--;
      }
      list[b] = v;
    }
  }
}

/* smallest step s > t with j_s = p, or m when there is none */
__device__ __forceinline__ uint32_t first_after(const uint32_t *__restrict__ start,
                                                const uint32_t *__restrict__ list, uint32_t p,
                                                uint32_t t, uint32_t m) {
  uint32_t lo = start[p], hi = start[p + 1];
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (list[mid] > t) hi = mid;
    else lo = mid + 1;
  }
  return lo < start[p + 1] ? list[lo] : m;
}

/* original index of the value position s holds just before step s */
__device__ __forceinline__ uint32_t held_before(const uint32_t *__restrict__ start,
                                                const uint32_t *__restrict__ list, uint32_t s,
                                                uint32_t m) {
  for (;;) { /* s strictly increases and stays below m */
    const uint32_t nx = first_after(start, list, s, s, m);
    if (nx == m) return s;
    s = nx;
  }
}

__global__ void k_shuffle_resolve(const int *__restrict__ counts,
                                  const uint32_t *__restrict__ draw,
                                  const uint32_t *__restrict__ start,
                                  const uint32_t *__restrict__ list,
                                  const uint32_t *__restrict__ water_idx,
                                  uint32_t *__restrict__ waters) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  const uint32_t um = (uint32_t)m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    uint32_t src;
    const uint32_t ui = (uint32_t)i;
    const uint32_t p = i == 0 ? 0u : draw[i];
    if (p == ui) {
      src = held_before(start, list, ui, um);
    } else {
      const uint32_t s = first_after(start, list, p, ui, um);
      src = s == um ? p : held_before(start, list, s, um);
    }
    waters[i] = water_idx[src % (uint32_t)w];
  }
}

/* Each stuck particle q placed at a keyed spot in cell waters[q]
 * (src/flip3D.cpp:435-441); also records q in rank[particle]. */
__global__ void k_repo_place(SimConst c, const int *__restrict__ counts,
                             const uint32_t *__restrict__ stuck_idx,
                             const uint32_t *__restrict__ waters, uint32_t *__restrict__ rank,
                             float *__restrict__ px, float *__restrict__ py,
                             float *__restrict__ pz) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  const int n = c.n;
  const double h = (double)c.re_repo;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    uint32_t cell = waters[q];
    int cc[3] = {(int)(cell / ((uint32_t)n * n)), (int)((cell / n) % n), (int)(cell % n)};
    float out[3];
    for (int d = 0; d < 3; d++) {
      uint32_t r = flip_rand31(c.seed, flip_stream(FLIP_RNG_PLACE, (uint64_t)*c.dstep, 0),
                               (uint64_t)(3 * q + d), 0);
      double frac = 0.5 * (double)(int)(r % 101) / 100;
      out[d] = (float)(h * ((double)cc[d] + 0.25 + frac));
    }
    uint32_t p = stuck_idx[q];
    px[p] = out[0];
    py[p] = out[1];
    pz[p] = out[2];
    rank[p] = (uint32_t)q;
  }
}

/* corrector::resample (src/corrector.cpp:15-47) at the position of stuck
 * particle q. The reference resamples the stuck particles one after another
 * (src/flip3D.cpp:445-450), so particle q sees the new velocity of every
 * stuck particle q' < q and the old velocity of every q' >= q. `vel_of`
 * supplies a neighbour's velocity under that rule; `dep` is set when a
 * contributing neighbour is a stuck particle q' < q. */
template <class V>
__device__ __forceinline__ float3 repo_resample_one(const SimConst &c, float3 P, uint32_t q,
                                                    const uint32_t *__restrict__ cs,
                                                    const uint32_t *__restrict__ perm,
                                                    const float4 *__restrict__ spos,
                                                    const uint8_t *__restrict__ stuck,
                                                    const uint32_t *__restrict__ rank,
                                                    bool &dep, V vel_of) {
  int ci = cell_clamp(P.x, c.fn, c.n), cj = cell_clamp(P.y, c.fn, c.n),
      ck = cell_clamp(P.z, c.fn, c.n);
  float u[3] = {0.0f, 0.0f, 0.0f};
  float wsum = 0.0f;
  visit_cells(c.n, cs, ci - 1, ci + 1, cj - 1, cj + 1, ck - 1, ck + 1, [&](uint32_t b) {
    float4 Q = spos[b];
    if (unpack_type(Q.w) != CELL_FLUID) return;
    float d2 = hypot2_ref(P.x - Q.x, P.y - Q.y, P.z - Q.z);
    if (!(d2 < c.re_repo_hh)) return; /* weight exactly 0 */
    float wt = sharp_ref(d2, c.re_repo_hh, c.r2_floor, c.sharp_small_repo);
    uint32_t o = perm[b];
    bool is_stuck = stuck[o] != 0;
    uint32_t ro = is_stuck ? rank[o] : 0xffffffffu;
    if (is_stuck && ro < q) dep = true;
    float3 v = vel_of(o, is_stuck, ro);
    u[0] += wt * v.x;
    u[1] += wt * v.y;
    u[2] += wt * v.z;
    wsum += wt;
  });
  if (wsum != 0.0f) {
    u[0] /= wsum;
    u[1] /= wsum;
    u[2] /= wsum;
  }
  return make_float3(u[0], u[1], u[2]);
}

/* Round 0: every stuck particle with the velocities before the resample.
 * A particle with no earlier stuck particle among its contributing
 * neighbours has its final value (state READY); the others stay PENDING for
 * the later rounds. old[q] keeps the velocity before the resample. */
enum { RP_PENDING = 0, RP_DONE = 1, RP_READY = 2 };

__global__ void k_repo_gather(SimConst c, const int *__restrict__ counts,
                              const uint32_t *__restrict__ stuck_idx,
                              const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
                              const float4 *__restrict__ spos, const uint8_t *__restrict__ stuck,
                              const uint32_t *__restrict__ rank, const float *__restrict__ px,
                              const float *__restrict__ py, const float *__restrict__ pz,
                              const float *__restrict__ vx, const float *__restrict__ vy,
                              const float *__restrict__ vz, float4 *__restrict__ res,
                              float4 *__restrict__ old, uint8_t *__restrict__ state,
                              int *__restrict__ left) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    uint32_t p = stuck_idx[q];
    float3 P = make_float3(px[p], py[p], pz[p]);
    bool dep = false;
    float3 u = repo_resample_one(c, P, (uint32_t)q, cs, perm, spos, stuck, rank, dep,
                                 [&](uint32_t o, bool, uint32_t) {
                                   return make_float3(vx[o], vy[o], vz[o]);
                                 });
    res[q] = make_float4(u.x, u.y, u.z, 0.0f);
    old[q] = make_float4(vx[p], vy[p], vz[p], 0.0f);
    state[q] = dep ? RP_PENDING : RP_READY;
    if (dep) atomicAdd(left, 1);
  }
}

/* Later rounds: a PENDING particle whose earlier stuck neighbours are all
 * DONE computes its value — new velocities for stuck q' < q, old ones for
 * q' > q — and becomes READY. */
__global__ void k_repo_round(SimConst c, const int *__restrict__ counts,
                             const uint32_t *__restrict__ stuck_idx,
                             const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
                             const float4 *__restrict__ spos, const uint8_t *__restrict__ stuck,
                             const uint32_t *__restrict__ rank, const float *__restrict__ px,
                             const float *__restrict__ py, const float *__restrict__ pz,
                             const float *__restrict__ vx, const float *__restrict__ vy,
                             const float *__restrict__ vz, float4 *__restrict__ res,
                             const float4 *__restrict__ old, uint8_t *__restrict__ state,
                             const int *__restrict__ left) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0 || *left == 0) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    if (state[q] != RP_PENDING) continue;
    uint32_t p = stuck_idx[q];
    float3 P = make_float3(px[p], py[p], pz[p]);
    bool dep = false, blocked = false;
    float3 u = repo_resample_one(c, P, (uint32_t)q, cs, perm, spos, stuck, rank, dep,
                                 [&](uint32_t o, bool is_stuck, uint32_t ro) {
                                   if (is_stuck && ro >= (uint32_t)q) {
                                     float4 v = old[ro];
                                     return make_float3(v.x, v.y, v.z);
                                   }
                                   if (is_stuck && state[ro] != RP_DONE) blocked = true;
                                   return make_float3(vx[o], vy[o], vz[o]);
                                 });
    if (blocked) continue;
    res[q] = make_float4(u.x, u.y, u.z, 0.0f);
    state[q] = RP_READY;
  }
}

__global__ void k_repo_commit(const int *__restrict__ counts,
                              const uint32_t *__restrict__ stuck_idx,
                              const float4 *__restrict__ res, uint8_t *__restrict__ state,
                              float *__restrict__ vx, float *__restrict__ vy,
                              float *__restrict__ vz, int *__restrict__ left, int round) {
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0 || (round > 0 && *left == 0)) return;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
    if (state[q] != RP_READY) continue;
    float4 r = res[q];
    uint32_t p = stuck_idx[q];
    vx[p] = r.x;
    vy[p] = r.y;
    vz[p] = r.z;
    state[q] = RP_DONE;
    if (round > 0) atomicSub(left, 1);
  }
}

/* Whatever is still PENDING after the rounds, in increasing q on one
 * thread: every earlier stuck particle is final by then. */
__global__ void k_repo_ordered(SimConst c, const int *__restrict__ counts,
                               const uint32_t *__restrict__ stuck_idx,
                               const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
                               const float4 *__restrict__ spos, const uint8_t *__restrict__ stuck,
                               const uint32_t *__restrict__ rank, const float *__restrict__ px,
                               const float *__restrict__ py, const float *__restrict__ pz,
                               float *__restrict__ vx, float *__restrict__ vy,
                               float *__restrict__ vz, const float4 *__restrict__ old,
                               const uint8_t *__restrict__ state, const int *__restrict__ left) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int m = counts[IF_NSTUCK], w = counts[IF_NWATER];
  if (w == 0 || *left == 0) return;
  for (int q = 0; q < m; q++) {
    if (state[q] == RP_DONE) continue;
    uint32_t p = stuck_idx[q];
    float3 P = make_float3(px[p], py[p], pz[p]);
    bool dep = false;
    float3 u = repo_resample_one(c, P, (uint32_t)q, cs, perm, spos, stuck, rank, dep,
                                 [&](uint32_t o, bool is_stuck, uint32_t ro) {
                                   if (is_stuck && ro >= (uint32_t)q) {
                                     float4 v = old[ro];
                                     return make_float3(v.x, v.y, v.z);
                                   }
                                   return make_float3(vx[o], vy[o], vz[o]);
                                 });
    vx[p] = u.x;
    vy[p] = u.y;
    vz[p] = u.z;
  }
}

/* ------------------------------------------------------ corrector */

/* Cells that can hold a particle within `reach` (world units) of p along one
 * axis, intersected with the reference's neighbourhood [c0-1, c0+1]. A
 * particle q lies in cell clamp(floor(n*q), 0, n-1), so one within reach lies
 * in clamp(floor(n(p-reach')), 0, n-1) .. clamp(floor(n(p+reach')), 0, n-1);
 * reach' carries a 2^-8 margin against rounding. */
__device__ __forceinline__ void reach_range(float p, float reach_m, float fn, int n, int c0,
                                            int &lo, int &hi) {
  int a = min(max((int)floorf(fn * (p - reach_m)), 0), n - 1);
  int b = min(max((int)floorf(fn * (p + reach_m)), 0), n - 1);
  lo = max(c0 - 1, a);
  hi = min(c0 + 1, b);
}

constexpr int NEAR_CAP = 24; /* near-list batch per thread */

/* The corrector's kicks (src/corrector.cpp:74-81) in the reference's double
 * arithmetic, out of line (rare branches; see refmath.h on FP64 hoisting).
 * k = 0.01*re/dt or 0.05*re/dt, precomputed on the host. */
__device__ __noinline__ float kick_add(float s, double k, int draw) {
  return (float)((double)s + k * (double)draw / 100.0);
}
__device__ __noinline__ float wall_kick_add(float s, double k, float nrm) {
  return (float)((double)s + k * (double)nrm);
}

/* Spring displacement (src/corrector.cpp:54-100). Two passes per batch: a
 * cheap test collects the neighbours within re*(1+2^-8) into a per-thread
 * list (all other neighbours have weight exactly 0 and add nothing), then
 * the exact arithmetic runs over the list in the same order. Writes the
 * moved position to the canonical arrays; neighbours come from the sorted
 * snapshot. */
template <class AR>
__global__ void __launch_bounds__(BLK)
k_spring(SimConst c, const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
         const float4 *__restrict__ spos, const float *__restrict__ nx,
         const float *__restrict__ ny, const float *__restrict__ nz, float *__restrict__ px,
         float *__restrict__ py, float *__restrict__ pz) {
  __shared__ uint32_t near_list[NEAR_CAP][BLK];
  int a = blockIdx.x * BLK + threadIdx.x;
  bool active = a < c.np;
  float4 P = active ? spos[a] : make_float4(0, 0, 0, 0);
  if (!active || unpack_type(P.w) != CELL_FLUID) return;
  uint32_t p = perm[a];
  const float re = c.re_corr;
  int x = cell_clamp_macro(P.x, c.fn), y = cell_clamp_macro(P.y, c.fn),
      z = cell_clamp_macro(P.z, c.fn);
  int i0, i1, j0, j1, k0, k1;
  reach_range(P.x, c.corr_reach, c.fn, c.n, x, i0, i1);
  reach_range(P.y, c.corr_reach, c.fn, c.n, y, j0, j1);
  reach_range(P.z, c.corr_reach, c.fn, c.n, z, k0, k1);
  float spring[3] = {0.0f, 0.0f, 0.0f};
  int cnt = 0;
  auto flush = [&]() {
    for (int t = 0; t < cnt; t++) {
      uint32_t b = near_list[t][threadIdx.x];
      float4 Q = __ldg(spos + b);
      float dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
      float dist = AR::length(dx, dy, dz);
      float w = 50.0f * AR::smooth_corr(c, dist * dist);
      if (dist > c.corr_near_thr) {
        spring[0] += AR::spring_term(w, dx, dist, re);
        spring[1] += AR::spring_term(w, dy, dist, re);
        spring[2] += AR::spring_term(w, dz, dist, re);
      } else if (unpack_type(Q.w) == CELL_FLUID) {
        uint32_t o = perm[b];
        for (int q = 0; q < 3; q++) {
          uint32_t r = flip_rand31(c.seed, flip_stream(FLIP_RNG_KICK, (uint64_t)*c.dstep, q),
                                   (uint64_t)p, (uint64_t)o);
          spring[q] = kick_add(spring[q], c.kick_fluid, (int)(r % 101));
        }
      } else {
        uint32_t o = perm[b];
        float nn[3] = {nx[o], ny[o], nz[o]};
        for (int q = 0; q < 3; q++) spring[q] = wall_kick_add(spring[q], c.kick_wall, nn[q]);
      }
    }
    cnt = 0;
  };
  visit_cells(c.n, cs, i0, i1, j0, j1, k0, k1, [&](uint32_t b) {
    if (b == (uint32_t)a) return;
    float4 Q = __ldg(spos + b);
    if (AR::hypot2(P.x - Q.x, P.y - Q.y, P.z - Q.z) > c.corr_cut2) return;
    near_list[cnt][threadIdx.x] = b;
    if (++cnt == NEAR_CAP) flush();
  });
  flush();
  px[p] = P.x + c.dt_f * spring[0];
  py[p] = P.y + c.dt_f * spring[1];
  pz[p] = P.z + c.dt_f * spring[2];
}

/* Velocity resample at the moved position (src/corrector.cpp:91-114 with
 * resample at :15-47): the same reach restriction and near list, with the
 * sharp kernel's exact support test r2 < re^2. */
template <class AR>
__global__ void __launch_bounds__(BLK)
k_resample(SimConst c, const uint32_t *__restrict__ cs, const uint32_t *__restrict__ perm,
           const float4 *__restrict__ spos, const float4 *__restrict__ svel,
           const float *__restrict__ px, const float *__restrict__ py,
           const float *__restrict__ pz, float *__restrict__ vx, float *__restrict__ vy,
           float *__restrict__ vz) {
  __shared__ uint32_t near_list[NEAR_CAP][BLK];
  int a = blockIdx.x * BLK + threadIdx.x;
  if (a >= c.np) return;
  if (unpack_type(spos[a].w) != CELL_FLUID) return;
  uint32_t p = perm[a];
  float T[3] = {px[p], py[p], pz[p]};
  int ci = cell_clamp(T[0], c.fn, c.n), cj = cell_clamp(T[1], c.fn, c.n),
      ck = cell_clamp(T[2], c.fn, c.n);
  int i0, i1, j0, j1, k0, k1;
  reach_range(T[0], c.corr_reach, c.fn, c.n, ci, i0, i1);
  reach_range(T[1], c.corr_reach, c.fn, c.n, cj, j0, j1);
  reach_range(T[2], c.corr_reach, c.fn, c.n, ck, k0, k1);
  float u[3] = {0.0f, 0.0f, 0.0f};
  float wsum = 0.0f;
  int cnt = 0;
  auto flush = [&]() {
    for (int t = 0; t < cnt; t++) {
      uint32_t b = near_list[t][threadIdx.x];
      float4 Q = __ldg(spos + b);
      float d2 = AR::hypot2(T[0] - Q.x, T[1] - Q.y, T[2] - Q.z);
      float w = AR::sharp(d2, c.re_corr_hh, c.r2_floor, c.sharp_small_corr);
      float4 V = __ldg(svel + b);
      u[0] += w * V.x;
      u[1] += w * V.y;
      u[2] += w * V.z;
      wsum += w;
    }
    cnt = 0;
  };
  visit_cells(c.n, cs, i0, i1, j0, j1, k0, k1, [&](uint32_t b) {
    float4 Q = __ldg(spos + b);
    if (unpack_type(Q.w) != CELL_FLUID) return;
    float d2 = AR::hypot2(T[0] - Q.x, T[1] - Q.y, T[2] - Q.z);
    if (!(d2 < c.re_corr_hh)) return;
    near_list[cnt][threadIdx.x] = b;
    if (++cnt == NEAR_CAP) flush();
  });
  flush();
  if (wsum != 0.0f) {
    vx[p] = u[0] / wsum;
    vy[p] = u[1] / wsum;
    vz[p] = u[2] / wsum;
  }
}

/* ------------------------------------------- cell-per-thread gathers */

__device__ __forceinline__ void cell_decode(size_t c, int n, int &i, int &j, int &k) {
  const unsigned row = (unsigned)c / (unsigned)n;
  k = (int)(c - (size_t)row * n);
  i = (int)(row / (unsigned)n);
  j = (int)(row - (unsigned)i * n);
}

/* mapP2G (k_p2g's arithmetic and order): one thread per face cell (i, j, k)
 * of the (n+1)^3 lattice computes the three faces there (u0 at (i, j, k)
 * when j, k < n; u1 when i, k < n; u2 when i, j < n). Their neighbourhoods
 * lie in cells [i-1, i+1] x [j-1, j+1] x [k-1, k+1]: each particle there is
 * loaded once and tested against each face whose own cells hold it, which
 * keeps every face's sums in k_p2g's order. */
template <class AR, int B = BLK>
__global__ void __launch_bounds__(B)
k_p2g_cells(SimConst c, int enforce, const uint32_t *__restrict__ cs,
            const float4 *__restrict__ spg, const float4 *__restrict__ svel,
            const uint8_t *__restrict__ A, float *__restrict__ u0, float *__restrict__ u1,
            float *__restrict__ u2, float *__restrict__ us0, float *__restrict__ us1,
            float *__restrict__ us2) {
  const int n = c.n, m1 = n + 1;
  const size_t t = (size_t)blockIdx.x * B + threadIdx.x;
  if (t >= (size_t)m1 * m1 * m1) return;
  int i, j, k;
  cell_decode(t, m1, i, j, k);
  const bool v0 = j < n && k < n, v1 = i < n && k < n, v2 = i < n && j < n;
  const float hh = c.re_p2g_hh;
  const float fi = (float)i, fj = (float)j, fk = (float)k;
  const float hi = fi + 0.5f, hj = fj + 0.5f, hk = fk + 0.5f;
  float sx[3] = {0.0f, 0.0f, 0.0f}, sw[3] = {0.0f, 0.0f, 0.0f};
  const int i0 = max(i - 1, 0), i1 = min(i + 1, n - 1), j0 = max(j - 1, 0),
            j1 = min(j + 1, n - 1), k0 = max(k - 1, 0), k1 = min(k + 1, n - 1);
  if (k0 <= k1) {
    for (int si = i0; si <= i1; si++)
      for (int sj = j0; sj <= j1; sj++) {
        const bool in0 = v0 && si <= i, in1 = v1 && sj <= j, in2 = v2;
        if (!(in0 || in1 || in2)) continue;
        const size_t base = ((size_t)si * n + sj) * n;
        const uint32_t a = __ldg(cs + base + k0), b = __ldg(cs + base + k1 + 1);
        /* u2's cells stop at k: the particles of cell k+1 are not its */
        const uint32_t split = k + 1 <= k1 ? __ldg(cs + base + k + 1) : b;
        for (uint32_t x = a; x < b; x++) {
          const float4 Q = __ldg(spg + x);
          if (unpack_type(Q.w) != CELL_FLUID) continue;
          float w[3] = {0.0f, 0.0f, 0.0f};
          bool acc[3] = {false, false, false};
          if (in0) {
            const float r2 = AR::hypot2(Q.x - fi, Q.y - hj, Q.z - hk);
            if (r2 < hh) {
              acc[0] = true;
              w[0] = AR::sharp(r2, hh, c.r2_floor, c.sharp_small_p2g);
            }
          }
          if (in1) {
            const float r2 = AR::hypot2(Q.x - hi, Q.y - fj, Q.z - hk);
            if (r2 < hh) {
              acc[1] = true;
              w[1] = AR::sharp(r2, hh, c.r2_floor, c.sharp_small_p2g);
            }
          }
          if (in2 && x < split) {
            const float r2 = AR::hypot2(Q.x - hi, Q.y - hj, Q.z - fk);
            if (r2 < hh) {
              acc[2] = true;
              w[2] = AR::sharp(r2, hh, c.r2_floor, c.sharp_small_p2g);
            }
          }
          if (!(acc[0] || acc[1] || acc[2])) continue;
          const float4 V = __ldg(svel + x);
          if (acc[0]) {
            sx[0] += w[0] * V.x;
            sw[0] += w[0];
          }
          if (acc[1]) {
            sx[1] += w[1] * V.y;
            sw[1] += w[1];
          }
          if (acc[2]) {
            sx[2] += w[2] * V.z;
            sw[2] += w[2];
          }
        }
      }
  }
  const bool valid[3] = {v0, v1, v2};
#pragma unroll
  for (int comp = 0; comp < 3; comp++) {
    if (!valid[comp]) continue;
    const float val = (sw[comp] != 0.0f) ? sx[comp] / sw[comp] : 0.0f;
    const int a = comp == 0 ? i : (comp == 1 ? j : k);
    float out = val;
    if (!enforce) {
    } else if (a == 0 || a == n) {
      out = 0.0f;
    } else {
      const size_t cc1 = cell_id(n, i, j, k);
      const size_t cc0 = comp == 0 ? cell_id(n, i - 1, j, k)
                                   : (comp == 1 ? cell_id(n, i, j - 1, k) : cell_id(n, i, j, k - 1));
      if ((__ldg(A + cc1) == CELL_WALL) != (__ldg(A + cc0) == CELL_WALL)) out = 0.0f;
    }
    size_t f;
    float *u, *us;
    if (comp == 0) {
      f = ((size_t)i * n + j) * n + k;
      u = u0;
      us = us0;
    } else if (comp == 1) {
      f = ((size_t)i * m1 + j) * n + k;
      u = u1;
      us = us1;
    } else {
      f = ((size_t)i * n + j) * m1 + k;
      u = u2;
      us = us2;
    }
    us[f] = val;
    u[f] = out;
  }
}

/* The corrector's spring and resample with the near-pair work inline
 * instead of through k_spring's and k_resample's per-thread near lists
 * (which hold 24 KB of shared memory per block); the same pairs in the same
 * order, so the same results. */
/* 1280 resident threads per SM (five blocks of 256): 48 registers (a few
 * spilled) instead of 56; the kernel is issue- and occupancy-bound, and
 * this is 5 % faster at N=256 (six blocks spill more and gain less) */
template <class AR, int B = BLK>
__global__ void __launch_bounds__(B, 1280 / B)
k_spring_inline(SimConst c, const uint32_t *__restrict__ cs, const uint32_t *__restrict__ mid,
                const uint32_t *__restrict__ perm, const float4 *__restrict__ spos,
                const float *__restrict__ nx,
                const float *__restrict__ ny, const float *__restrict__ nz,
                float *__restrict__ px, float *__restrict__ py, float *__restrict__ pz) {
  const int a = blockIdx.x * B + threadIdx.x;
  if (a >= c.np) return;
  const float4 P = __ldg(spos + a);
  if (unpack_type(P.w) != CELL_FLUID) return;
  const uint32_t pid = __ldg(perm + a);
  const float re = c.re_corr;
  const int x = cell_clamp_macro(P.x, c.fn), y = cell_clamp_macro(P.y, c.fn),
            z = cell_clamp_macro(P.z, c.fn);
  int i0, i1, j0, j1, k0, k1;
  reach_range(P.x, c.corr_reach, c.fn, c.n, x, i0, i1);
  reach_range(P.y, c.corr_reach, c.fn, c.n, y, j0, j1);
  reach_range(P.z, c.corr_reach, c.fn, c.n, z, k0, k1);
  float spring[3] = {0.0f, 0.0f, 0.0f};
  const float reach2 = c.corr_reach * c.corr_reach;
  visit_ball(c.n, c.fn, c.h, cs, mid, P.x, P.y, P.z, reach2, i0, i1, j0, j1, k0, k1,
             [&](uint32_t b) {
    if (b == (uint32_t)a) return;
    const float4 Q = __ldg(spos + b);
    if (AR::hypot2(P.x - Q.x, P.y - Q.y, P.z - Q.z) > c.corr_cut2) return;
    const float dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
    const float dist = AR::length(dx, dy, dz);
    const float w = 50.0f * AR::smooth_corr(c, dist * dist);
    if (dist > c.corr_near_thr) {
      spring[0] += AR::spring_term(w, dx, dist, re);
      spring[1] += AR::spring_term(w, dy, dist, re);
      spring[2] += AR::spring_term(w, dz, dist, re);
    } else {
      const uint32_t o = __ldg(perm + b);
      if (unpack_type(Q.w) == CELL_FLUID) {
        for (int d = 0; d < 3; d++) {
          const uint32_t r = flip_rand31(c.seed, flip_stream(FLIP_RNG_KICK, (uint64_t)*c.dstep, d),
                                         (uint64_t)pid, (uint64_t)o);
          spring[d] = kick_add(spring[d], c.kick_fluid, (int)(r % 101));
        }
      } else {
        const float nn[3] = {nx[o], ny[o], nz[o]};
        for (int d = 0; d < 3; d++) spring[d] = wall_kick_add(spring[d], c.kick_wall, nn[d]);
      }
    }
  });
  px[pid] = P.x + c.dt_f * spring[0];
  py[pid] = P.y + c.dt_f * spring[1];
  pz[pid] = P.z + c.dt_f * spring[2];
}

template <class AR, int B = BLK>
__global__ void __launch_bounds__(B)
k_resample_inline(SimConst c, const uint32_t *__restrict__ cs,
                  const uint32_t *__restrict__ mid, const uint32_t *__restrict__ perm,
                  const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                  const float *__restrict__ px, const float *__restrict__ py,
                  const float *__restrict__ pz, float *__restrict__ vx, float *__restrict__ vy,
                  float *__restrict__ vz) {
  const int a = blockIdx.x * B + threadIdx.x;
  if (a >= c.np) return;
  if (unpack_type(__ldg(spos + a).w) != CELL_FLUID) return;
  const uint32_t p = __ldg(perm + a);
  const float T[3] = {px[p], py[p], pz[p]};
  const int ci = cell_clamp(T[0], c.fn, c.n), cj = cell_clamp(T[1], c.fn, c.n),
            ck = cell_clamp(T[2], c.fn, c.n);
  int i0, i1, j0, j1, k0, k1;
  reach_range(T[0], c.corr_reach, c.fn, c.n, ci, i0, i1);
  reach_range(T[1], c.corr_reach, c.fn, c.n, cj, j0, j1);
  reach_range(T[2], c.corr_reach, c.fn, c.n, ck, k0, k1);
  float u[3] = {0.0f, 0.0f, 0.0f};
  float wsum = 0.0f;
  const float reach2 = c.corr_reach * c.corr_reach;
  visit_ball(c.n, c.fn, c.h, cs, mid, T[0], T[1], T[2], reach2, i0, i1, j0, j1, k0, k1,
             [&](uint32_t b) {
    const float4 Q = __ldg(spos + b);
    if (unpack_type(Q.w) != CELL_FLUID) return;
    const float d2 = AR::hypot2(T[0] - Q.x, T[1] - Q.y, T[2] - Q.z);
    if (!(d2 < c.re_corr_hh)) return;
    const float w = AR::sharp(d2, c.re_corr_hh, c.r2_floor, c.sharp_small_corr);
    const float4 V = __ldg(svel + b);
    u[0] += w * V.x;
    u[1] += w * V.y;
    u[2] += w * V.z;
    wsum += w;
  });
  if (wsum != 0.0f) {
    vx[p] = u[0] / wsum;
    vy[p] = u[1] / wsum;
    vz[p] = u[2] / wsum;
  }
}

/* mapper::fetchVelocity at arbitrary points (AoS in and out). */
__global__ void k_fetch_points(SimConst c, int count, const float *__restrict__ pts,
                               const float *__restrict__ u0, const float *__restrict__ u1,
                               const float *__restrict__ u2, float *__restrict__ out) {
  int t = blockIdx.x * BLK + threadIdx.x;
  if (t >= count) return;
  float v[3];
  fetch_velocity(c.n, c.fn, u0, u1, u2, pts[3 * (size_t)t], pts[3 * (size_t)t + 1],
                 pts[3 * (size_t)t + 2], v);
  out[3 * (size_t)t] = v[0];
  out[3 * (size_t)t + 1] = v[1];
  out[3 * (size_t)t + 2] = v[2];
}

/* corrector::resample (src/corrector.cpp:15-47) at arbitrary points; each
 * point only reads the sorted snapshot, so points are independent. */
__global__ void k_resample_points(SimConst c, int count, const float *__restrict__ pts,
                                  float *__restrict__ vel, float re_hh, float small,
                                  const uint32_t *__restrict__ cs,
                                  const float4 *__restrict__ spos,
                                  const float4 *__restrict__ svel) {
  int t = blockIdx.x * BLK + threadIdx.x;
  if (t >= count) return;
  float P[3] = {pts[3 * (size_t)t], pts[3 * (size_t)t + 1], pts[3 * (size_t)t + 2]};
  int ci = cell_clamp(P[0], c.fn, c.n), cj = cell_clamp(P[1], c.fn, c.n),
      ck = cell_clamp(P[2], c.fn, c.n);
  float u[3] = {0.0f, 0.0f, 0.0f};
  float wsum = 0.0f;
  visit_cells(c.n, cs, ci - 1, ci + 1, cj - 1, cj + 1, ck - 1, ck + 1, [&](uint32_t b) {
    float4 Q = __ldg(spos + b);
    if (unpack_type(Q.w) != CELL_FLUID) return;
    float d2 = hypot2_ref(P[0] - Q.x, P[1] - Q.y, P[2] - Q.z);
    if (!(d2 < re_hh)) return;
    float w = sharp_ref(d2, re_hh, c.r2_floor, small);
    float4 V = __ldg(svel + b);
    u[0] += w * V.x;
    u[1] += w * V.y;
    u[2] += w * V.z;
    wsum += w;
  });
  if (wsum != 0.0f) {
    vel[3 * (size_t)t] = u[0] / wsum;
    vel[3 * (size_t)t + 1] = u[1] / wsum;
    vel[3 * (size_t)t + 2] = u[2] / wsum;
  }
}

} // namespace

cudaError_t launch_fetch_points(FlipGpu *h, int count, const float *pts, float *out) {
  if (count == 0) return cudaSuccess;
  SimConst c = make_const(h);
  k_fetch_points<<<grid_for(count, BLK), BLK, 0, h->stream>>>(c, count, pts, h->u[0], h->u[1],
                                                              h->u[2], out);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_resample_points(FlipGpu *h, int count, const float *pts, float *vel,
                                   float re) {
  if (count == 0) return cudaSuccess;
  SimConst c = make_const(h);
  float hh = re * re;
  float small = (float)fmax((double)hh / 1.0e-5 - 1.0, 0.0);
  k_resample_points<<<grid_for(count, BLK), BLK, 0, h->stream>>>(
      c, count, pts, vel, hh, small, h->cell_start, h->spos, h->svel);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

/* FAST arithmetic runs the gathers restructured for speed (P2G with one
 * thread per face cell, the corrector without near lists);
 * FLIPGPU_GATHER=particle in the environment selects the per-particle
 * kernels instead (read at each launch, so one process can compare the two:
 * the results are identical) */
static bool cell_gathers(const FlipGpu *h) {
  if (h->prm.arith != FLIPGPU_ARITH_FAST) return false;
  const char *e = getenv("FLIPGPU_GATHER");
  return !(e && strcmp(e, "particle") == 0);
}

/* The FAST gathers' block size, tuned per kernel and problem size (key: the
 * kernel, N and the power of two at or above its thread count) over 256
 * (the default, and the choice while a stream is being captured or an
 * asynchronous step runs), 128 and 512 threads. Every thread computes one
 * particle's or face cell's sums on its own, so the results do not depend
 * on the choice; each kernel only writes outputs that it does not read, so
 * the tuner's repeated launches leave the same state. FLIPGPU_GATHER_BLOCK
 * = 128, 256 or 512 in the environment (read at each launch) fixes it. */
template <class L>
static cudaError_t tuned_gather(FlipGpu *h, const char *kernel, size_t threads, L launch) {
  auto run = [&](int i) -> cudaError_t {
    if (i == 1)
      launch(std::integral_constant<int, 128>{});
    else if (i == 2)
      launch(std::integral_constant<int, 512>{});
    else
      launch(std::integral_constant<int, 256>{});
    return cudaGetLastError();
  };
  const char *e = getenv("FLIPGPU_GATHER_BLOCK");
  int pick = 0;
  if (e && e[0]) {
    const int b = atoi(e);
    pick = b == 128 ? 1 : (b == 512 ? 2 : 0);
  } else {
    int lg = 0;
    while (((size_t)1 << lg) < threads) lg++;
    char key[96];
    snprintf(key, sizeof key, "%s block n=%d threads<=2^%d", kernel, h->n, lg);
    static const std::vector<std::string> names = {"256", "128", "512"};
    pick = h->async_mode ? autotune::cached(key) : autotune::choose(key, names, h->stream, run);
  }
  ktime_begin(h, kernel);
  cudaError_t err = run(pick);
  ktime_end(h);
  FG_LAUNCHED(h, 1);
  return err;
}

cudaError_t launch_density(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  if (h->prm.arith == FLIPGPU_ARITH_FAST)
    return tuned_gather(h, "k_density", h->np, [&](auto B) {
      constexpr int b = decltype(B)::value;
      k_density<FastArith, b><<<grid_for(h->np, b), b, 0, h->stream>>>(
          c, h->cell_start, h->perm, h->spos, h->dens, h->sdens);
    });
  k_density<RefArith><<<grid_for(h->np, BLK), BLK, 0, h->stream>>>(c, h->cell_start, h->perm,
                                                                   h->spos, h->dens, h->sdens);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_p2g(FlipGpu *h, int enforce) {
  SimConst c = make_const(h);
  if (cell_gathers(h)) {
    const size_t m1 = (size_t)h->n + 1, cells = m1 * m1 * m1;
    return tuned_gather(h, "k_p2g_cells", cells, [&](auto B) {
      constexpr int b = decltype(B)::value;
      k_p2g_cells<FastArith, b><<<grid_for(cells, b), b, 0, h->stream>>>(
          c, enforce, h->cell_start, h->spg, h->svel, h->A, h->u[0], h->u[1], h->u[2], h->us[0],
          h->us[1], h->us[2]);
    });
  }
  const unsigned grid = 3u * grid_for(h->nf, BLK);
  if (h->prm.arith == FLIPGPU_ARITH_FAST)
    k_p2g<FastArith><<<grid, BLK, 0, h->stream>>>(c, enforce, h->cell_start, h->spg, h->svel,
                                                  h->A, h->u[0], h->u[1], h->u[2], h->us[0],
                                                  h->us[1], h->us[2]);
  else
    k_p2g<RefArith><<<grid, BLK, 0, h->stream>>>(c, enforce, h->cell_start, h->spg, h->svel,
                                                 h->A, h->u[0], h->u[1], h->u[2], h->us[0],
                                                 h->us[1], h->us[2]);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_g2p(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  k_g2p<<<grid_for(h->np, BLK), BLK, 0, h->stream>>>(c, h->px, h->py, h->pz, h->type, h->u[0],
                                                     h->u[1], h->u[2], h->vx, h->vy, h->vz);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_flip_blend(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  const unsigned g = grid_for(h->np, BLK);
  if (h->prm.arith == FLIPGPU_ARITH_FAST)
    k_flip_blend<FastArith><<<g, BLK, 0, h->stream>>>(c, h->px, h->py, h->pz, h->type, h->u[0],
                                                      h->u[1], h->u[2], h->us[0], h->us[1],
                                                      h->us[2], h->vx, h->vy, h->vz);
  else
    k_flip_blend<RefArith><<<g, BLK, 0, h->stream>>>(c, h->px, h->py, h->pz, h->type, h->u[0],
                                                     h->u[1], h->u[2], h->us[0], h->us[1],
                                                     h->us[2], h->vx, h->vy, h->vz);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_flip_advect(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  const unsigned g = grid_for(h->np, BLK);
  ktime_begin(h, "k_flip_advect");
  if (h->prm.arith == FLIPGPU_ARITH_FAST)
    k_flip_advect<FastArith><<<g, BLK, 0, h->stream>>>(
        c, h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->type, h->dens, h->u[0], h->u[1], h->u[2],
        h->us[0], h->us[1], h->us[2], h->A, h->wall_start, h->wall_pos, h->wall_nrm, h->flag);
  else
    k_flip_advect<RefArith><<<g, BLK, 0, h->stream>>>(
        c, h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->type, h->dens, h->u[0], h->u[1], h->u[2],
        h->us[0], h->us[1], h->us[2], h->A, h->wall_start, h->wall_pos, h->wall_nrm, h->flag);
  ktime_end(h);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_advect(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  const unsigned g = grid_for(h->np, BLK);
  if (h->prm.arith == FLIPGPU_ARITH_FAST)
    k_advect<FastArith><<<g, BLK, 0, h->stream>>>(
        c, h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->type, h->dens, h->u[0], h->u[1], h->u[2],
        h->A, h->wall_start, h->wall_pos, h->wall_nrm, h->flag);
  else
    k_advect<RefArith><<<g, BLK, 0, h->stream>>>(
        c, h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->type, h->dens, h->u[0], h->u[1], h->u[2],
        h->A, h->wall_start, h->wall_pos, h->wall_nrm, h->flag);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

/* Compute stuck and deep-water lists, place the stuck particles. The sort
 * and the ordered resample follow in launch_reposition_resample. */
cudaError_t launch_reposition(FlipGpu *h, int *stuck_host, bool in_step) {
  SimConst c = make_const(h);
  cudaError_t e;
  if (h->np == 0) {
    if (stuck_host) *stuck_host = 0;
    return cudaSuccess;
  }
  /* the stuck particles and the deep-water cells, each in ascending order */
  if ((e = compact_flags(h, h->flag, h->np, h->stuck_idx, h->iflags + IF_NSTUCK)) != cudaSuccess)
    return e;
  if ((e = compact_deep_water(h, h->water_idx, h->iflags + IF_NWATER)) != cudaSuccess) return e;
  /* my_rand_shuffle: draws, lists of the steps per position, chains (over
   * the m stuck particles only) */
  {
    const size_t np1 = (size_t)h->np + 1;
    k_zero_live<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags + IF_NSTUCK, h->repo_cnt);
    k_shuffle_draws<<<REPO_GRID, BLK, 0, h->stream>>>(c, h->iflags, h->repo_draw, h->repo_cnt);
    FG_LAUNCHED(h, 2);
    if ((e = scan_exclusive_live(h, h->repo_cnt, h->repo_start, np1, h->iflags + IF_NSTUCK)) !=
        cudaSuccess)
      return e;
    k_shuffle_fill<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags, h->repo_draw, h->repo_start,
                                                     h->repo_cnt, h->repo_list);
    k_shuffle_sort<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags, h->repo_start, h->repo_list);
    k_shuffle_resolve<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags, h->repo_draw, h->repo_start,
                                                        h->repo_list, h->water_idx, h->scan_b);
    FG_LAUNCHED(h, 3);
  }
  k_repo_place<<<REPO_GRID, BLK, 0, h->stream>>>(c, h->iflags, h->stuck_idx, h->scan_b,
                                                 h->scan_a, h->px, h->py, h->pz);
  FG_LAUNCHED(h, 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  /* sorter::sort (src/flip3D.cpp:443), shared with the corrector's sort. */
  if ((e = launch_sort(h, 0, in_step ? 0 : PL_ALL)) != cudaSuccess) return e;
  /* corrector::resample of each stuck particle in order (src/flip3D.cpp:445-450) */
  int *left = h->iflags + IF_REPO_LEFT;
  if ((e = cudaMemsetAsync(left, 0, sizeof(int), h->stream)) != cudaSuccess) return e;
  k_repo_gather<<<REPO_GRID, BLK, 0, h->stream>>>(
      c, h->iflags, h->stuck_idx, h->cell_start, h->perm, h->spos, h->flag, h->scan_a, h->px,
      h->py, h->pz, h->vx, h->vy, h->vz, h->repo_res, h->repo_old, h->repo_state, left);
  k_repo_commit<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags, h->stuck_idx, h->repo_res,
                                                  h->repo_state, h->vx, h->vy, h->vz, left, 0);
  FG_LAUNCHED(h, 2);
  for (int r = 1; r <= REPO_ROUNDS; r++) {
    k_repo_round<<<REPO_GRID, BLK, 0, h->stream>>>(
        c, h->iflags, h->stuck_idx, h->cell_start, h->perm, h->spos, h->flag, h->scan_a, h->px,
        h->py, h->pz, h->vx, h->vy, h->vz, h->repo_res, h->repo_old, h->repo_state, left);
    k_repo_commit<<<REPO_GRID, BLK, 0, h->stream>>>(h->iflags, h->stuck_idx, h->repo_res,
                                                    h->repo_state, h->vx, h->vy, h->vz, left, r);
    FG_LAUNCHED(h, 2);
  }
  k_repo_ordered<<<1, 32, 0, h->stream>>>(c, h->iflags, h->stuck_idx, h->cell_start, h->perm,
                                          h->spos, h->flag, h->scan_a, h->px, h->py, h->pz,
                                          h->vx, h->vy, h->vz, h->repo_old, h->repo_state, left);
  FG_LAUNCHED(h, 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  /* refresh the sorted velocities of the resampled particles (positions,
   * grid positions and densities are those of the sort above) */
  if ((e = launch_payload_vel(h, 0)) != cudaSuccess) return e;
  if (stuck_host) {
    int v = 0;
    e = cudaMemcpyAsync(&v, h->iflags + IF_NSTUCK, sizeof(int), cudaMemcpyDeviceToHost,
                        h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    *stuck_host = v;
  }
  return e;
}

cudaError_t launch_correct(FlipGpu *h) {
  if (h->np == 0) return cudaSuccess;
  SimConst c = make_const(h);
  const unsigned g = grid_for(h->np, BLK);
  const bool fast = h->prm.arith == FLIPGPU_ARITH_FAST;
  if (cell_gathers(h)) {
    cudaError_t e = tuned_gather(h, "k_spring_inline", h->np, [&](auto B) {
      constexpr int b = decltype(B)::value;
      k_spring_inline<FastArith, b><<<grid_for(h->np, b), b, 0, h->stream>>>(
          c, h->cell_start, h->cell_mid, h->perm, h->spos, h->nx, h->ny, h->nz, h->px, h->py,
          h->pz);
    });
    if (e != cudaSuccess) return e;
    if (h->xfer_pos_out && (e = xfer_positions_out(h)) != cudaSuccess) return e;
    return tuned_gather(h, "k_resample_inline", h->np, [&](auto B) {
      constexpr int b = decltype(B)::value;
      k_resample_inline<FastArith, b><<<grid_for(h->np, b), b, 0, h->stream>>>(
          c, h->cell_start, h->cell_mid, h->perm, h->spos, h->svel, h->px, h->py, h->pz, h->vx,
          h->vy, h->vz);
    });
  }
  if (fast)
    k_spring<FastArith><<<g, BLK, 0, h->stream>>>(c, h->cell_start, h->perm, h->spos, h->nx,
                                                  h->ny, h->nz, h->px, h->py, h->pz);
  else
    k_spring<RefArith><<<g, BLK, 0, h->stream>>>(c, h->cell_start, h->perm, h->spos, h->nx,
                                                 h->ny, h->nz, h->px, h->py, h->pz);
  FG_LAUNCHED(h, 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  /* the positions are final: their download can run beside the resample */
  if (h->xfer_pos_out && (e = xfer_positions_out(h)) != cudaSuccess) return e;
  if (fast)
    k_resample<FastArith><<<g, BLK, 0, h->stream>>>(c, h->cell_start, h->perm, h->spos, h->svel,
                                                    h->px, h->py, h->pz, h->vx, h->vy, h->vz);
  else
    k_resample<RefArith><<<g, BLK, 0, h->stream>>>(c, h->cell_start, h->perm, h->spos, h->svel,
                                                   h->px, h->py, h->pz, h->vx, h->vy, h->vz);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

int particles_init_device() { return 0; }
