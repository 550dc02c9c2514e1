/*
 * k_mesh.cu — mesher::generateMesh (src/mesher.cpp:137-195) and
 * implicit::implicit_func (src/implicit.cpp:14-38).
 *
 * The reference samples a distance field on the (n+1)^3 grid nodes, runs
 * marching cubes over it (src/rchandra/CIsoSurface.cpp:331-780: std::map
 * keyed by edge id, per-cell triangle vectors merged x-major), drops faces
 * with an edge of length >= 0.1, sums area-weighted normals triangle by
 * triangle and smooths vertices and normals twice over face neighbours.
 * Here every step is a data-parallel pass with the same results:
 *
 *   field      one thread per node; neighbour cells are visited nearest
 *              first and skipped when they are provably farther than the
 *              current minimum (the value is a minimum, so the order of
 *              visits cannot change it). The lists may be older than the
 *              positions (the reference meshes after the corrector moved the
 *              particles), so the bound comes from the particles' current
 *              coordinates: per axis, the range of every slab of cells;
 *   vertices   one per cut grid edge, numbered by an exclusive scan of the
 *              per-node cut counts in node order (x fastest) — the order of
 *              the reference's edge-id map; each vertex is interpolated with
 *              the orientation of the cell that owns its edge;
 *   triangles  per-cell counts scanned in the reference's merge order
 *              (x outermost, z innermost), then emitted from the case table;
 *   normals    each vertex gathers the normals of its incident triangles
 *              from the (at most four) cells around its edge, in triangle
 *              order — the reference's sequential accumulation order, with
 *              no atomics;
 *   faces      kept-face flags scanned and compacted in triangle order;
 *   smoothing  per-vertex neighbour lists (CSR) filled by the same gather in
 *              face order, then two Jacobi passes in FP64 like the
 *              reference's double accumulators.
 *
 * The field layout is the reference's dense_grid: node (x,y,z) at
 * (z*mg + y)*mg + x with mg = n+1.
 */
#include <cfloat>
#include <cstdio>

#include "devcommon.cuh"
#include "flipgpu_impl.h"
#include "refmath.h"
#include "../../include/flip_mc_table.h"

using namespace refmath;

struct MeshBufs {
  int mg = 0;
  size_t nn = 0, ncell = 0;
  float *phi = nullptr;
  uint32_t *vcnt = nullptr, *vbase = nullptr; /* nn + 1 */
  uint32_t *tcnt = nullptr, *tbase = nullptr; /* ncell + 1 */
  uint8_t *ccase = nullptr;                    /* ncell, triangle order */
  uint32_t *slab = nullptr;                    /* 6 n: per-axis slab bounds */
  uint32_t *tmp = nullptr;
  size_t tmp_blocks = 0;
  size_t vcap = 0, tcap = 0, fcap = 0;
  float *vf = nullptr;                         /* 3 nv */
  double *V = nullptr, *N = nullptr, *CV = nullptr, *CN = nullptr;
  uint32_t *ccnt = nullptr, *cbase = nullptr;  /* nv + 1 */
  int32_t *T = nullptr;                        /* 3 nt */
  float *TN = nullptr;                         /* 3 nt */
  uint32_t *keep = nullptr, *fbase = nullptr;  /* nt + 1 */
  uint32_t *conn = nullptr;                    /* 6 nf */
  int32_t *F = nullptr;                        /* 3 nf */
  int64_t nv = 0, nt = 0, nf = 0;
  bool valid = false;
};

namespace {

constexpr int MBLK = 256;

__constant__ signed char c_tri[256][16];
__constant__ unsigned char c_tcount[256];
__constant__ unsigned char c_enode[12][4];

/* For a vertex on the edge leaving node (X,Y,Z) along `axis`: the four cells
 * that share the edge, in the reference's triangle order (x, then y, then
 * z), as offsets from the node, with the edge's number inside each cell. */
__constant__ signed char c_ring[3][4][4] = {
    {{0, -1, -1, 5}, {0, -1, 0, 1}, {0, 0, -1, 7}, {0, 0, 0, 3}},
    {{-1, 0, -1, 6}, {-1, 0, 0, 2}, {0, 0, -1, 4}, {0, 0, 0, 0}},
    {{-1, -1, 0, 10}, {-1, 0, 0, 11}, {0, -1, 0, 9}, {0, 0, 0, 8}}};

struct FieldConst {
  int n, mg;
  float fn, wall_r, wall_thr2;
  double h, phi0, wall_val;
  const uint32_t *slab; /* [axis][lo/hi][n] order-preserving keys */
};

FieldConst field_const(const FlipGpu *h) {
  FieldConst f;
  SimConst c = make_const(h);
  f.n = c.n;
  f.mg = c.n + 1;
  f.fn = c.fn;
  f.slab = nullptr;
  f.wall_r = c.density / (float)c.n;           /* density/gn, FLOAT */
  f.wall_thr2 = f.wall_r * f.wall_r * 1.000244140625f;
  f.h = 1.0 / (double)(f.mg - 1);
  f.phi0 = 8.0 * (double)c.density / c.n;
  f.wall_val = 4.5 * (double)c.density / c.n;
  return f;
}

/* float <-> unsigned key with the same order (NaN excluded by callers) */
__device__ __forceinline__ uint32_t ord_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

/* per axis a and slab s (cells with that coordinate): the smallest and
 * largest current coordinate of the particles listed there */
__global__ void k_slab_bounds(int n, const uint32_t *__restrict__ cs,
                              const float4 *__restrict__ spos, uint32_t *__restrict__ slab) {
  const size_t nc = (size_t)n * n * n;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const uint32_t s = cs[c], e = cs[c + 1];
  if (s == e) return;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  bool any[3] = {false, false, false};
  for (uint32_t q = s; q < e; q++) {
    const float4 Q = spos[q];
    const float v[3] = {Q.x, Q.y, Q.z};
    for (int a = 0; a < 3; a++)
      if (v[a] == v[a]) {
        lo[a] = fminf(lo[a], v[a]);
        hi[a] = fmaxf(hi[a], v[a]);
        any[a] = true;
      }
  }
  const int cell[3] = {(int)(c / ((size_t)n * n)), (int)((c / n) % n), (int)(c % n)};
  for (int a = 0; a < 3; a++) {
    if (!any[a]) continue;
    atomicMin(slab + (2 * a) * n + cell[a], ord_key(lo[a]));
    atomicMax(slab + (2 * a + 1) * n + cell[a], ord_key(hi[a]));
  }
}

/* distance from p to slab s of axis a (infinite when the slab is empty) */
__device__ __forceinline__ float axis_gap(const FieldConst &f, int a, int s, float p) {
  const uint32_t kl = f.slab[(2 * a) * f.n + s], kh = f.slab[(2 * a + 1) * f.n + s];
  if (kl == 0xffffffffu || kh == 0u) return FLT_MAX;
  const float lo = key_float(kl), hi = key_float(kh);
  return fmaxf(0.0f, fmaxf(lo - p, p - hi));
}

/* implicit_func (src/implicit.cpp:14-38) at p. Fluid candidates whose
 * squared distance exceeds the current minimum by a margin far above the
 * rounding of hypot (2^-12 relative) cannot lower it; only the others get
 * the reference's hypotf(hypotf()) distance. */
__device__ double implicit_value(const FieldConst &f, const uint32_t *__restrict__ cs,
                                 const float4 *__restrict__ spos, float px, float py,
                                 float pz) {
  const int n = f.n;
  const int ci = cell_clamp(px, f.fn, n), cj = cell_clamp(py, f.fn, n),
            ck = cell_clamp(pz, f.fn, n);
  const int i0 = max(ci - 2, 0), i1 = min(ci + 2, n - 1);
  const int j0 = max(cj - 2, 0), j1 = min(cj + 2, n - 1);
  const int k0 = max(ck - 2, 0), k1 = min(ck + 2, n - 1);
  float gx[5], gy[5], gz[5];
#pragma unroll
  for (int a = 0; a < 5; a++) {
    gx[a] = (i0 + a <= i1) ? axis_gap(f, 0, i0 + a, px) : FLT_MAX;
    gy[a] = (j0 + a <= j1) ? axis_gap(f, 1, j0 + a, py) : FLT_MAX;
    gz[a] = (k0 + a <= k1) ? axis_gap(f, 2, k0 + a, pz) : FLT_MAX;
    gx[a] *= gx[a];
    gy[a] *= gy[a];
    gz[a] *= gz[a];
  }
  double phi = f.phi0;
  float best2 = (float)(phi * phi) * 1.000244140625f;
  /* pass 0: cells at zero distance; pass 1: the rest, nearest bound first
   * is not needed for exactness, only the skip test */
  for (int pass = 0; pass < 2; pass++) {
    for (int a = 0; a <= i1 - i0; a++)
      for (int b = 0; b <= j1 - j0; b++) {
        const float gab = gx[a] + gy[b];
        const size_t row = ((size_t)(i0 + a) * n + (j0 + b)) * n;
        for (int c = 0; c <= k1 - k0; c++) {
          const float lb2 = gab + gz[c];
          if ((lb2 == 0.0f) != (pass == 0)) continue;
          if (lb2 * 0.99998f >= fmaxf(best2, f.wall_thr2)) continue;
          const uint32_t s = __ldg(cs + row + k0 + c), e = __ldg(cs + row + k0 + c + 1);
          for (uint32_t q = s; q < e; q++) {
            const float4 Q = __ldg(spos + q);
            const float dx = Q.x - px, dy = Q.y - py, dz = Q.z - pz;
            const float d2 = dx * dx + dy * dy + dz * dz;
            if (unpack_type(Q.w) == CELL_WALL) {
              if (d2 <= f.wall_thr2 && length_ref(dx, dy, dz) < f.wall_r) return f.wall_val;
            } else if (d2 < best2) {
              const float d = length_ref(dx, dy, dz);
              if ((double)d < phi) {
                phi = d;
                best2 = (float)(phi * phi) * 1.000244140625f;
              }
            }
          }
        }
      }
  }
  return phi - (double)f.wall_r;
}

/* density field (src/mesher.cpp:142-153): node (x,y,z) at x*h, boundary
 * nodes raised to at least 0.01, stored negated */
__global__ void k_mesh_field(FieldConst f, const uint32_t *__restrict__ cs,
                             const float4 *__restrict__ spos, float *__restrict__ phi) {
  const size_t nn = (size_t)f.mg * f.mg * f.mg;
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int mg = f.mg;
  const int x = (int)(v % mg), y = (int)((v / mg) % mg), z = (int)(v / ((size_t)mg * mg));
  const float px = (float)(x * f.h), py = (float)(y * f.h), pz = (float)(z * f.h);
  double value = implicit_value(f, cs, spos, px, py, pz);
  if (x == 0 || x == mg - 1 || y == 0 || y == mg - 1 || z == 0 || z == mg - 1)
    value = fmax(value, 0.01);
  phi[v] = (float)(-value);
}

__global__ void k_implicit_points(FieldConst f, int m, const float *__restrict__ pts,
                                  const uint32_t *__restrict__ cs,
                                  const float4 *__restrict__ spos, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  out[i] = implicit_value(f, cs, spos, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
}

__device__ __forceinline__ bool inside(const float *__restrict__ phi, size_t v) {
  return phi[v] < 0.0f;
}

/* is the edge leaving node (x,y,z) along axis a cut? */
__device__ __forceinline__ bool edge_cut(const float *__restrict__ phi, int mg, int x, int y,
                                         int z, int a) {
  const int C = mg - 1;
  if ((a == 0 && x >= C) || (a == 1 && y >= C) || (a == 2 && z >= C)) return false;
  const size_t v = ((size_t)z * mg + y) * mg + x;
  const size_t d = a == 0 ? 1 : (a == 1 ? (size_t)mg : (size_t)mg * mg);
  return inside(phi, v) != inside(phi, v + d);
}

__global__ void k_mesh_vcount(int mg, const float *__restrict__ phi, uint32_t *__restrict__ vcnt) {
  const size_t nn = (size_t)mg * mg * mg;
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int x = (int)(v % mg), y = (int)((v / mg) % mg), z = (int)(v / ((size_t)mg * mg));
  vcnt[v] = (uint32_t)edge_cut(phi, mg, x, y, z, 0) + (uint32_t)edge_cut(phi, mg, x, y, z, 1) +
            (uint32_t)edge_cut(phi, mg, x, y, z, 2);
}

/* vertex id of the edge leaving node (x,y,z) along a (which must be cut) */
__device__ __forceinline__ uint32_t vertex_of(const float *__restrict__ phi,
                                              const uint32_t *__restrict__ vbase, int mg,
                                              int x, int y, int z, int a) {
  uint32_t r = vbase[((size_t)z * mg + y) * mg + x];
  for (int b = 0; b < a; b++) r += edge_cut(phi, mg, x, y, z, b);
  return r;
}

/* CalculateIntersection + Interpolate (src/rchandra/CIsoSurface.cpp:
 * 580-700) with the owning cell's orientation: x edges below the top y row
 * and y edges on the last x column run from the far node to the base node. */
__global__ void k_mesh_vertices(int mg, float cell_len, const float *__restrict__ phi,
                                const uint32_t *__restrict__ vbase, float *__restrict__ vf,
                                double *__restrict__ V) {
  const size_t nn = (size_t)mg * mg * mg;
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int C = mg - 1;
  const int x = (int)(v % mg), y = (int)((v / mg) % mg), z = (int)(v / ((size_t)mg * mg));
  uint32_t id = vbase[v];
  for (int a = 0; a < 3; a++) {
    if (!edge_cut(phi, mg, x, y, z, a)) continue;
    int b[3] = {x, y, z}, f[3] = {x + (a == 0), y + (a == 1), z + (a == 2)};
    const bool rev = (a == 0 && y < C) || (a == 1 && x == C);
    const int *v1 = rev ? f : b, *v2 = rev ? b : f;
    const float val1 = phi[((size_t)v1[2] * mg + v1[1]) * mg + v1[0]];
    const float val2 = phi[((size_t)v2[2] * mg + v2[1]) * mg + v2[0]];
    const float mu = (0.0f - val1) / (val2 - val1);
    for (int d = 0; d < 3; d++) {
      const float p1 = (float)(unsigned)v1[d] * cell_len, p2 = (float)(unsigned)v2[d] * cell_len;
      const float p = p1 + mu * (p2 - p1);
      vf[3 * (size_t)id + d] = p;
      V[3 * (size_t)id + d] = (double)p;
    }
    id++;
  }
}

/* cell t in triangle order: t = (x*C + y)*C + z */
__device__ __forceinline__ unsigned cell_case(const float *__restrict__ phi, int mg, int x, int y,
                                              int z) {
  unsigned idx = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int dx = (c == 2 || c == 3 || c == 6 || c == 7);
    const int dy = (c == 1 || c == 2 || c == 5 || c == 6);
    const int dz = c >= 4;
    if (inside(phi, ((size_t)(z + dz) * mg + (y + dy)) * mg + (x + dx))) idx |= 1u << c;
  }
  return idx;
}

__global__ void k_mesh_ccount(int mg, const float *__restrict__ phi, uint8_t *__restrict__ ccase,
                              uint32_t *__restrict__ tcnt) {
  const int C = mg - 1;
  const size_t nc = (size_t)C * C * C;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int z = (int)(t % C), y = (int)((t / C) % C), x = (int)(t / ((size_t)C * C));
  const unsigned k = cell_case(phi, mg, x, y, z);
  ccase[t] = (uint8_t)k;
  tcnt[t] = c_tcount[k];
}

__device__ __forceinline__ float len2f(const float *a, const float *b) {
  const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return dx * dx + dy * dy + dz * dz;
}

/* triangles of each cell (table order), their normals as CalculateNormals
 * forms them (src/rchandra/CIsoSurface.cpp:756-764) and the long-edge filter
 * of src/mesher.cpp:172-182 */
__global__ void k_mesh_tris(int mg, const float *__restrict__ phi,
                            const uint32_t *__restrict__ vbase, const uint8_t *__restrict__ ccase,
                            const uint32_t *__restrict__ tbase, const float *__restrict__ vf,
                            int32_t *__restrict__ T, float *__restrict__ TN,
                            uint32_t *__restrict__ keep) {
  const int C = mg - 1;
  const size_t nc = (size_t)C * C * C;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const unsigned k = ccase[t];
  const int cnt = c_tcount[k];
  if (cnt == 0) return;
  const int z = (int)(t % C), y = (int)((t / C) % C), x = (int)(t / ((size_t)C * C));
  const size_t base = tbase[t];
  for (int j = 0; j < cnt; j++) {
    uint32_t id[3];
    for (int q = 0; q < 3; q++) {
      const int e = c_tri[k][3 * j + q];
      id[q] = vertex_of(phi, vbase, mg, x + c_enode[e][0], y + c_enode[e][1], z + c_enode[e][2],
                        c_enode[e][3]);
      T[3 * (base + j) + q] = (int32_t)id[q];
    }
    const float *p0 = vf + 3 * (size_t)id[0], *p1 = vf + 3 * (size_t)id[1],
                *p2 = vf + 3 * (size_t)id[2];
    const float a0 = p1[0] - p0[0], a1 = p1[1] - p0[1], a2 = p1[2] - p0[2];
    const float b0 = p2[0] - p0[0], b1 = p2[1] - p0[1], b2 = p2[2] - p0[2];
    TN[3 * (base + j) + 0] = a2 * b1 - a1 * b2;
    TN[3 * (base + j) + 1] = a0 * b2 - a2 * b0;
    TN[3 * (base + j) + 2] = a1 * b0 - a0 * b1;
    const double maxlen2 = 0.1 * 0.1;
    keep[base + j] = ((double)len2f(p0, p1) < maxlen2 && (double)len2f(p1, p2) < maxlen2 &&
                      (double)len2f(p0, p2) < maxlen2)
                         ? 1u
                         : 0u;
  }
}

/* Visit the triangles incident to the vertex on edge (x,y,z,a) in triangle
 * order: f(global triangle index, position of the vertex in it). */
template <class Fn>
__device__ __forceinline__ void for_incident(int mg, int x, int y, int z, int a,
                                             const uint8_t *__restrict__ ccase,
                                             const uint32_t *__restrict__ tbase, Fn f) {
  const int C = mg - 1;
  for (int r = 0; r < 4; r++) {
    const int cx = x + c_ring[a][r][0], cy = y + c_ring[a][r][1], cz = z + c_ring[a][r][2];
    if (cx < 0 || cy < 0 || cz < 0 || cx >= C || cy >= C || cz >= C) continue;
    const int le = c_ring[a][r][3];
    const size_t t = ((size_t)cx * C + cy) * C + cz;
    const unsigned k = ccase[t];
    const int cnt = c_tcount[k];
    for (int j = 0; j < cnt; j++)
      for (int q = 0; q < 3; q++)
        if (c_tri[k][3 * j + q] == le) f(tbase[t] + j, q);
  }
}

/* per-vertex normal: sum of incident triangle normals in triangle order,
 * normalised (src/rchandra/CIsoSurface.cpp:766-777); also the number of
 * face-neighbour entries the vertex gets (src/mesher.cpp:89-101) */
__global__ void k_mesh_vnormals(int mg, const float *__restrict__ phi,
                                const uint32_t *__restrict__ vbase,
                                const uint8_t *__restrict__ ccase,
                                const uint32_t *__restrict__ tbase, const float *__restrict__ TN,
                                const uint32_t *__restrict__ keep, double *__restrict__ N,
                                uint32_t *__restrict__ ccnt) {
  const size_t nn = (size_t)mg * mg * mg;
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int x = (int)(v % mg), y = (int)((v / mg) % mg), z = (int)(v / ((size_t)mg * mg));
  uint32_t id = vbase[v];
  for (int a = 0; a < 3; a++) {
    if (!edge_cut(phi, mg, x, y, z, a)) continue;
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    uint32_t nk = 0;
    for_incident(mg, x, y, z, a, ccase, tbase, [&](uint32_t tri, int) {
      s0 += TN[3 * (size_t)tri];
      s1 += TN[3 * (size_t)tri + 1];
      s2 += TN[3 * (size_t)tri + 2];
      nk += keep[tri];
    });
    const float len = sqrtf(s0 * s0 + s1 * s1 + s2 * s2);
    N[3 * (size_t)id] = (double)(s0 / len);
    N[3 * (size_t)id + 1] = (double)(s1 / len);
    N[3 * (size_t)id + 2] = (double)(s2 / len);
    ccnt[id] = 2 * nk;
    id++;
  }
}

/* neighbour lists in face order: for a kept face (a,b,c) a gets b,c; b gets
 * a,c; c gets a,b (src/mesher.cpp:92-99) */
__global__ void k_mesh_conn(int mg, const float *__restrict__ phi,
                            const uint32_t *__restrict__ vbase, const uint8_t *__restrict__ ccase,
                            const uint32_t *__restrict__ tbase, const int32_t *__restrict__ T,
                            const uint32_t *__restrict__ keep, const uint32_t *__restrict__ cbase,
                            uint32_t *__restrict__ conn) {
  const size_t nn = (size_t)mg * mg * mg;
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  const int x = (int)(v % mg), y = (int)((v / mg) % mg), z = (int)(v / ((size_t)mg * mg));
  uint32_t id = vbase[v];
  for (int a = 0; a < 3; a++) {
    if (!edge_cut(phi, mg, x, y, z, a)) continue;
    uint32_t o = cbase[id];
    for_incident(mg, x, y, z, a, ccase, tbase, [&](uint32_t tri, int q) {
      if (!keep[tri]) return;
      const int32_t *tv = T + 3 * (size_t)tri;
      conn[o++] = (uint32_t)tv[q == 0 ? 1 : 0];
      conn[o++] = (uint32_t)tv[q == 2 ? 1 : 2];
    });
    id++;
  }
}

__global__ void k_mesh_faces(size_t nt, const int32_t *__restrict__ T,
                             const uint32_t *__restrict__ keep, const uint32_t *__restrict__ fbase,
                             int32_t *__restrict__ F) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt || !keep[t]) return;
  const size_t f = fbase[t];
  F[3 * f] = T[3 * t];
  F[3 * f + 1] = T[3 * t + 1];
  F[3 * f + 2] = T[3 * t + 2];
}

__device__ __forceinline__ bool is_normal(double x) {
  const double a = fabs(x);
  return a >= DBL_MIN && a <= DBL_MAX;
}

/* one pass of smoothMesh (src/mesher.cpp:21-71): unit weights, a vertex or
 * neighbour joins only when all six of its coordinates are normal numbers;
 * an output without weight (or with a zero normal length) keeps the value
 * the copy buffer already holds */
__global__ void k_mesh_smooth(size_t nv, const double *__restrict__ V,
                              const double *__restrict__ N, const uint32_t *__restrict__ cbase,
                              const uint32_t *__restrict__ conn, double *__restrict__ CV,
                              double *__restrict__ CN) {
  const size_t vi = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vi >= nv) return;
  float wsum = 0.0f;
  double v0 = 0.0, v1 = 0.0, v2 = 0.0, n0 = 0.0, n1 = 0.0, n2 = 0.0;
  auto add = [&](size_t u) {
    const double a0 = V[3 * u], a1 = V[3 * u + 1], a2 = V[3 * u + 2];
    const double b0 = N[3 * u], b1 = N[3 * u + 1], b2 = N[3 * u + 2];
    if (!(is_normal(a0) && is_normal(a1) && is_normal(a2) && is_normal(b0) && is_normal(b1) &&
          is_normal(b2)))
      return;
    v0 += a0;
    v1 += a1;
    v2 += a2;
    n0 += b0;
    n1 += b1;
    n2 += b2;
    wsum += 1.0f;
  };
  add(vi);
  for (uint32_t k = cbase[vi]; k < cbase[vi + 1]; k++) add(conn[k]);
  const float len = hypot_ref((float)n0, hypot_ref((float)n1, (float)n2));
  if (wsum != 0.0f) {
    CV[3 * vi] = v0 / (double)wsum;
    CV[3 * vi + 1] = v1 / (double)wsum;
    CV[3 * vi + 2] = v2 / (double)wsum;
  }
  if (len != 0.0f) {
    CN[3 * vi] = n0 / (double)len;
    CN[3 * vi + 1] = n1 / (double)len;
    CN[3 * vi + 2] = n2 / (double)len;
  }
}

int mesh_init_device() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  signed char tri[256][16];
  unsigned char cnt[256];
  flip_mc_decode(tri, cnt);
  if (cudaMemcpyToSymbol(c_tri, tri, sizeof tri) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_tcount, cnt, sizeof cnt) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_enode, FLIP_MC_EDGE_NODE, sizeof FLIP_MC_EDGE_NODE) != cudaSuccess)
    return -1;
  done[dev] = true;
  return 0;
}

void free_bufs(MeshBufs *m) {
  void *ptrs[] = {m->phi, m->vcnt, m->vbase, m->tcnt, m->tbase, m->ccase, m->slab, m->tmp, m->vf,
                  m->V,   m->N,    m->CV,    m->CN,   m->ccnt,  m->cbase, m->T,   m->TN,
                  m->keep, m->fbase, m->conn, m->F};
  for (void *p : ptrs)
    if (p) cudaFree(p);
}

#define MCK(x)                          \
  do {                                  \
    cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) return e_;   \
  } while (0)

template <class T> cudaError_t dalloc_n(T *&p, size_t n) {
  if (p) cudaFree(p);
  p = nullptr;
  return cudaMalloc(&p, (n ? n : 1) * sizeof(T));
}

cudaError_t read_u32(FlipGpu *h, const uint32_t *src, uint32_t *dst) {
  MCK(cudaMemcpyAsync(dst, src, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  return cudaStreamSynchronize(h->stream);
}

/* refresh the sorted copy from current positions and the slab bounds the
 * field's pruning reads */
cudaError_t field_prepare(FlipGpu *h, FieldConst &f) {
  if (!h->mesh) h->mesh = new MeshBufs;
  MeshBufs *m = h->mesh;
  const int n = h->n;
  if (!m->slab) MCK(dalloc_n(m->slab, 6 * (size_t)n));
  MCK(launch_payload(h, 0));
  for (int a = 0; a < 3; a++) {
    MCK(cudaMemsetAsync(m->slab + (2 * a) * (size_t)n, 0xff, (size_t)n * sizeof(uint32_t),
                        h->stream));
    MCK(cudaMemsetAsync(m->slab + (2 * a + 1) * (size_t)n, 0, (size_t)n * sizeof(uint32_t),
                        h->stream));
  }
  const size_t nc = (size_t)n * n * n;
  k_slab_bounds<<<grid_for(nc, MBLK), MBLK, 0, h->stream>>>(n, h->cell_start, h->spos, m->slab);
  FG_LAUNCHED(h, 1);
  MCK(cudaGetLastError());
  f = field_const(h);
  f.slab = m->slab;
  return cudaSuccess;
}

cudaError_t mesh_run_impl(FlipGpu *h, int64_t *nverts, int64_t *nfaces) {
  FieldConst f;
  MCK(field_prepare(h, f));
  MeshBufs *m = h->mesh;
  m->valid = false;
  const int n = h->n, mg = n + 1;
  const size_t nn = (size_t)mg * mg * mg, ncell = (size_t)n * n * n;
  if (m->mg != mg) {
    MCK(dalloc_n(m->phi, nn));
    MCK(dalloc_n(m->vcnt, nn + 1));
    MCK(dalloc_n(m->vbase, nn + 1));
    MCK(dalloc_n(m->tcnt, ncell + 1));
    MCK(dalloc_n(m->tbase, ncell + 1));
    MCK(dalloc_n(m->ccase, ncell));
    m->tmp_blocks = scan_tmp_blocks(nn + 1);
    MCK(dalloc_n(m->tmp, m->tmp_blocks));
    m->mg = mg;
    m->nn = nn;
    m->ncell = ncell;
  }
  k_mesh_field<<<grid_for(nn, MBLK), MBLK, 0, h->stream>>>(f, h->cell_start, h->spos, m->phi);
  k_mesh_vcount<<<grid_for(nn, MBLK), MBLK, 0, h->stream>>>(mg, m->phi, m->vcnt);
  k_mesh_ccount<<<grid_for(ncell, MBLK), MBLK, 0, h->stream>>>(mg, m->phi, m->ccase, m->tcnt);
  FG_LAUNCHED(h, 3);
  MCK(cudaGetLastError());
  MCK(cudaMemsetAsync(m->vcnt + nn, 0, sizeof(uint32_t), h->stream));
  MCK(cudaMemsetAsync(m->tcnt + ncell, 0, sizeof(uint32_t), h->stream));
  MCK(scan_exclusive_tmp(h, m->vcnt, m->vbase, nn + 1, m->tmp, m->tmp_blocks));
  MCK(scan_exclusive_tmp(h, m->tcnt, m->tbase, ncell + 1, m->tmp, m->tmp_blocks));
  uint32_t nv = 0, nt = 0;
  MCK(read_u32(h, m->vbase + nn, &nv));
  MCK(read_u32(h, m->tbase + ncell, &nt));
  if (nv >= m->vcap) { /* also the first time: ccnt[nv] is written even when nv = 0 */
    size_t cap = nv + nv / 4 + 1024;
    MCK(dalloc_n(m->vf, 3 * cap));
    MCK(dalloc_n(m->V, 3 * cap));
    MCK(dalloc_n(m->N, 3 * cap));
    MCK(dalloc_n(m->CV, 3 * cap));
    MCK(dalloc_n(m->CN, 3 * cap));
    MCK(dalloc_n(m->ccnt, cap + 1));
    MCK(dalloc_n(m->cbase, cap + 1));
    m->vcap = cap;
  }
  if (nt >= m->tcap) {
    size_t cap = nt + nt / 4 + 1024;
    MCK(dalloc_n(m->T, 3 * cap));
    MCK(dalloc_n(m->TN, 3 * cap));
    MCK(dalloc_n(m->keep, cap + 1));
    MCK(dalloc_n(m->fbase, cap + 1));
    m->tcap = cap;
  }
  const size_t need_blocks = scan_tmp_blocks((nv > nt ? nv : nt) + 1);
  if (need_blocks > m->tmp_blocks) {
    MCK(dalloc_n(m->tmp, need_blocks));
    m->tmp_blocks = need_blocks;
  }
  const float cell_len = (float)(1.0 / (double)(mg - 1));
  k_mesh_vertices<<<grid_for(nn, MBLK), MBLK, 0, h->stream>>>(mg, cell_len, m->phi, m->vbase,
                                                              m->vf, m->V);
  k_mesh_tris<<<grid_for(ncell, MBLK), MBLK, 0, h->stream>>>(mg, m->phi, m->vbase, m->ccase,
                                                             m->tbase, m->vf, m->T, m->TN,
                                                             m->keep);
  k_mesh_vnormals<<<grid_for(nn, MBLK), MBLK, 0, h->stream>>>(mg, m->phi, m->vbase, m->ccase,
                                                              m->tbase, m->TN, m->keep, m->N,
                                                              m->ccnt);
  FG_LAUNCHED(h, 3);
  MCK(cudaGetLastError());
  MCK(cudaMemsetAsync(m->ccnt + nv, 0, sizeof(uint32_t), h->stream));
  MCK(cudaMemsetAsync(m->keep + nt, 0, sizeof(uint32_t), h->stream));
  MCK(scan_exclusive_tmp(h, m->ccnt, m->cbase, (size_t)nv + 1, m->tmp, m->tmp_blocks));
  MCK(scan_exclusive_tmp(h, m->keep, m->fbase, (size_t)nt + 1, m->tmp, m->tmp_blocks));
  uint32_t nf = 0;
  MCK(read_u32(h, m->fbase + nt, &nf));
  if (nf >= m->fcap) {
    size_t cap = nf + nf / 4 + 1024;
    MCK(dalloc_n(m->conn, 6 * cap));
    MCK(dalloc_n(m->F, 3 * cap));
    m->fcap = cap;
  }
  k_mesh_conn<<<grid_for(nn, MBLK), MBLK, 0, h->stream>>>(mg, m->phi, m->vbase, m->ccase,
                                                          m->tbase, m->T, m->keep, m->cbase,
                                                          m->conn);
  if (nt > 0)
    k_mesh_faces<<<grid_for(nt, MBLK), MBLK, 0, h->stream>>>(nt, m->T, m->keep, m->fbase, m->F);
  FG_LAUNCHED(h, nt > 0 ? 2 : 1);
  MCK(cudaGetLastError());
  /* smoothMesh(sort, vertices, normals, connections, 2, 1, 1) */
  const size_t vb = 3 * (size_t)nv * sizeof(double);
  if (vb) {
    MCK(cudaMemsetAsync(m->CV, 0, vb, h->stream));
    MCK(cudaMemsetAsync(m->CN, 0, vb, h->stream));
  }
  for (int it = 0; it < 2 && nv > 0; it++) {
    k_mesh_smooth<<<grid_for(nv, MBLK), MBLK, 0, h->stream>>>(nv, m->V, m->N, m->cbase, m->conn,
                                                              m->CV, m->CN);
    FG_LAUNCHED(h, 1);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(m->V, m->CV, vb, cudaMemcpyDeviceToDevice, h->stream));
    MCK(cudaMemcpyAsync(m->N, m->CN, vb, cudaMemcpyDeviceToDevice, h->stream));
  }
  MCK(cudaStreamSynchronize(h->stream));
  m->nv = nv;
  m->nt = nt;
  m->nf = nf;
  m->valid = true;
  if (nverts) *nverts = nv;
  if (nfaces) *nfaces = nf;
  return cudaSuccess;
}

} // namespace

int mesh_run(FlipGpu *h, int64_t *nverts, int64_t *nfaces) {
  if (mesh_init_device() != 0) return FLIPGPU_ECUDA;
  cudaError_t e = mesh_run_impl(h, nverts, nfaces);
  if (e == cudaErrorMemoryAllocation) return FLIPGPU_ENOMEM;
  return e == cudaSuccess ? FLIPGPU_OK : FLIPGPU_ECUDA;
}

int mesh_get(FlipGpu *h, double *vertices, double *normals, int32_t *faces, float *phi) {
  MeshBufs *m = h->mesh;
  if (!m || !m->valid) return FLIPGPU_EINVAL;
  cudaError_t e = cudaSuccess;
  const size_t vb = 3 * (size_t)m->nv * sizeof(double);
  if (vertices && vb && e == cudaSuccess)
    e = cudaMemcpyAsync(vertices, m->V, vb, cudaMemcpyDeviceToHost, h->stream);
  if (normals && vb && e == cudaSuccess)
    e = cudaMemcpyAsync(normals, m->N, vb, cudaMemcpyDeviceToHost, h->stream);
  if (faces && m->nf && e == cudaSuccess)
    e = cudaMemcpyAsync(faces, m->F, 3 * (size_t)m->nf * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        h->stream);
  if (phi && e == cudaSuccess)
    e = cudaMemcpyAsync(phi, m->phi, m->nn * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  return e == cudaSuccess ? FLIPGPU_OK : FLIPGPU_ECUDA;
}

/* counts of the last mesh and, if the pointers are set, its copies into
 * host memory enqueued on the handle's stream (no synchronisation) */
int mesh_download_async(FlipGpu *h, double *vertices, double *normals, int32_t *faces,
                        int64_t *nv, int64_t *nf) {
  MeshBufs *m = h->mesh;
  if (!m || !m->valid) return FLIPGPU_EINVAL;
  *nv = m->nv;
  *nf = m->nf;
  cudaError_t e = cudaSuccess;
  const size_t vb = 3 * (size_t)m->nv * sizeof(double);
  if (vertices && vb) e = cudaMemcpyAsync(vertices, m->V, vb, cudaMemcpyDeviceToHost, h->stream);
  if (normals && vb && e == cudaSuccess)
    e = cudaMemcpyAsync(normals, m->N, vb, cudaMemcpyDeviceToHost, h->stream);
  if (faces && m->nf && e == cudaSuccess)
    e = cudaMemcpyAsync(faces, m->F, 3 * (size_t)m->nf * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        h->stream);
  return e == cudaSuccess ? FLIPGPU_OK : FLIPGPU_ECUDA;
}

cudaError_t launch_implicit_points(FlipGpu *h, int count, const float *pts, double *out) {
  if (count == 0) return cudaSuccess;
  FieldConst f;
  cudaError_t e = field_prepare(h, f);
  if (e != cudaSuccess) return e;
  k_implicit_points<<<grid_for(count, MBLK), MBLK, 0, h->stream>>>(f, count, pts, h->cell_start,
                                                                   h->spos, out);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

void mesh_free(FlipGpu *h) {
  if (!h->mesh) return;
  free_bufs(h->mesh);
  delete h->mesh;
  h->mesh = nullptr;
}
