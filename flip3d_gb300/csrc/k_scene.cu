/*
 * k_scene.cu — scene setup on the device: flip3D::init's particle seeding
 * (src/flip3D.cpp:649-777 with pushParticle at :580-647), the cube walls
 * of placeWalls (:300-362) with compute_wall_normal's face normals
 * (:75-130), and the static wall lists the advection walks.
 *
 * The arithmetic is the host generator's (flip3d_gb300/scenes.py:build),
 * itself the reference's with the counter-based generator of
 * include/flip_rng.h in place of rand(): lattice coordinates and jitter in
 * double, object tests as the reference's FLOAT/double mix, positions
 * rounded to float once. The particle order is the host's: liquid in
 * lattice order (i, then j, then k), then one wall particle per wall cell
 * in cell order.
 *
 * Three passes over the liquid lattice rows (one warp per (i, j) row, 32
 * consecutive k per ballot): count the kept points of each row, scan the
 * counts, emit each point at its row offset plus its rank in the row. The
 * walls: flag the wall cells, scan, emit particle, position and normal at
 * the cell's rank; that scan is also the wall lists' cell start array.
 */
#include <cmath>
#include <cstdio>
#include <cstring>

#include "devcommon.cuh"

using namespace refmath;

namespace {

constexpr int SBLK = 256;
constexpr int MAX_OBJ = 16;

struct SceneArgs {
  int n, m, nobj;
  double wall, w, jitter;
  uint64_t seed;
  FlipSceneObject obj[MAX_OBJ];
};

/* scenes.py:_inside for one lattice point (x, y, z double) */
__device__ bool inside(const FlipSceneObject &o, double x, double y, double z) {
  if (o.shape == FLIPGPU_SHAPE_BOX)
    return x > (double)o.lo[0] && x < (double)o.hi[0] && y > (double)o.lo[1] &&
           y < (double)o.hi[1] && z > (double)o.lo[2] && z < (double)o.hi[2];
  const float px = (float)x, py = (float)y, pz = (float)z;
  const float ln = hypot_ref(hypot_ref(px - o.c[0], py - o.c[1]), pz - o.c[2]);
  return ln < o.r;
}

/* Lattice point (i, j, k): whether it is seeded (interior, inside an
 * object, not jittered into a wall cell), its float position and owner. */
__device__ bool lattice_point(const SceneArgs &a, int i, int j, int k, float pos[3], int &owner) {
  const double c[3] = {(double)i * a.w + a.w / 2.0, (double)j * a.w + a.w / 2.0,
                       (double)k * a.w + a.w / 2.0};
  for (int d = 0; d < 3; d++)
    if (!(c[d] > a.wall && c[d] < 1.0 - a.wall)) return false;
  owner = -1;
  for (int q = 0; q < a.nobj; q++)
    if (inside(a.obj[q], c[0], c[1], c[2])) {
      owner = q;
      break;
    }
  if (owner < 0) return false;
  const uint64_t lattice = ((uint64_t)i * (uint64_t)a.m + (uint64_t)j) * (uint64_t)a.m + (uint64_t)k;
  bool keep = true;
  for (int d = 0; d < 3; d++) {
    const uint32_t r = flip_rand31(a.seed, flip_stream(FLIP_RNG_SEED, 0, (uint64_t)d), lattice, 0);
    const double u01 = (double)r / 2147483648.0;
    pos[d] = (float)(c[d] + (u01 - 0.5) * 2.0 * a.jitter * a.wall);
    /* cell = clip(float(n) * pos, 0, n-1) truncated; wall cells are the outer layer */
    const double g = fmin(fmax((double)((float)a.n * pos[d]), 0.0), (double)(a.n - 1));
    const int cell = (int)g;
    if (cell == 0 || cell == a.n - 1) keep = false;
  }
  return keep;
}

/* one warp per lattice row (i, j): number of seeded points */
__global__ void k_scene_count(SceneArgs a, uint32_t *__restrict__ count) {
  const int warp = (blockIdx.x * SBLK + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= a.m * a.m) return;
  const int i = warp / a.m, j = warp % a.m;
  uint32_t cnt = 0;
  for (int k0 = 0; k0 < a.m; k0 += 32) {
    const int k = k0 + lane;
    float p[3];
    int owner;
    const bool ok = k < a.m && lattice_point(a, i, j, k, p, owner);
    cnt += __popc(__ballot_sync(0xffffffffu, ok));
  }
  if (lane == 0) count[warp] = cnt;
}

/* the same rows again, each point written at its row offset + rank */
__global__ void k_scene_emit(SceneArgs a, const uint32_t *__restrict__ row_off,
                             float *__restrict__ px, float *__restrict__ py,
                             float *__restrict__ pz, float *__restrict__ vx,
                             float *__restrict__ vy, float *__restrict__ vz,
                             uint8_t *__restrict__ type, float *__restrict__ nx,
                             float *__restrict__ ny, float *__restrict__ nz) {
  const int warp = (blockIdx.x * SBLK + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= a.m * a.m) return;
  const int i = warp / a.m, j = warp % a.m;
  uint32_t at = row_off[warp];
  for (int k0 = 0; k0 < a.m; k0 += 32) {
    const int k = k0 + lane;
    float p[3];
    int owner = 0;
    const bool ok = k < a.m && lattice_point(a, i, j, k, p, owner);
    const uint32_t bal = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const uint32_t s = at + __popc(bal & ((1u << lane) - 1u));
      px[s] = p[0];
      py[s] = p[1];
      pz[s] = p[2];
      vx[s] = a.obj[owner].vel[0];
      vy[s] = a.obj[owner].vel[1];
      vz[s] = a.obj[owner].vel[2];
      type[s] = CELL_FLUID;
      nx[s] = ny[s] = nz[s] = 0.0f;
    }
    at += __popc(bal);
  }
}

__device__ __forceinline__ bool on_wall(int n, size_t c, int &i, int &j, int &k) {
  k = (int)(c % n);
  j = (int)((c / n) % n);
  i = (int)(c / ((size_t)n * n));
  return i == 0 || i == n - 1 || j == 0 || j == n - 1 || k == 0 || k == n - 1;
}

__global__ void k_wall_flags(int n, uint32_t *__restrict__ flag) {
  const size_t c = (size_t)blockIdx.x * SBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c > nc) return;
  int i, j, k;
  flag[c] = c < nc && on_wall(n, c, i, j, k) ? 1u : 0u;
}

/* wall particle of wall cell c at fluid_count + rank, with compute_wall_normal's
 * face normal for the cube walls (scenes.py:build), and the wall lists */
__global__ void k_wall_emit(int n, double wall, uint32_t nfluid, const uint32_t *__restrict__ rank,
                            float *__restrict__ px, float *__restrict__ py,
                            float *__restrict__ pz, float *__restrict__ vx,
                            float *__restrict__ vy, float *__restrict__ vz,
                            uint8_t *__restrict__ type, float *__restrict__ nx,
                            float *__restrict__ ny, float *__restrict__ nz,
                            float4 *__restrict__ wall_pos, float4 *__restrict__ wall_nrm) {
  const size_t c = (size_t)blockIdx.x * SBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  int ijk[3];
  if (!on_wall(n, c, ijk[0], ijk[1], ijk[2])) return;
  const uint32_t r = rank[c];
  const size_t s = nfluid + r;
  float p[3], wn[3];
  const double lo = 1.1 * wall, hi = 1.0 - 1.1 * wall;
  for (int d = 0; d < 3; d++) {
    p[d] = (float)((double)ijk[d] * wall + wall / 2.0);
    wn[d] = 0.0f;
    if ((double)p[d] <= lo) wn[d] = 1.0f;
    if ((double)p[d] >= hi) wn[d] = -1.0f;
  }
  const float dn = hypot_ref(hypot_ref(wn[0], wn[1]), wn[2]);
  if (dn != 0.0f)
    for (int d = 0; d < 3; d++) wn[d] = wn[d] / dn;
  px[s] = p[0];
  py[s] = p[1];
  pz[s] = p[2];
  vx[s] = vy[s] = vz[s] = 0.0f;
  type[s] = CELL_WALL;
  nx[s] = wn[0];
  ny[s] = wn[1];
  nz[s] = wn[2];
  wall_pos[r] = make_float4(p[0], p[1], p[2], 0.0f);
  wall_nrm[r] = make_float4(wn[0], wn[1], wn[2], 0.0f);
}

#define SCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      snprintf(h->err, sizeof h->err, "seed_scene: %s: %s", #call, cudaGetErrorString(e_)); \
      return FLIPGPU_ECUDA;                                                              \
    }                                                                                    \
  } while (0)

} // namespace

extern "C" int flipgpu_seed_scene(FlipGpu *h, const FlipSceneObject *objs, int nobj,
                                  uint64_t seed, double density, double jitter) {
  if (!h || nobj < 0 || nobj > MAX_OBJ || (nobj && !objs) || !(density > 0.0)) {
    if (h) snprintf(h->err, sizeof h->err, "seed_scene: bad arguments (at most %d objects)", MAX_OBJ);
    return FLIPGPU_EINVAL;
  }
  SceneArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = h->n;
  a.wall = 1.0 / h->n;
  a.w = density * a.wall;
  a.m = (int)std::lround(h->n / density);
  a.jitter = jitter;
  a.seed = seed;
  a.nobj = nobj;
  for (int q = 0; q < nobj; q++) a.obj[q] = objs[q];
  const size_t rows = (size_t)a.m * a.m, nc = h->nc;
  if (rows + 1 > nc + 1) {
    snprintf(h->err, sizeof h->err, "seed_scene: lattice rows exceed the scan scratch");
    return FLIPGPU_ETOOBIG;
  }
  cudaStream_t S = h->stream;
  /* liquid: count, scan, emit */
  const unsigned rgrid = (unsigned)((rows * 32 + SBLK - 1) / SBLK);
  k_scene_count<<<rgrid, SBLK, 0, S>>>(a, h->scan_a);
  SCK(cudaMemsetAsync(h->scan_a + rows, 0, sizeof(uint32_t), S));
  SCK(scan_exclusive(h, h->scan_a, h->scan_b, rows + 1));
  uint32_t nfluid = 0;
  SCK(cudaMemcpyAsync(&nfluid, h->scan_b + rows, sizeof nfluid, cudaMemcpyDeviceToHost, S));
  /* walls: flags and their scan (the wall lists' start array) */
  k_wall_flags<<<(unsigned)((nc + 1 + SBLK - 1) / SBLK), SBLK, 0, S>>>(h->n, h->wall_start);
  SCK(scan_exclusive(h, h->wall_start, h->wall_start, nc + 1));
  uint32_t nwall = 0;
  SCK(cudaMemcpyAsync(&nwall, h->wall_start + nc, sizeof nwall, cudaMemcpyDeviceToHost, S));
  SCK(cudaStreamSynchronize(S));
  if ((size_t)nfluid + nwall > (size_t)h->cap) {
    snprintf(h->err, sizeof h->err, "seed_scene: %u particles exceed the capacity %d",
             nfluid + nwall, h->cap);
    return FLIPGPU_ETOOBIG;
  }
  float *arrs[] = {h->vx, h->vy, h->vz, h->nx, h->ny, h->nz, h->dens};
  for (float *p : arrs) SCK(cudaMemsetAsync(p, 0, h->cap * sizeof(float), S));
  k_scene_emit<<<rgrid, SBLK, 0, S>>>(a, h->scan_b, h->px, h->py, h->pz, h->vx, h->vy, h->vz,
                                       h->type, h->nx, h->ny, h->nz);
  cudaFree(h->wall_pos);
  cudaFree(h->wall_nrm);
  h->wall_pos = h->wall_nrm = nullptr;
  SCK(cudaMalloc(&h->wall_pos, (nwall ? nwall : 1) * sizeof(float4)));
  SCK(cudaMalloc(&h->wall_nrm, (nwall ? nwall : 1) * sizeof(float4)));
  k_wall_emit<<<(unsigned)((nc + SBLK - 1) / SBLK), SBLK, 0, S>>>(
      h->n, a.wall, nfluid, h->wall_start, h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->type,
      h->nx, h->ny, h->nz, h->wall_pos, h->wall_nrm);
  SCK(cudaGetLastError());
  SCK(cudaStreamSynchronize(S));
  h->np = (int)(nfluid + nwall);
  h->nwall = (int)nwall;
  h->cells_valid = false;
  FG_LAUNCHED(h, 6);
  return FLIPGPU_OK;
}
