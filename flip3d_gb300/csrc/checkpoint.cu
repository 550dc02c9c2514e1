/*
 * checkpoint.cu — the reference's checkpoint file (saveState / loadState,
 * src/flip3D.cpp:453-578): a host reader and writer of its byte layout, and
 * the handle-level save and load. The wall-normal grid the file carries is
 * what compute_wall_normal (src/flip3D.cpp:75-164) leaves for the current
 * walls, computed on the device from the static wall lists:
 *   wall cells: the normal of the cell's last wall particle in particle
 *     order (the walls' normals are nonzero);
 *   other cells with wall neighbours (the perimeter): the sum of those
 *     neighbours' normals in the order -i, +i, -j, +j, -k, +k, divided by its
 *     length hypot(hypot(x, y), z) taken in double and rounded to float,
 *     and the flag 1;
 *   every other cell 0 (the reference zeroes the cells that hold particles
 *     and leaves empty ones as allocated).
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "devcommon.cuh"

namespace {

/* src/common.h:34-45 with FLOAT = float: 72 bytes, no padding */
struct RefParticle {
  float p[3], u[3], n[3];
  char type, visible, remove, thinparticle;
  float tmp[2][3];
  float m, dens;
};
static_assert(sizeof(RefParticle) == 72, "the reference's particle record is 72 bytes");
constexpr long HEADER_BYTES = 4 + 4 + 4 + 8 + 4;

long expected_size(int n, long count) {
  const long n3 = (long)n * n * n;
  return HEADER_BYTES + count * (long)sizeof(RefParticle) + n3 * 4 * 5;
}

constexpr int CBLK = 256;

__global__ void k_wall_cells(int n, const uint32_t *__restrict__ wall_start,
                             const float4 *__restrict__ wall_nrm, float *__restrict__ wn) {
  const size_t c = (size_t)blockIdx.x * CBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  const uint32_t s = wall_start[c], e = wall_start[c + 1];
  float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (e > s) v = wall_nrm[e - 1];
  wn[4 * c + 0] = v.x;
  wn[4 * c + 1] = v.y;
  wn[4 * c + 2] = v.z;
  wn[4 * c + 3] = 0.0f;
}

__global__ void k_wall_perimeter(int n, const uint32_t *__restrict__ wall_start,
                                 float *__restrict__ wn) {
  const size_t c = (size_t)blockIdx.x * CBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  auto is_wall = [&](size_t q) { return wall_start[q + 1] > wall_start[q]; };
  if (is_wall(c)) return;
  const int k = (int)(c % n), j = (int)((c / n) % n), i = (int)(c / ((size_t)n * n));
  const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                        {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
  int sum = 0;
  float norm[3] = {0.0f, 0.0f, 0.0f};
  for (int m = 0; m < 6; m++) {
    const int si = nb[m][0], sj = nb[m][1], sk = nb[m][2];
    if (si < 0 || si > n - 1 || sj < 0 || sj > n - 1 || sk < 0 || sk > n - 1) continue;
    const size_t q = ((size_t)si * n + sj) * n + sk;
    if (!is_wall(q)) continue;
    sum++;
    norm[0] += wn[4 * q + 0];
    norm[1] += wn[4 * q + 1];
    norm[2] += wn[4 * q + 2];
  }
  float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (sum > 0) {
    const float d = (float)hypot(hypot((double)norm[0], (double)norm[1]), (double)norm[2]);
    out[0] = norm[0] / d;
    out[1] = norm[1] / d;
    out[2] = norm[2] / d;
    out[3] = 1.0f;
  }
  for (int q = 0; q < 4; q++) wn[4 * c + q] = out[q];
}

int set_err(FlipGpu *h, int code, const char *what) {
  if (h) snprintf(h->err, sizeof h->err, "%s", what);
  return code;
}

} // namespace

extern "C" {

int flipgpu_checkpoint_write(const char *path, const FlipCheckpoint *c) {
  if (!path || !c || c->n < 1 || c->count < 0 || (c->count && (!c->pos || !c->type)) ||
      !c->press || !c->wall_normal)
    return FLIPGPU_EINVAL;
  FILE *fp = fopen(path, "wb");
  if (!fp) return FLIPGPU_EINVAL;
  bool ok = fwrite(&c->count, sizeof(int), 1, fp) == 1 &&
            fwrite(&c->max_dens, sizeof(float), 1, fp) == 1 &&
            fwrite(&c->pour_time, sizeof(int), 1, fp) == 1 &&
            fwrite(c->pour_pos, 2 * sizeof(float), 1, fp) == 1 &&
            fwrite(&c->pour_rad, sizeof(float), 1, fp) == 1;
  std::vector<RefParticle> rec(4096);
  for (long base = 0; ok && base < c->count; base += (long)rec.size()) {
    const long m = std::min<long>((long)rec.size(), c->count - base);
    for (long q = 0; q < m; q++) {
      const long p = base + q;
      RefParticle &r = rec[q];
      std::memset(&r, 0, sizeof r);
      for (int d = 0; d < 3; d++) {
        r.p[d] = c->pos[3 * p + d];
        r.u[d] = c->vel ? c->vel[3 * p + d] : 0.0f;
        r.n[d] = c->nrm ? c->nrm[3 * p + d] : 0.0f;
      }
      r.type = (char)c->type[p];
      r.visible = c->visible ? (char)c->visible[p] : (char)(c->type[p] == CELL_FLUID);
      r.m = 1.0f;
      r.dens = c->dens ? c->dens[p] : 0.0f;
    }
    ok = fwrite(rec.data(), sizeof(RefParticle), (size_t)m, fp) == (size_t)m;
  }
  const size_t n3 = (size_t)c->n * c->n * c->n;
  ok = ok && fwrite(c->press, sizeof(float), n3, fp) == n3;
  ok = ok && fwrite(c->wall_normal, sizeof(float), 4 * n3, fp) == 4 * n3;
  ok = (fclose(fp) == 0) && ok;
  return ok ? FLIPGPU_OK : FLIPGPU_EINVAL;
}

int flipgpu_checkpoint_count(const char *path, int n, int *count) {
  if (!path || !count || n < 1) return FLIPGPU_EINVAL;
  FILE *fp = fopen(path, "rb");
  if (!fp) return FLIPGPU_EINVAL;
  int np = -1;
  const bool ok = fread(&np, sizeof(int), 1, fp) == 1 && fseek(fp, 0, SEEK_END) == 0;
  const long size = ok ? ftell(fp) : -1;
  fclose(fp);
  if (!ok || np < 0 || size != expected_size(n, np)) return FLIPGPU_EINVAL;
  *count = np;
  return FLIPGPU_OK;
}

int flipgpu_checkpoint_read(const char *path, FlipCheckpoint *c) {
  if (!path || !c || c->n < 1) return FLIPGPU_EINVAL;
  int np = 0;
  if (flipgpu_checkpoint_count(path, c->n, &np) != FLIPGPU_OK) return FLIPGPU_EINVAL;
  /* c->count is the capacity of every per-particle array given */
  const bool per_particle = c->pos || c->vel || c->nrm || c->type || c->visible || c->dens;
  if (c->count < 0) return FLIPGPU_EINVAL;
  if (np > c->count && per_particle) return FLIPGPU_ETOOBIG;
  FILE *fp = fopen(path, "rb");
  if (!fp) return FLIPGPU_EINVAL;
  bool ok = fread(&np, sizeof(int), 1, fp) == 1 &&
            fread(&c->max_dens, sizeof(float), 1, fp) == 1 &&
            fread(&c->pour_time, sizeof(int), 1, fp) == 1 &&
            fread(c->pour_pos, 2 * sizeof(float), 1, fp) == 1 &&
            fread(&c->pour_rad, sizeof(float), 1, fp) == 1;
  c->count = np;
  std::vector<RefParticle> rec(4096);
  for (long base = 0; ok && base < np; base += (long)rec.size()) {
    const long m = std::min<long>((long)rec.size(), np - base);
    ok = fread(rec.data(), sizeof(RefParticle), (size_t)m, fp) == (size_t)m;
    for (long q = 0; ok && q < m; q++) {
      const long p = base + q;
      const RefParticle &r = rec[q];
      for (int d = 0; d < 3; d++) {
        if (c->pos) c->pos[3 * p + d] = r.p[d];
        if (c->vel) c->vel[3 * p + d] = r.u[d];
        if (c->nrm) c->nrm[3 * p + d] = r.n[d];
      }
      if (c->type) c->type[p] = (uint8_t)r.type;
      if (c->visible) c->visible[p] = (uint8_t)r.visible;
      if (c->dens) c->dens[p] = r.dens;
    }
  }
  const size_t n3 = (size_t)c->n * c->n * c->n;
  std::vector<float> skip;
  float *press = c->press, *wn = c->wall_normal;
  if (!press || !wn) skip.resize(4 * n3);
  ok = ok && fread(press ? press : skip.data(), sizeof(float), n3, fp) == n3;
  ok = ok && fread(wn ? wn : skip.data(), sizeof(float), 4 * n3, fp) == 4 * n3;
  fclose(fp);
  return ok ? FLIPGPU_OK : FLIPGPU_EINVAL;
}

int flipgpu_save_state(FlipGpu *h, const char *path, int pour_time, const float *pour_pos,
                       float pour_rad) {
  if (!h || !path) return FLIPGPU_EINVAL;
  const int n = h->n, np = h->np;
  const size_t nc = h->nc;
  std::vector<float> pos(3 * (size_t)np), vel(3 * (size_t)np), nrm(3 * (size_t)np), dens(np);
  std::vector<uint8_t> type(np);
  std::vector<float> press(nc), wn(4 * nc);
  int r = flipgpu_get_particles(h, pos.data(), vel.data(), dens.data(), type.data(), 0);
  if (r != FLIPGPU_OK) return r;
  float *dwn = nullptr;
  if (cudaMalloc(&dwn, 4 * nc * sizeof(float)) != cudaSuccess)
    return set_err(h, FLIPGPU_ENOMEM, "save_state: no device memory for the wall normals");
  const unsigned g = (unsigned)((nc + CBLK - 1) / CBLK);
  k_wall_cells<<<g, CBLK, 0, h->stream>>>(n, h->wall_start, h->wall_nrm, dwn);
  k_wall_perimeter<<<g, CBLK, 0, h->stream>>>(n, h->wall_start, dwn);
  FG_LAUNCHED(h, 2);
  bool ok = cudaGetLastError() == cudaSuccess &&
            cudaMemcpyAsync(wn.data(), dwn, 4 * nc * sizeof(float), cudaMemcpyDeviceToHost,
                            h->stream) == cudaSuccess &&
            cudaMemcpyAsync(press.data(), h->press, nc * sizeof(float), cudaMemcpyDeviceToHost,
                            h->stream) == cudaSuccess;
  float *cx[3] = {h->nx, h->ny, h->nz};
  std::vector<float> comp(np);
  for (int d = 0; ok && np > 0 && d < 3; d++) {
    ok = cudaMemcpyAsync(comp.data(), cx[d], np * sizeof(float), cudaMemcpyDeviceToHost,
                         h->stream) == cudaSuccess &&
         cudaStreamSynchronize(h->stream) == cudaSuccess;
    for (int p = 0; ok && p < np; p++) nrm[3 * (size_t)p + d] = comp[p];
  }
  ok = ok && cudaStreamSynchronize(h->stream) == cudaSuccess;
  cudaFree(dwn);
  if (!ok) return set_err(h, FLIPGPU_ECUDA, "save_state: device copy failed");
  FlipCheckpoint c;
  std::memset(&c, 0, sizeof c);
  c.n = n;
  c.count = np;
  c.max_dens = h->max_dens;
  c.pour_time = pour_time;
  c.pour_pos[0] = pour_pos ? pour_pos[0] : 0.0f;
  c.pour_pos[1] = pour_pos ? pour_pos[1] : 0.0f;
  c.pour_rad = pour_rad;
  c.pos = pos.data();
  c.vel = vel.data();
  c.nrm = nrm.data();
  c.type = type.data();
  c.dens = dens.data();
  c.press = press.data();
  c.wall_normal = wn.data();
  if (flipgpu_checkpoint_write(path, &c) != FLIPGPU_OK)
    return set_err(h, FLIPGPU_EINVAL, "save_state: cannot write the file");
  return FLIPGPU_OK;
}

int flipgpu_load_state(FlipGpu *h, const char *path, int *pour_time, float *pour_pos,
                       float *pour_rad) {
  if (!h || !path) return FLIPGPU_EINVAL;
  int np = 0;
  if (flipgpu_checkpoint_count(path, h->n, &np) != FLIPGPU_OK)
    return set_err(h, FLIPGPU_EINVAL, "load_state: not a checkpoint of this grid size");
  if (np > h->cap) return set_err(h, FLIPGPU_ETOOBIG, "load_state: more particles than capacity");
  const size_t nc = h->nc;
  std::vector<float> pos(3 * (size_t)np), vel(3 * (size_t)np), nrm(3 * (size_t)np), dens(np);
  std::vector<uint8_t> type(np);
  std::vector<float> press(nc);
  FlipCheckpoint c;
  std::memset(&c, 0, sizeof c);
  c.n = h->n;
  c.count = np;
  c.pos = pos.data();
  c.vel = vel.data();
  c.nrm = nrm.data();
  c.type = type.data();
  c.dens = dens.data();
  c.press = press.data();
  if (flipgpu_checkpoint_read(path, &c) != FLIPGPU_OK)
    return set_err(h, FLIPGPU_EINVAL, "load_state: read failed");
  int r = flipgpu_set_particles(h, np, pos.data(), vel.data(), type.data(), nrm.data(),
                                dens.data(), 0);
  if (r != FLIPGPU_OK) return r;
  if ((r = flipgpu_set_grid(h, nullptr, nullptr, nullptr, nullptr, nullptr, press.data(), nullptr,
                            0)) != FLIPGPU_OK)
    return r;
  if ((r = flipgpu_set_max_density(h, c.max_dens)) != FLIPGPU_OK) return r;
  if (pour_time) *pour_time = c.pour_time;
  if (pour_pos) {
    pour_pos[0] = c.pour_pos[0];
    pour_pos[1] = c.pour_pos[1];
  }
  if (pour_rad) *pour_rad = c.pour_rad;
  return FLIPGPU_OK;
}

} // extern "C"
