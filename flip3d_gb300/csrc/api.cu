/*
 * api.cu — the C ABI of include/flipgpu.h: handle lifetime, transfers and
 * the orchestration of the per-step stages.
 */
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "autotune.h"
#include "devcommon.cuh"

namespace {

int fail(FlipGpu *h, int code, const char *fmt, ...) {
  if (h) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(h->err, sizeof h->err, fmt, ap);
    va_end(ap);
  }
  return code;
}

#define CK(h, call)                                                              \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess)                                                       \
      return fail((h), FLIPGPU_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T> cudaError_t dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, count * sizeof(T));
}

float largest_float_le(double d) {
  float f = (float)d;
  if ((double)f > d) f = nextafterf(f, -INFINITY);
  return f;
}
float largest_float_lt(double d) {
  float f = largest_float_le(d);
  if ((double)f == d) f = nextafterf(f, -INFINITY);
  return f;
}
float smallest_float_ge(double d) {
  float f = (float)d;
  if ((double)f < d) f = nextafterf(f, INFINITY);
  return f;
}
/* 1/x when x is an exact power of two (the reciprocal is then exact), else 0 */
float pow2_rcp(float x) {
  int e;
  float m = frexpf(x, &e);
  return (x > 0.0f && m == 0.5f) ? ldexpf(1.0f, 1 - e) : 0.0f;
}
void split(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

constexpr int BLK = 256;

__global__ void k_deinterleave(int np, const float *__restrict__ aos, float *__restrict__ x,
                               float *__restrict__ y, float *__restrict__ z) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= np) return;
  x[p] = aos[3 * (size_t)p];
  y[p] = aos[3 * (size_t)p + 1];
  z[p] = aos[3 * (size_t)p + 2];
}
__global__ void k_interleave(int np, const float *__restrict__ x, const float *__restrict__ y,
                             const float *__restrict__ z, float *__restrict__ aos) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= np) return;
  aos[3 * (size_t)p] = x[p];
  aos[3 * (size_t)p + 1] = y[p];
  aos[3 * (size_t)p + 2] = z[p];
}
__global__ void k_add_force(SimConst c, const uint8_t *__restrict__ type, float *__restrict__ vy) {
  int p = blockIdx.x * BLK + threadIdx.x;
  if (p >= c.np || type[p] != CELL_FLUID) return;
  vy[p] = refmath::add_fd(vy[p], c.grav_h, c.grav_l, c.grav);
}

/* Upload an AoS float[np][3] (host or device) into three SoA arrays. */
int put3(FlipGpu *h, const float *src, int on_device, float *x, float *y, float *z) {
  if (!src || h->np == 0) return FLIPGPU_OK;
  size_t bytes = (size_t)h->np * 3 * sizeof(float);
  float *stage = (float *)h->spos; /* 16 B per slot >= 12 B per particle */
  CK(h, cudaMemcpyAsync(stage, src, bytes,
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
  k_deinterleave<<<grid_for(h->np, BLK), BLK, 0, h->stream>>>(h->np, stage, x, y, z);
  FG_LAUNCHED(h, 1);
  CK(h, cudaGetLastError());
  return FLIPGPU_OK;
}

int get3(FlipGpu *h, float *dst, int on_device, const float *x, const float *y, const float *z,
         float *stage) {
  if (!dst || h->np == 0) return FLIPGPU_OK;
  size_t bytes = (size_t)h->np * 3 * sizeof(float);
  k_interleave<<<grid_for(h->np, BLK), BLK, 0, h->stream>>>(h->np, x, y, z, stage);
  FG_LAUNCHED(h, 1);
  CK(h, cudaGetLastError());
  CK(h, cudaMemcpyAsync(dst, stage, bytes,
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
  return FLIPGPU_OK;
}

/* Static wall lists: wall particles grouped by cell in particle order
 * (walls never move, so the wall part of every cell list is fixed). */
int build_walls(FlipGpu *h, const std::vector<float> &pos, const std::vector<uint8_t> &type) {
  const int n = h->n;
  const float fn = (float)n;
  std::vector<uint32_t> start(h->nc + 1, 0);
  std::vector<uint32_t> key;
  std::vector<int> idx;
  for (int p = 0; p < h->np; p++) {
    if (type[p] != CELL_WALL) continue;
    int c[3];
    for (int a = 0; a < 3; a++)
      c[a] = (int)fmaxf(0.0f, fminf((float)(n - 1), fn * pos[3 * (size_t)p + a]));
    uint32_t kk = (uint32_t)(((size_t)c[0] * n + c[1]) * n + c[2]);
    key.push_back(kk);
    idx.push_back(p);
    start[kk + 1]++;
  }
  for (size_t c = 0; c < h->nc; c++) start[c + 1] += start[c];
  const size_t nw = idx.size();
  std::vector<uint32_t> fillp(start.begin(), start.end() - 1);
  std::vector<float4> wpos(nw), wnrm(nw);
  /* nrm is uploaded separately; read it back from the canonical arrays */
  std::vector<float> nx(h->np), ny(h->np), nz(h->np);
  CK(h, cudaMemcpyAsync(nx.data(), h->nx, h->np * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaMemcpyAsync(ny.data(), h->ny, h->np * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaMemcpyAsync(nz.data(), h->nz, h->np * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  for (size_t w = 0; w < nw; w++) {
    int p = idx[w];
    uint32_t slot = fillp[key[w]]++;
    wpos[slot] = make_float4(pos[3 * (size_t)p], pos[3 * (size_t)p + 1], pos[3 * (size_t)p + 2], 0.0f);
    wnrm[slot] = make_float4(nx[p], ny[p], nz[p], 0.0f);
  }
  cudaFree(h->wall_pos);
  cudaFree(h->wall_nrm);
  h->wall_pos = h->wall_nrm = nullptr;
  CK(h, dalloc(&h->wall_pos, nw));
  CK(h, dalloc(&h->wall_nrm, nw));
  h->nwall = (int)nw;
  CK(h, cudaMemcpyAsync(h->wall_start, start.data(), (h->nc + 1) * sizeof(uint32_t),
                        cudaMemcpyHostToDevice, h->stream));
  if (nw) {
    CK(h, cudaMemcpyAsync(h->wall_pos, wpos.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->wall_nrm, wnrm.data(), nw * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

void free_all(FlipGpu *h) {
  void *ptrs[] = {h->px, h->py, h->pz, h->vx, h->vy, h->vz, h->dens, h->type, h->nx, h->ny,
                  h->nz, h->key, h->rank, h->perm, h->cell_start, h->cell_count, h->spos,
                  h->spg, h->svel, h->sdens, h->wall_start, h->wall_pos, h->wall_nrm, h->u[0],
                  h->u[1], h->u[2], h->us[0], h->us[1], h->us[2], h->A, h->L, h->press,
                  h->div, h->press_lo, h->ir_b, h->ir_e, h->r, h->z, h->s, h->s1, h->w, h->w1, h->pdir, h->chunk_off, h->chunk_list, h->bar, h->P, h->Pf, h->diag,
                  h->partial, h->scal,
                  h->iflags, h->flag, h->scan_a, h->scan_b, h->scan_tmp, h->stuck_idx,
                  h->water_idx, h->stage,
                  h->ticket, h->dstep, h->repo_draw, h->repo_res, h->repo_old,
                  h->repo_cnt, h->repo_start, h->repo_list, h->repo_state, h->cell_mid};
  for (void *p : ptrs)
    if (p) cudaFree(p);
}

/* Stage timing: one event per stage boundary; flushed after the step. */
struct StageClock {
  FlipGpu *h;
  int last = -1;
  bool used[FLIPGPU_NSTAGES] = {};
  int order[FLIPGPU_NSTAGES + 1];
  int nmark = 0;
  explicit StageClock(FlipGpu *hh) : h(hh) {}
  void mark(int stage) {
    if (!h->prof_on) return;
    cudaEventRecord(h->prof_ev[nmark], h->stream);
    order[nmark++] = stage;
  }
  void flush() {
    ktime_flush(h);
    if (!h->prof_on || nmark < 2) return;
    cudaEventSynchronize(h->prof_ev[nmark - 1]);
    for (int i = 0; i + 1 < nmark; i++) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, h->prof_ev[i], h->prof_ev[i + 1]);
      h->prof_ms[order[i]] += ms;
      h->prof_calls[order[i]]++;
    }
  }
};

} // namespace

void ktime_begin(FlipGpu *h, const char *name) {
  if (!h->prof_on) return;
  if (h->kt_n >= FlipGpu::KT_SLOTS) ktime_flush(h); /* calls outside a step: read as we go */
  if (!h->kt_ready) {
    for (int i = 0; i < 2 * FlipGpu::KT_SLOTS; i++)
      if (cudaEventCreate(&h->kt_ev[i]) != cudaSuccess) return;
    h->kt_ready = 1;
  }
  cudaEventRecord(h->kt_ev[2 * h->kt_n], h->stream);
  h->kt_pending[h->kt_n] = name;
}

void ktime_end(FlipGpu *h) {
  if (!h->prof_on || !h->kt_ready || h->kt_n >= FlipGpu::KT_SLOTS) return;
  cudaEventRecord(h->kt_ev[2 * h->kt_n + 1], h->stream);
  h->kt_n++;
}

void ktime_flush(FlipGpu *h) {
  if (h->kt_n == 0) return;
  cudaEventSynchronize(h->kt_ev[2 * h->kt_n - 1]);
  for (int i = 0; i < h->kt_n; i++) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, h->kt_ev[2 * i], h->kt_ev[2 * i + 1]) != cudaSuccess) continue;
    int k = 0;
    while (k < h->kt_nnames && strcmp(h->kt_name[k], h->kt_pending[i]) != 0) k++;
    if (k == h->kt_nnames) {
      if (k == FlipGpu::KT_NAMES) continue;
      h->kt_name[k] = h->kt_pending[i];
      h->kt_ms[k] = 0.0;
      h->kt_calls[k] = 0;
      h->kt_nnames++;
    }
    h->kt_ms[k] += ms;
    h->kt_calls[k]++;
  }
  h->kt_n = 0;
  cudaGetLastError();
}

/* After the corrector's spring: the positions are final, so the transfer
 * stream interleaves them into the sorted grid-position buffer (unused by
 * the resample) and copies them to the host while the resample runs. */
cudaError_t xfer_positions_out(FlipGpu *h) {
  cudaError_t e = cudaEventRecord(h->xev[2], h->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h->xstream, h->xev[2], 0);
  if (e != cudaSuccess) return e;
  float *stage = reinterpret_cast<float *>(h->spg);
  k_interleave<<<grid_for(h->np, BLK), BLK, 0, h->xstream>>>(h->np, h->px, h->py, h->pz, stage);
  FG_LAUNCHED(h, 1);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->xfer_pos_out, stage, (size_t)h->np * 3 * sizeof(float),
                        cudaMemcpyDeviceToHost, h->xstream);
  return e;
}


SimConst make_const(const FlipGpu *h) {
  SimConst c;
  const FlipGpuParams &p = h->prm;
  const int n = h->n;
  c.n = n;
  c.np = h->np;
  c.fn = (float)n;
  c.h = (float)(1.0 / n);
  c.density = p.density;
  float kh = (float)(4.0 * (double)p.density / n);
  c.kd_hh = kh * kh;
  c.kd_rcp = pow2_rcp(c.kd_hh);
  c.kd_inv = 1.0f / c.kd_hh;
  c.max_dens = h->max_dens;
  const float RE = (float)1.4;
  c.re_p2g_hh = RE * RE;
  c.re_corr = (float)((double)p.density / n);
  c.re_corr_hh = c.re_corr * c.re_corr;
  c.corr_rcp = pow2_rcp(c.re_corr_hh);
  c.corr_inv = 1.0f / c.re_corr_hh;
  c.re_repo = (float)(1.0 / n);
  c.re_repo_hh = c.re_repo * c.re_repo;
  c.r2_floor = smallest_float_ge(1.0e-5);
  c.sharp_small_p2g = (float)fmax((double)c.re_p2g_hh / 1.0e-5 - 1.0, 0.0);
  c.sharp_small_corr = (float)fmax((double)c.re_corr_hh / 1.0e-5 - 1.0, 0.0);
  c.sharp_small_repo = (float)fmax((double)c.re_repo_hh / 1.0e-5 - 1.0, 0.0);
  c.wall_r = (float)(1.0 / n);
  c.wall_hi = (float)(1.0 - (double)c.wall_r);
  c.wall_hi_thr = largest_float_le(1.0 - (double)c.wall_r);
  c.push_re = 1.5 * (double)p.density / n;
  c.push_re_thr = largest_float_lt(c.push_re);
  c.corr_near_thr = largest_float_le(0.1 * (double)c.re_corr);
  double re2 = (double)c.re_corr * (double)c.re_corr;
  c.corr_cut2 = smallest_float_ge(re2 * (1.0 + 1.0 / 256.0));
  c.corr_reach = smallest_float_ge((double)c.re_corr * (1.0 + 1.0 / 256.0));
  c.dt = p.dt;
  c.dt_f = (float)p.dt;
  c.kick_fluid = 0.01 * (double)c.re_corr / (double)c.dt_f;
  c.kick_wall = 0.05 * (double)c.re_corr / (double)c.dt_f;
  split(p.dt, c.dt_h, c.dt_l);
  c.grav = -p.dt * p.gravity;
  split(c.grav, c.grav_h, c.grav_l);
  c.c1 = 1.0 - p.alpha;
  c.c2 = p.alpha;
  split(c.c1, c.c1h, c.c1l);
  split(c.c2, c.c2h, c.c2l);
  float dens3 = p.density * p.density * p.density;
  float n0 = (float)(1.0 / (double)dens3);
  c.l0 = 0.2 * (double)n0;
  split(c.l0, c.l0h, c.l0l);
  c.seed = p.seed;
  c.step = h->step;
  c.dstep = h->dstep;
  return c;
}

extern "C" {

void flipgpu_default_params(FlipGpuParams *p, int n, int max_particles) {
  std::memset(p, 0, sizeof *p);
  p->n = n;
  p->max_particles = max_particles;
  p->density = 0.5f;
  p->alpha = 0.95;
  p->dt = 0.6e-2;
  p->gravity = 9.8;
  p->subcell = 1;
  p->seed = 0;
  p->solve_mode = FLIPGPU_SOLVE_REF;
  p->precond = FLIPGPU_PRECOND_REF;
  p->mic_tau = 0.0;
  p->rel_tol = 0.0;
  p->eps_abs = -1.0;
  p->max_iters = 0;
  p->refine_steps = 4;
  p->arith = FLIPGPU_ARITH_REF;
  p->mg_sweeps = 0;
}

const char *flipgpu_last_error(const FlipGpu *h) { return h ? h->err : "null handle"; }

int flipgpu_particle_count(const FlipGpu *h) { return h ? h->np : -1; }

int flipgpu_create(const FlipGpuParams *p, FlipGpu **out) {
  if (!p || !out) return FLIPGPU_EINVAL;
  *out = nullptr;
  if (p->n < 3 || p->n > 1024 || p->max_particles < 0) return FLIPGPU_EINVAL;
  const size_t n = (size_t)p->n;
  if (n * n * n >= 0xffffffffull) return FLIPGPU_EINVAL;
  FlipGpu *h = new (std::nothrow) FlipGpu();
  if (!h) return FLIPGPU_ENOMEM;
  std::memset((void *)h, 0, sizeof *h);
  h->prm = *p;
  h->n = p->n;
  h->cap = p->max_particles;
  h->nc = n * n * n;
  h->nf = (n + 1) * n * n;
  h->max_dens = 1.0f;
  const size_t cap = (size_t)h->cap;
  const size_t nc = h->nc, nf = h->nf;
  cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return FLIPGPU_ECUDA;
  }
  h->stream = h->own_stream;
  cudaEventCreate(&h->ev0);
  cudaEventCreate(&h->ev1);
  for (int i = 0; i <= FLIPGPU_NSTAGES; i++) cudaEventCreate(&h->prof_ev[i]);
  size_t scan_n = cap > nc + 1 ? cap : nc + 1;
  h->scan_cap = (scan_n + 4095) / 4096 + 1;
#define AL(ptr, cnt)                                                  \
  if ((e = dalloc(&(ptr), (cnt))) != cudaSuccess) {                   \
    free_all(h);                                                      \
    cudaStreamDestroy(h->own_stream);                                 \
    delete h;                                                         \
    return FLIPGPU_ENOMEM;                                            \
  }
  AL(h->px, cap) AL(h->py, cap) AL(h->pz, cap) AL(h->vx, cap) AL(h->vy, cap) AL(h->vz, cap)
  AL(h->dens, cap) AL(h->type, cap) AL(h->nx, cap) AL(h->ny, cap) AL(h->nz, cap)
  AL(h->key, cap) AL(h->rank, cap) AL(h->perm, cap) AL(h->cell_start, nc + 1)
  AL(h->cell_count, nc + 1) AL(h->spos, cap) AL(h->spg, cap) AL(h->svel, cap)
  AL(h->sdens, cap) AL(h->wall_start, nc + 1) AL(h->cell_mid, nc)
  for (int c = 0; c < 3; c++) {
    AL(h->u[c], nf) AL(h->us[c], nf)
  }
  AL(h->A, nc) AL(h->L, nc) AL(h->press, nc) AL(h->div, nc) AL(h->r, nc) AL(h->z, nc)
  AL(h->press_lo, nc) AL(h->ir_b, nc) AL(h->ir_e, nc)
  AL(h->s, nc) AL(h->s1, nc) AL(h->w, nc) AL(h->w1, nc) AL(h->pdir, nc) AL(h->chunk_off, nc / 128 + 2) AL(h->chunk_list, nc / 128 + 1) AL(h->P, 2 * nc) AL(h->Pf, nc) AL(h->diag, nc)
  AL(h->partial, 8192) AL(h->bar, 2)
  AL(h->scal, SC_COUNT) AL(h->iflags, IF_COUNT) AL(h->flag, cap) AL(h->scan_a, scan_n)
  AL(h->scan_b, scan_n) AL(h->scan_tmp, h->scan_cap) AL(h->stuck_idx, cap)
  AL(h->water_idx, nc) AL(h->stage, 3 * cap)
  AL(h->repo_draw, cap) AL(h->repo_res, cap) AL(h->repo_old, cap)
  AL(h->repo_cnt, cap + 1) AL(h->repo_start, cap + 1) AL(h->repo_list, cap)
  AL(h->repo_state, cap)
  AL(h->ticket, 1) AL(h->dstep, 1)
#undef AL
  for (int c = 0; c < 3; c++) {
    cudaMemsetAsync(h->u[c], 0, nf * sizeof(float), h->stream);
    cudaMemsetAsync(h->us[c], 0, nf * sizeof(float), h->stream);
  }
  cudaMemsetAsync(h->A, 0, nc, h->stream);
  cudaMemsetAsync(h->L, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->press, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->press_lo, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->div, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->wall_start, 0, (nc + 1) * sizeof(uint32_t), h->stream);
  cudaMemsetAsync(h->iflags, 0, IF_COUNT * sizeof(int), h->stream);
  cudaMemsetAsync(h->s, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->s1, 0, nc * sizeof(float), h->stream);
  cudaMemsetAsync(h->dstep, 0, sizeof(int64_t), h->stream);
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    free_all(h);
    delete h;
    return FLIPGPU_ECUDA;
  }
  if (cg_grid_size(h->cg_grid) != 0)
    for (int v = 0; v < CG_VARIANTS; v++) h->cg_grid[v] = 0;
  /* the multigrid or wavefront buffers now, so that a captured step never
   * allocates */
  if (p->precond == FLIPGPU_PRECOND_MG && p->n % 4 == 0 && p->n >= 8) {
    int r = mg_alloc(h);
    if (r != FLIPGPU_OK) {
      free_all(h);
      cudaStreamDestroy(h->own_stream);
      delete h;
      return r;
    }
  }
  if (p->precond == FLIPGPU_PRECOND_IC && p->solve_mode == FLIPGPU_SOLVE_FAST) {
    int r = ic_alloc(h);
    if (r != FLIPGPU_OK) {
      mg_free(h);
      free_all(h);
      cudaStreamDestroy(h->own_stream);
      delete h;
      return r;
    }
  }
  if (particles_init_device() != 0) {
    free_all(h);
    cudaStreamDestroy(h->own_stream);
    delete h;
    return FLIPGPU_ECUDA;
  }
  *out = h;
  return FLIPGPU_OK;
}

int flipgpu_destroy(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  cudaStreamSynchronize(h->stream);
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  export_free(h);
  mesh_free(h);
  mg_free(h);
  ic_free(h);
  if (h->xstream) {
    cudaStreamSynchronize(h->xstream);
    for (int e = 0; e < 3; e++) cudaEventDestroy(h->xev[e]);
    cudaStreamDestroy(h->xstream);
  }
  if (h->wdelta) {
    cudaFree(h->wdelta);
    cudaFree(h->wpart);
    cudaEventDestroy(h->wev[0]);
    cudaEventDestroy(h->wev[1]);
  }
  if (h->cap_b) {
    cudaFree(h->cap_b);
    cudaFree(h->cap_x0);
    cudaFree(h->cap_r0);
  }
  free_all(h);
  cudaEventDestroy(h->ev0);
  cudaEventDestroy(h->ev1);
  for (int i = 0; i <= FLIPGPU_NSTAGES; i++) cudaEventDestroy(h->prof_ev[i]);
  if (h->kt_ready)
    for (int i = 0; i < 2 * FlipGpu::KT_SLOTS; i++) cudaEventDestroy(h->kt_ev[i]);
  cudaStreamDestroy(h->own_stream);
  delete h;
  return FLIPGPU_OK;
}

int flipgpu_set_params(FlipGpu *h, const FlipGpuParams *p) {
  if (!h || !p) return FLIPGPU_EINVAL;
  if (p->n != h->prm.n || p->max_particles != h->prm.max_particles)
    return fail(h, FLIPGPU_EINVAL, "set_params: n and max_particles are fixed per handle");
  if (p->precond == FLIPGPU_PRECOND_MG && p->n % 4 == 0 && p->n >= 8) {
    int r = mg_alloc(h);
    if (r != FLIPGPU_OK) return fail(h, r, "set_params: multigrid buffers");
  }
  if (p->precond == FLIPGPU_PRECOND_IC && p->solve_mode == FLIPGPU_SOLVE_FAST) {
    int r = ic_alloc(h);
    if (r != FLIPGPU_OK) return fail(h, r, "set_params: wavefront buffers");
  }
  /* the two arithmetics order a cell's particles differently (FAST by z
   * half): lists sorted under the other one are sorted again before use */
  if (p->arith != h->prm.arith) h->cells_valid = false;
  h->prm = *p;
  return FLIPGPU_OK;
}

int flipgpu_set_stream(FlipGpu *h, void *stream) {
  if (!h) return FLIPGPU_EINVAL;
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return FLIPGPU_OK;
}

int flipgpu_sync(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_set_step(FlipGpu *h, int64_t step) {
  if (!h) return FLIPGPU_EINVAL;
  h->step = step;
  CK(h, cudaMemcpyAsync(h->dstep, &h->step, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_count(const FlipGpu *h) { return h ? h->np : -1; }
int64_t flipgpu_launch_count(const FlipGpu *h) { return h ? h->launches : -1; }

int flipgpu_set_particles(FlipGpu *h, int count, const float *pos, const float *vel,
                          const uint8_t *type, const float *nrm, const float *dens,
                          int on_device) {
  if (!h || count < 0 || count > h->cap) return fail(h, FLIPGPU_EINVAL, "bad particle count %d", count);
  if (!pos || !type) return fail(h, FLIPGPU_EINVAL, "pos and type are required");
  h->np = count;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  CK(h, cudaMemsetAsync(h->vx, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->vy, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->vz, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->nx, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->ny, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->nz, 0, h->cap * sizeof(float), h->stream));
  CK(h, cudaMemsetAsync(h->dens, 0, h->cap * sizeof(float), h->stream));
  int r;
  if ((r = put3(h, pos, on_device, h->px, h->py, h->pz)) != FLIPGPU_OK) return r;
  if ((r = put3(h, vel, on_device, h->vx, h->vy, h->vz)) != FLIPGPU_OK) return r;
  if ((r = put3(h, nrm, on_device, h->nx, h->ny, h->nz)) != FLIPGPU_OK) return r;
  CK(h, cudaMemcpyAsync(h->type, type, count, kind, h->stream));
  if (dens) CK(h, cudaMemcpyAsync(h->dens, dens, count * sizeof(float), kind, h->stream));
  /* host copies of positions and types for the static wall lists */
  std::vector<float> hpos((size_t)count * 3);
  std::vector<uint8_t> htype(count);
  CK(h, cudaMemcpyAsync(hpos.data(), pos, hpos.size() * sizeof(float),
                        on_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, h->stream));
  CK(h, cudaMemcpyAsync(htype.data(), type, count,
                        on_device ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->cells_valid = false;
  return build_walls(h, hpos, htype);
}

int flipgpu_get_particles(FlipGpu *h, float *pos, float *vel, float *dens, uint8_t *type,
                          int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  int r;
  if ((r = get3(h, pos, on_device, h->px, h->py, h->pz, h->stage)) != FLIPGPU_OK) return r;
  if ((r = get3(h, vel, on_device, h->vx, h->vy, h->vz, h->stage + 0)) != FLIPGPU_OK) return r;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (dens) CK(h, cudaMemcpyAsync(dens, h->dens, h->np * sizeof(float), kind, h->stream));
  if (type) CK(h, cudaMemcpyAsync(type, h->type, h->np, kind, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_set_grid(FlipGpu *h, const float *u0, const float *u1, const float *u2,
                     const uint8_t *A, const float *L, const float *press, const float *div,
                     int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const float *us[3] = {u0, u1, u2};
  for (int c = 0; c < 3; c++)
    if (us[c]) CK(h, cudaMemcpyAsync(h->u[c], us[c], h->nf * sizeof(float), kind, h->stream));
  if (A) CK(h, cudaMemcpyAsync(h->A, A, h->nc, kind, h->stream));
  if (L) CK(h, cudaMemcpyAsync(h->L, L, h->nc * sizeof(float), kind, h->stream));
  if (press) {
    CK(h, cudaMemcpyAsync(h->press, press, h->nc * sizeof(float), kind, h->stream));
    h->press_lo_valid = 0;
  }
  if (div) CK(h, cudaMemcpyAsync(h->div, div, h->nc * sizeof(float), kind, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_get_grid(FlipGpu *h, float *u0, float *u1, float *u2, uint8_t *A, float *L,
                     float *press, float *div, int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  float *us[3] = {u0, u1, u2};
  for (int c = 0; c < 3; c++)
    if (us[c]) CK(h, cudaMemcpyAsync(us[c], h->u[c], h->nf * sizeof(float), kind, h->stream));
  if (A) CK(h, cudaMemcpyAsync(A, h->A, h->nc, kind, h->stream));
  if (L) CK(h, cudaMemcpyAsync(L, h->L, h->nc * sizeof(float), kind, h->stream));
  if (press) CK(h, cudaMemcpyAsync(press, h->press, h->nc * sizeof(float), kind, h->stream));
  if (div) CK(h, cudaMemcpyAsync(div, h->div, h->nc * sizeof(float), kind, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_get_cells(FlipGpu *h, uint32_t *cell_start, uint32_t *perm, int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->lists_exist) return fail(h, FLIPGPU_EINVAL, "no cell lists: call flipgpu_sort first");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (cell_start)
    CK(h, cudaMemcpyAsync(cell_start, h->cell_start, (h->nc + 1) * sizeof(uint32_t), kind, h->stream));
  if (perm) CK(h, cudaMemcpyAsync(perm, h->perm, h->np * sizeof(uint32_t), kind, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_set_max_density(FlipGpu *h, float md) {
  if (!h || !(md > 0.0f)) return FLIPGPU_EINVAL;
  h->max_dens = md;
  return FLIPGPU_OK;
}

int flipgpu_calibrate_max_density(FlipGpu *h, float *out) {
  if (!h) return FLIPGPU_EINVAL;
  FlipGpuParams p = h->prm;
  p.max_particles = 1000;
  FlipGpu *t = nullptr;
  int r = flipgpu_create(&p, &t);
  if (r != FLIPGPU_OK) return fail(h, r, "calibration handle: %d", r);
  const float hh = (float)((double)p.density / p.n);
  std::vector<float> pos(3000);
  std::vector<uint8_t> type(1000, CELL_FLUID);
  int m = 0;
  for (int i = 0; i < 10; i++)
    for (int j = 0; j < 10; j++)
      for (int k = 0; k < 10; k++, m++) {
        pos[3 * m] = (float)((i + 0.5) * (double)hh);
        pos[3 * m + 1] = (float)((j + 0.5) * (double)hh);
        pos[3 * m + 2] = (float)((k + 0.5) * (double)hh);
      }
  std::vector<float> dens(1000);
  r = flipgpu_set_particles(t, 1000, pos.data(), nullptr, type.data(), nullptr, nullptr, 0);
  if (r == FLIPGPU_OK) r = flipgpu_set_max_density(t, 1.0f);
  if (r == FLIPGPU_OK) r = flipgpu_sort(t);
  if (r == FLIPGPU_OK) r = flipgpu_compute_density(t);
  if (r == FLIPGPU_OK) r = flipgpu_get_particles(t, nullptr, nullptr, dens.data(), nullptr, 0);
  h->launches += t->launches;
  flipgpu_destroy(t);
  if (r != FLIPGPU_OK) return fail(h, r, "calibration failed");
  float md = 0.0f;
  for (float d : dens) md = fmaxf(md, d);
  h->max_dens = md;
  if (out) *out = md;
  return FLIPGPU_OK;
}

/* ------------------------------------------------------------- stages */

int flipgpu_sort(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  CK(h, launch_sort(h, 0));
  return FLIPGPU_OK;
}

int flipgpu_compute_density(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cells_valid) CK(h, launch_sort(h, 0));
  CK(h, launch_density(h));
  return FLIPGPU_OK;
}

int flipgpu_mark_water(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cells_valid) CK(h, launch_sort(h, 0));
  CK(h, launch_mark_water(h));
  return FLIPGPU_OK;
}

int flipgpu_add_force(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  SimConst c = make_const(h);
  if (h->np) {
    k_add_force<<<grid_for(h->np, BLK), BLK, 0, h->stream>>>(c, h->type, h->vy);
    FG_LAUNCHED(h, 1);
    CK(h, cudaGetLastError());
    if (h->cells_valid) CK(h, launch_payload(h, 0));
  }
  return FLIPGPU_OK;
}

int flipgpu_p2g(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cells_valid) CK(h, launch_sort(h, 0));
  CK(h, launch_p2g(h, 0));
  return FLIPGPU_OK;
}

int flipgpu_g2p(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  CK(h, launch_g2p(h));
  if (h->cells_valid) CK(h, launch_payload(h, 0));
  return FLIPGPU_OK;
}

/* Point buffers: device pointers are used directly; host ones are staged
 * through h->stage (3*cap floats) in chunks. */
static int point_query(FlipGpu *h, int count, const float *pts, float *io, int on_device,
                       int what, float re) {
  if (!h || count < 0 || (count > 0 && (!pts || !io))) return FLIPGPU_EINVAL;
  if (what == 1) {
    if (!h->lists_exist) return fail(h, FLIPGPU_EINVAL, "resample: no cell lists");
    /* the lists of the last sort over the particles' current data, as the
     * reference's sorter keeps particle pointers */
    CK(h, launch_payload(h, 0));
  }
  if (on_device) {
    CK(h, what == 0 ? launch_fetch_points(h, count, pts, io)
                    : launch_resample_points(h, count, pts, io, re));
    return FLIPGPU_OK;
  }
  const int chunk = h->cap > 0 ? (h->cap > 1 ? h->cap / 2 : 1) : 0;
  if (chunk == 0) return fail(h, FLIPGPU_EINVAL, "no staging capacity");
  float *dp = h->stage, *dio = h->stage + 3 * (size_t)chunk;
  for (int off = 0; off < count; off += chunk) {
    int m = count - off < chunk ? count - off : chunk;
    size_t bytes = (size_t)m * 3 * sizeof(float);
    CK(h, cudaMemcpyAsync(dp, pts + 3 * (size_t)off, bytes, cudaMemcpyHostToDevice, h->stream));
    if (what == 1)
      CK(h, cudaMemcpyAsync(dio, io + 3 * (size_t)off, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(h, what == 0 ? launch_fetch_points(h, m, dp, dio)
                    : launch_resample_points(h, m, dp, dio, re));
    CK(h, cudaMemcpyAsync(io + 3 * (size_t)off, dio, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
  }
  return FLIPGPU_OK;
}

int flipgpu_fetch_velocity(FlipGpu *h, int count, const float *pts, float *out, int on_device) {
  return point_query(h, count, pts, out, on_device, 0, 0.0f);
}

int flipgpu_resample(FlipGpu *h, int count, const float *pts, float *vel, float re,
                     int on_device) {
  return point_query(h, count, pts, vel, on_device, 1, re);
}

int flipgpu_get_pressure(FlipGpu *h, double *press, int on_device) {
  if (!h || !press) return FLIPGPU_EINVAL;
  double *dst = press;
  if (!on_device) CK(h, cudaMalloc(&dst, h->nc * sizeof(double)));
  launch_pressure_double(h, dst);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !on_device) {
    e = cudaMemcpyAsync(press, dst, h->nc * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  }
  if (!on_device) cudaFree(dst);
  if (e != cudaSuccess) return fail(h, FLIPGPU_ECUDA, "get_pressure: %s", cudaGetErrorString(e));
  return FLIPGPU_OK;
}

int flipgpu_solve(FlipGpu *h, FlipGpuSolveStats *st) {
  if (!h) return FLIPGPU_EINVAL;
  return run_solve(h, st);
}

int flipgpu_implicit(FlipGpu *h, int count, const float *pts, double *out, int on_device) {
  if (!h || count < 0 || (count > 0 && (!pts || !out))) return FLIPGPU_EINVAL;
  if (!h->lists_exist) return fail(h, FLIPGPU_EINVAL, "implicit: no cell lists");
  if (on_device) {
    CK(h, launch_implicit_points(h, count, pts, out));
    return FLIPGPU_OK;
  }
  /* points (3 floats) and values (1 double) share the staging buffer */
  const int chunk = (int)(((size_t)h->cap * 3 / 5) & ~(size_t)1);
  if (chunk <= 0) return fail(h, FLIPGPU_EINVAL, "no staging capacity");
  float *dp = h->stage;
  double *dout = reinterpret_cast<double *>(h->stage + 3 * (size_t)chunk);
  for (int off = 0; off < count; off += chunk) {
    int m = count - off < chunk ? count - off : chunk;
    CK(h, cudaMemcpyAsync(dp, pts + 3 * (size_t)off, (size_t)m * 3 * sizeof(float),
                          cudaMemcpyHostToDevice, h->stream));
    CK(h, launch_implicit_points(h, m, dp, dout));
    CK(h, cudaMemcpyAsync(out + off, dout, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
  }
  return FLIPGPU_OK;
}

int flipgpu_set_warm_start(FlipGpu *h, FlipUNet *u) {
  if (!h) return FLIPGPU_EINVAL;
  if (u && h->n % 8 != 0)
    return fail(h, FLIPGPU_EINVAL, "warm start needs a grid that is a multiple of 8 cells");
  h->warm = u;
  return FLIPGPU_OK;
}

int flipgpu_set_capture(FlipGpu *h, int on) {
  if (!h) return FLIPGPU_EINVAL;
  if (on && !h->cap_b) {
    CK(h, cudaMalloc(&h->cap_b, h->nc * sizeof(float)));
    CK(h, cudaMalloc(&h->cap_x0, h->nc * sizeof(float)));
    CK(h, cudaMalloc(&h->cap_r0, h->nc * sizeof(float)));
  }
  h->capture = on ? 1 : 0;
  return FLIPGPU_OK;
}

int flipgpu_get_solve_system(FlipGpu *h, uint8_t *A, float *L, float *b, float *x0, float *r0,
                             float *x, int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cap_b) return fail(h, FLIPGPU_EINVAL, "get_solve_system: capture is off");
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (A) CK(h, cudaMemcpyAsync(A, h->A, h->nc, k, h->stream));
  if (L) CK(h, cudaMemcpyAsync(L, h->L, h->nc * sizeof(float), k, h->stream));
  if (b) CK(h, cudaMemcpyAsync(b, h->cap_b, h->nc * sizeof(float), k, h->stream));
  if (x0) CK(h, cudaMemcpyAsync(x0, h->cap_x0, h->nc * sizeof(float), k, h->stream));
  if (r0) CK(h, cudaMemcpyAsync(r0, h->cap_r0, h->nc * sizeof(float), k, h->stream));
  if (x) CK(h, cudaMemcpyAsync(x, h->press, h->nc * sizeof(float), k, h->stream));
  if (!on_device) CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_mesh(FlipGpu *h, int64_t *n_vertices, int64_t *n_faces) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->lists_exist) return fail(h, FLIPGPU_EINVAL, "mesh: no cell lists");
  int r = mesh_run(h, n_vertices, n_faces);
  if (r != FLIPGPU_OK) return fail(h, r, "mesh: %s", cudaGetErrorString(cudaGetLastError()));
  return FLIPGPU_OK;
}

int flipgpu_get_mesh(FlipGpu *h, double *vertices, double *normals, int32_t *faces,
                     float *field) {
  if (!h) return FLIPGPU_EINVAL;
  int r = mesh_get(h, vertices, normals, faces, field);
  if (r != FLIPGPU_OK) return fail(h, r, "get_mesh: no mesh or copy failed");
  return FLIPGPU_OK;
}

int flipgpu_project(FlipGpu *h, FlipGpuSolveStats *st) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cells_valid) CK(h, launch_sort(h, 0));
  CK(h, launch_mark_water(h)); /* L = levelset per cell (src/flip3D.cpp:824-826) */
  CK(h, launch_divergence(h));
  int r = run_solve(h, st);
  if (r != FLIPGPU_OK) return r;
  CK(h, launch_gradient_enforce(h, 0));
  return FLIPGPU_OK;
}

/* solve_picflip; with blend false the FLIP blend is left to the caller
 * (step_body fuses it with the advection) */
static int picflip(FlipGpu *h, FlipGpuSolveStats *st, StageClock *clk, bool blend = true) {
  StageClock none(h);
  if (!clk) clk = &none;
  clk->mark(FLIPGPU_STAGE_MARK);
  CK(h, launch_mark_water(h));
  clk->mark(FLIPGPU_STAGE_P2G);
  CK(h, launch_p2g(h, 1));
  clk->mark(FLIPGPU_STAGE_DIV);
  CK(h, launch_divergence(h));
  clk->mark(FLIPGPU_STAGE_SOLVE);
  int r = run_solve(h, st);
  if (r != FLIPGPU_OK) return r;
  clk->mark(FLIPGPU_STAGE_GRAD);
  CK(h, launch_gradient_enforce(h, 1));
  clk->mark(FLIPGPU_STAGE_EXTRAP);
  CK(h, launch_extrapolate_delta(h));
  if (blend) {
    clk->mark(FLIPGPU_STAGE_FLIP);
    CK(h, launch_flip_blend(h));
  }
  return FLIPGPU_OK;
}

int flipgpu_picflip(FlipGpu *h, FlipGpuSolveStats *st) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->cells_valid) CK(h, launch_sort(h, 0));
  int r = picflip(h, st, nullptr);
  if (r == FLIPGPU_OK && h->cells_valid) CK(h, launch_payload(h, 0));
  return r;
}

int flipgpu_advect(FlipGpu *h, int *stuck) {
  if (!h) return FLIPGPU_EINVAL;
  CK(h, cudaMemsetAsync(h->iflags + IF_NSTUCK, 0, 2 * sizeof(int), h->stream));
  CK(h, launch_advect(h));
  CK(h, launch_reposition(h, stuck));
  return FLIPGPU_OK;
}

int flipgpu_correct(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  CK(h, launch_sort(h, 0)); /* src/corrector.cpp:52 */
  CK(h, launch_correct(h));
  h->cells_valid = false;
  return FLIPGPU_OK;
}

static __global__ void k_step_inc(int64_t *dstep) { *dstep += 1; }

/* simulateStep (src/flip3D.cpp:1194-1264) minus the preview, pouring and
 * file output. With async_mode set nothing in it waits for the device, so it
 * can be recorded into a CUDA graph. */
static int step_body(FlipGpu *h, FlipGpuSolveStats *st) {
  h->step++;
  k_step_inc<<<1, 1, 0, h->stream>>>(h->dstep);
  FG_LAUNCHED(h, 1);
  StageClock clk(h);
  /* sort + add_ExtForce fused into the payload, then computeDensity */
  clk.mark(FLIPGPU_STAGE_SORT);
  CK(h, launch_sort(h, 1, PL_SPG | PL_SVEL)); /* the density stage writes sdens */
  clk.mark(FLIPGPU_STAGE_DENSITY);
  CK(h, launch_density(h));
  if (h->defer_vel) {
    /* flipgpu_step_host: the velocities have arrived on the transfer stream */
    CK(h, cudaStreamWaitEvent(h->stream, h->xev[1], 0));
    h->defer_vel = 0;
    CK(h, launch_payload_vel(h, h->defer_gravity));
  }
  int r = picflip(h, st, &clk, false);
  if (r != FLIPGPU_OK) return r;
  /* the FLIP blend and advect_particle in one kernel (both sample the new
   * grid at the old positions), then reposition, whose closing sort serves
   * the corrector (its own sort would see the same positions) */
  clk.mark(FLIPGPU_STAGE_FLIP);
  CK(h, cudaMemsetAsync(h->iflags + IF_NSTUCK, 0, 2 * sizeof(int), h->stream));
  CK(h, launch_flip_advect(h));
  clk.mark(FLIPGPU_STAGE_ADVECT);
  clk.mark(FLIPGPU_STAGE_REPOSITION);
  CK(h, launch_reposition(h, nullptr, true));
  clk.mark(FLIPGPU_STAGE_CORRECT);
  CK(h, launch_correct(h));
  clk.mark(FLIPGPU_NSTAGES);
  clk.flush();
  h->cells_valid = false;
  return FLIPGPU_OK;
}

int flipgpu_step(FlipGpu *h, FlipGpuSolveStats *st) {
  if (!h) return FLIPGPU_EINVAL;
  return step_body(h, st);
}

/* the transfer stream and its events, on first use. The stream has the
 * device's highest priority: its (de)interleave kernels are dispatched
 * ahead of the blocks the step's kernels still have queued, so the copies
 * start at once instead of after the concurrent kernel drains. */
static int xfer_init(FlipGpu *h) {
  if (h->xstream) return FLIPGPU_OK;
  int least = 0, greatest = 0;
  CK(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CK(h, cudaStreamCreateWithPriority(&h->xstream, cudaStreamNonBlocking, greatest));
  for (int e = 0; e < 3; e++) CK(h, cudaEventCreateWithFlags(&h->xev[e], cudaEventDisableTiming));
  return FLIPGPU_OK;
}

int flipgpu_step_host(FlipGpu *h, const float *pos_in, const float *vel_in, float *pos_out,
                      float *vel_out, FlipGpuSolveStats *st) {
  if (!h) return FLIPGPU_EINVAL;
  int r = xfer_init(h);
  if (r != FLIPGPU_OK) return r;
  /* positions in on the step's stream (staged through the sorted-position
   * buffer, as flipgpu_put_state does) */
  if ((r = put3(h, pos_in, 0, h->px, h->py, h->pz)) != FLIPGPU_OK) return r;
  /* velocities in on the transfer stream, staged through the sorted-velocity
   * buffer, which the step does not touch before the deferred payload */
  if (vel_in && h->np > 0) {
    CK(h, cudaEventRecord(h->xev[0], h->stream));
    CK(h, cudaStreamWaitEvent(h->xstream, h->xev[0], 0));
    float *stage = reinterpret_cast<float *>(h->svel);
    CK(h, cudaMemcpyAsync(stage, vel_in, (size_t)h->np * 3 * sizeof(float),
                          cudaMemcpyHostToDevice, h->xstream));
    k_deinterleave<<<grid_for(h->np, BLK), BLK, 0, h->xstream>>>(h->np, stage, h->vx, h->vy,
                                                                 h->vz);
    FG_LAUNCHED(h, 1);
    CK(h, cudaGetLastError());
    CK(h, cudaEventRecord(h->xev[1], h->xstream));
    h->defer_vel = 1;
  }
  h->cells_valid = false;
  h->xfer_pos_out = h->np > 0 ? pos_out : nullptr;
  r = step_body(h, st);
  h->xfer_pos_out = nullptr;
  if (h->defer_vel) { /* the step stopped before the payload */
    cudaStreamWaitEvent(h->stream, h->xev[1], 0);
    h->defer_vel = 0;
  }
  if (r == FLIPGPU_OK && vel_out)
    r = get3(h, vel_out, 0, h->vx, h->vy, h->vz, reinterpret_cast<float *>(h->spos));
  /* join the transfer stream before returning */
  CK(h, cudaEventRecord(h->xev[2], h->xstream));
  CK(h, cudaStreamWaitEvent(h->stream, h->xev[2], 0));
  CK(h, cudaStreamSynchronize(h->stream));
  return r;
}

static int async_ok(FlipGpu *h) {
  if (h->prm.solve_mode != FLIPGPU_SOLVE_FAST)
    return fail(h, FLIPGPU_EINVAL, "asynchronous steps need the FAST solver");
  if (h->warm) return fail(h, FLIPGPU_EINVAL, "asynchronous steps run without a warm start");
  if (h->prof_on) return fail(h, FLIPGPU_EINVAL, "asynchronous steps run without profiling");
  return FLIPGPU_OK;
}

int flipgpu_step_async(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  int r = async_ok(h);
  if (r != FLIPGPU_OK) return r;
  h->async_mode = 1;
  r = step_body(h, nullptr);
  h->async_mode = 0;
  return r;
}

int flipgpu_capture_step(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  int r = async_ok(h);
  if (r != FLIPGPU_OK) return r;
  if (h->graph_exec) {
    cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
  }
  if (h->graph) {
    cudaGraphDestroy(h->graph);
    h->graph = nullptr;
  }
  CK(h, cudaStreamSynchronize(h->stream));
  const int64_t step0 = h->step, launches0 = h->launches;
  CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
  h->async_mode = 1;
  r = step_body(h, nullptr);
  h->async_mode = 0;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->step = step0; /* recording ran nothing */
  h->graph_launches = h->launches - launches0;
  h->launches = launches0;
  if (r != FLIPGPU_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail(h, FLIPGPU_ECUDA, "capture_step: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph_exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(h, FLIPGPU_ECUDA, "capture_step: instantiate: %s", cudaGetErrorString(e));
  }
  h->graph = g;
  return FLIPGPU_OK;
}

int flipgpu_step_graph(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  if (!h->graph_exec) return fail(h, FLIPGPU_EINVAL, "step_graph: no captured step");
  h->step++;
  h->launches += h->graph_launches;
  CK(h, cudaGraphLaunch(h->graph_exec, h->stream));
  h->cells_valid = false;
  return FLIPGPU_OK;
}

int flipgpu_last_solve_stats(FlipGpu *h, FlipGpuSolveStats *st) {
  if (!h || !st) return FLIPGPU_EINVAL;
  return read_solve_stats(h, st);
}

/* ----------------------------------------------------------------- batches */

struct FlipBatch {
  std::vector<FlipGpu *> sims;
  bool graphs = false;
};

int flipbatch_create(FlipBatch **out) {
  if (!out) return FLIPGPU_EINVAL;
  *out = new (std::nothrow) FlipBatch();
  return *out ? FLIPGPU_OK : FLIPGPU_ENOMEM;
}

int flipbatch_destroy(FlipBatch *b) {
  if (!b) return FLIPGPU_EINVAL;
  delete b;
  return FLIPGPU_OK;
}

int flipbatch_add(FlipBatch *b, FlipGpu *h) {
  if (!b || !h) return FLIPGPU_EINVAL;
  b->sims.push_back(h);
  return FLIPGPU_OK;
}

int flipbatch_capture(FlipBatch *b) {
  if (!b) return FLIPGPU_EINVAL;
  for (FlipGpu *h : b->sims) {
    int r = flipgpu_capture_step(h);
    if (r != FLIPGPU_OK) return r;
  }
  b->graphs = true;
  return FLIPGPU_OK;
}

int flipbatch_step(FlipBatch *b) {
  if (!b) return FLIPGPU_EINVAL;
  for (FlipGpu *h : b->sims) {
    int r = b->graphs ? flipgpu_step_graph(h) : flipgpu_step_async(h);
    if (r != FLIPGPU_OK) return r;
  }
  return FLIPGPU_OK;
}

int flipbatch_sync(FlipBatch *b) {
  if (!b) return FLIPGPU_EINVAL;
  for (FlipGpu *h : b->sims) CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_set_solve_blocks(FlipGpu *h, int blocks) {
  if (!h || blocks < 0) return FLIPGPU_EINVAL;
  h->solve_blocks = blocks;
  return FLIPGPU_OK;
}

int flipgpu_get_solve_blocks(const FlipGpu *h, int *blocks) {
  if (!h || !blocks) return FLIPGPU_EINVAL;
  *blocks = h->solve_blocks;
  return FLIPGPU_OK;
}

/* Member i's persistent solve gets max(1, share * C_i * cells_i / cells of
 * all members) blocks, C_i its solve kernel's co-resident grid: at share 1
 * the members' solves fit on the GPU side by side. share <= 0 lifts the
 * caps. Members without a persistent solve (the IC wavefront, no
 * preconditioner) keep none. */
static void batch_share(FlipBatch *b, double share) {
  double cells = 0.0;
  for (FlipGpu *h : b->sims) cells += (double)h->nc;
  for (FlipGpu *h : b->sims) {
    if (share <= 0.0 || h->solve_capacity <= 0) {
      h->solve_blocks = 0;
      continue;
    }
    const double v = share * h->solve_capacity * (double)h->nc / cells;
    h->solve_blocks = v < 1.0 ? 1 : (int)std::lround(v);
  }
}

/* The tuner's trial: every member solves its current system (the one its
 * last step solved) on its own stream, all at once, from the saved warm
 * start. Returns the span in ms, or < 0 on a CUDA error. */
static float batch_solve_trial(FlipBatch *b, cudaStream_t root, cudaEvent_t t0, cudaEvent_t t1,
                               const std::vector<cudaEvent_t> &done,
                               const std::vector<float *> &saved) {
  for (size_t m = 0; m < b->sims.size(); m++) {
    FlipGpu *h = b->sims[m];
    const size_t bytes = (size_t)h->nc * sizeof(float);
    if (cudaMemcpyAsync(h->press, saved[m], bytes, cudaMemcpyDeviceToDevice, h->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(h->press_lo, saved[m] + h->nc, bytes, cudaMemcpyDeviceToDevice,
                        h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      return -1.0f;
  }
  if (cudaEventRecord(t0, root) != cudaSuccess) return -1.0f;
  for (size_t m = 0; m < b->sims.size(); m++) {
    FlipGpu *h = b->sims[m];
    if (cudaStreamWaitEvent(h->stream, t0, 0) != cudaSuccess) return -1.0f;
    h->async_mode = 1;
    const int r = run_solve(h, nullptr);
    h->async_mode = 0;
    if (r != FLIPGPU_OK || cudaEventRecord(done[m], h->stream) != cudaSuccess ||
        cudaStreamWaitEvent(root, done[m], 0) != cudaSuccess)
      return -1.0f;
  }
  float ms = -1.0f;
  if (cudaEventRecord(t1, root) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
      cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess)
    return -1.0f;
  return ms;
}

int flipbatch_tune(FlipBatch *b, double *share_out) {
  if (!b) return FLIPGPU_EINVAL;
  if (share_out) *share_out = 0.0;
  bool any = false;
  for (FlipGpu *h : b->sims) {
    if (h->step == 0)
      return fail(h, FLIPGPU_EINVAL, "batch_tune: step the batch once before tuning it");
    any = any || h->solve_capacity > 0;
  }
  if (!any) return FLIPGPU_OK;
  for (FlipGpu *h : b->sims) CK(h, cudaStreamSynchronize(h->stream));
  FlipGpu *h0 = b->sims[0];
  const double shares[] = {0.0, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0};
  const int ns = (int)(sizeof shares / sizeof shares[0]);
  std::vector<std::string> names;
  for (int c = 0; c < ns; c++) {
    char nm[32];
    snprintf(nm, sizeof nm, c == 0 ? "uncapped" : "share %.1f", shares[c]);
    names.push_back(nm);
  }
  std::vector<float> ms(ns, -1.0f);
  std::vector<float *> saved(b->sims.size(), nullptr);
  std::vector<int> lo_valid(b->sims.size(), 0);
  std::vector<cudaEvent_t> done(b->sims.size(), nullptr);
  cudaStream_t root = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  int rc = FLIPGPU_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&root, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  for (size_t m = 0; e == cudaSuccess && m < b->sims.size(); m++) {
    FlipGpu *h = b->sims[m];
    e = cudaEventCreateWithFlags(&done[m], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&saved[m], 2 * (size_t)h->nc * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMemcpy(saved[m], h->press, (size_t)h->nc * sizeof(float), cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(saved[m] + h->nc, h->press_lo, (size_t)h->nc * sizeof(float),
                     cudaMemcpyDeviceToDevice);
    lo_valid[m] = h->press_lo_valid;
  }
  if (e != cudaSuccess) rc = fail(h0, FLIPGPU_ECUDA, "batch_tune: setup: %s", cudaGetErrorString(e));
  /* one warm-up trial per candidate, then the median of three */
  for (int c = 0; rc == FLIPGPU_OK && c < ns; c++) {
    batch_share(b, shares[c]);
    float t[4];
    for (int r = 0; r < 4 && rc == FLIPGPU_OK; r++) {
      t[r] = batch_solve_trial(b, root, t0, t1, done, saved);
      if (t[r] < 0.0f) rc = fail(h0, FLIPGPU_ECUDA, "batch_tune: trial solve failed");
    }
    if (rc != FLIPGPU_OK) break;
    std::sort(t + 1, t + 4);
    ms[c] = t[2];
  }
  int best = 0;
  for (int c = 1; c < ns; c++)
    if (ms[c] >= 0.0f && (ms[best] < 0.0f || ms[c] < ms[best])) best = c;
  batch_share(b, rc == FLIPGPU_OK ? shares[best] : 0.0);
  /* the members' pressure as their last step left it */
  for (size_t m = 0; m < b->sims.size(); m++) {
    FlipGpu *h = b->sims[m];
    if (saved[m]) {
      const size_t bytes = (size_t)h->nc * sizeof(float);
      cudaError_t e2 = cudaMemcpy(h->press, saved[m], bytes, cudaMemcpyDeviceToDevice);
      if (e2 == cudaSuccess)
        e2 = cudaMemcpy(h->press_lo, saved[m] + h->nc, bytes, cudaMemcpyDeviceToDevice);
      if (e2 != cudaSuccess && rc == FLIPGPU_OK)
        rc = fail(h, FLIPGPU_ECUDA, "batch_tune: restore: %s", cudaGetErrorString(e2));
      cudaFree(saved[m]);
    }
    h->press_lo_valid = lo_valid[m];
    if (done[m]) cudaEventDestroy(done[m]);
  }
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  if (root) cudaStreamDestroy(root);
  if (rc != FLIPGPU_OK) return rc;
  char key[96];
  double cells = 0.0;
  for (FlipGpu *h : b->sims) cells += (double)h->nc;
  snprintf(key, sizeof key, "batch solve share (%zu simulations, %.0f cells)", b->sims.size(),
           cells);
  autotune::record(key, names, ms, best);
  if (share_out) *share_out = shares[best];
  /* the captured steps hold the old grids */
  if (b->graphs) return flipbatch_capture(b);
  return FLIPGPU_OK;
}

int flipgpu_put_state(FlipGpu *h, const float *pos, const float *vel, int on_device) {
  if (!h) return FLIPGPU_EINVAL;
  int r;
  if ((r = put3(h, pos, on_device, h->px, h->py, h->pz)) != FLIPGPU_OK) return r;
  if ((r = put3(h, vel, on_device, h->vx, h->vy, h->vz)) != FLIPGPU_OK) return r;
  h->cells_valid = false;
  return FLIPGPU_OK;
}

int flipgpu_set_profiling(FlipGpu *h, int on) {
  if (!h) return FLIPGPU_EINVAL;
  ktime_flush(h);
  h->prof_on = on;
  for (int i = 0; i < FLIPGPU_NSTAGES; i++) {
    h->prof_ms[i] = 0.0;
    h->prof_calls[i] = 0;
  }
  h->kt_nnames = 0;
  return FLIPGPU_OK;
}

int flipgpu_get_kernel_profile(FlipGpu *h, char *buf, int len) {
  if (!h || len < 0) return FLIPGPU_EINVAL;
  ktime_flush(h);
  std::string s;
  char line[160];
  for (int k = 0; k < h->kt_nnames; k++) {
    snprintf(line, sizeof line, "%s\t%.6f\t%lld\n", h->kt_name[k], h->kt_ms[k],
             (long long)h->kt_calls[k]);
    s += line;
  }
  if (buf && len > 0) {
    strncpy(buf, s.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)s.size();
}

int flipgpu_set_ic_tag_counter(FlipGpu *h, unsigned value) {
  if (!h) return FLIPGPU_EINVAL;
  int r = ic_alloc(h);
  if (r != FLIPGPU_OK) return fail(h, r, "set_ic_tag_counter: wavefront buffers");
  CK(h, cudaMemcpyAsync(h->ic_ctr, &value, sizeof value, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_get_ic_tag_counter(FlipGpu *h, unsigned *value) {
  if (!h || !value) return FLIPGPU_EINVAL;
  int r = ic_alloc(h);
  if (r != FLIPGPU_OK) return fail(h, r, "get_ic_tag_counter: wavefront buffers");
  CK(h, cudaMemcpyAsync(value, h->ic_ctr, sizeof *value, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return FLIPGPU_OK;
}

int flipgpu_get_profile(FlipGpu *h, double *ms, int64_t *calls, int max) {
  if (!h || max < 0) return FLIPGPU_EINVAL;
  for (int i = 0; i < FLIPGPU_NSTAGES && i < max; i++) {
    if (ms) ms[i] = h->prof_ms[i];
    if (calls) calls[i] = h->prof_calls[i];
  }
  return FLIPGPU_OK;
}

} // extern "C"
