/*
 * flipgpu_impl.h — device-resident state of one simulation and the kernel
 * launchers shared by the translation units of libflipgpu.so.
 *
 * Particle data lives twice:
 *   canonical  SoA in the caller's particle order (px..vz, dens, type, nrm):
 *              per-particle stages read and write it coalesced;
 *   sorted     a copy grouped by cell (spos/spg/svel/sdens, index = slot of
 *              the cell lists): gather stages read neighbours as contiguous
 *              runs, k-adjacent cells being adjacent in memory.
 */
#ifndef FLIPGPU_IMPL_H
#define FLIPGPU_IMPL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/flipgpu.h"

enum { CELL_AIR = 0, CELL_FLUID = 1, CELL_WALL = 2 };

struct MeshBufs; /* mesher buffers (k_mesh.cu) */

/* Per-run constants handed to kernels by value. */
struct SimConst {
  int n;              /* grid cells per axis */
  int np;             /* particle count */
  float fn;           /* (float)n */
  float h;            /* (float)(1.0/n): cell width (src/flip3D.cpp:809) */
  float density;      /* DENSITY */
  float kd_hh;        /* density kernel radius^2: h*h of (float)(4*DENSITY/N) */
  float kd_rcp;       /* 1/kd_hh when kd_hh is a power of two, else 0 */
  float corr_rcp;     /* 1/re_corr_hh when it is a power of two, else 0 */
  float kd_inv, corr_inv; /* 1/kd_hh, 1/re_corr_hh in float (FAST arithmetic) */
  float max_dens;
  float re_p2g_hh;    /* RE*RE for P2G (src/mapper.cpp:14) */
  float re_corr;      /* DENSITY/N (src/flip3D.cpp:1242) */
  float re_corr_hh;
  float re_repo;      /* 1.0/gn: resample radius in reposition (src/flip3D.cpp:435) */
  float re_repo_hh;
  float r2_floor;     /* smallest float above 1e-5 (sharp kernel clamp) */
  float sharp_small_p2g, sharp_small_corr, sharp_small_repo;
  float wall_r;       /* (float)WALL_THICK */
  float wall_hi;      /* (float)(1.0 - WALL_THICK) */
  float wall_hi_thr;  /* largest float <= 1.0 - WALL_THICK */
  double push_re;     /* 1.5*DENSITY/N (src/flip3D.cpp:909) */
  float push_re_thr;  /* largest float < push_re */
  float corr_near_thr;/* largest float <= 0.1*re (src/corrector.cpp:68) */
  float corr_cut2;    /* squared distance beyond which the spring weight is 0 */
  float corr_reach;   /* re*(1+2^-8): cell-range reach of the corrector */
  float dt_f;         /* (float)DT, the corrector's dt */
  double kick_fluid;  /* 0.01*re/dt (src/corrector.cpp:75) */
  double kick_wall;   /* 0.05*re/dt (src/corrector.cpp:80) */
  double dt;
  float dt_h, dt_l;   /* DT split into floats */
  double grav;        /* -DT*GRAVITY */
  float grav_h, grav_l;
  double c1, c2;      /* 1-ALPHA, ALPHA */
  float c1h, c1l, c2h, c2l;
  double l0;          /* 0.2 * n0 of sorter::levelset */
  float l0h, l0l;
  uint64_t seed;
  int64_t step;
  const int64_t *dstep; /* the step counter in device memory (graph replays advance it) */
};

constexpr int CG_VARIANTS = 6; /* persistent CG kernels (k_pcg.cu cg_grid_size) */

struct FlipGpu {
  FlipGpuParams prm;
  int n;
  int np;
  int cap;
  size_t nc;          /* n^3 */
  size_t nf;          /* (n+1)*n*n faces per component */
  cudaStream_t stream;
  cudaStream_t own_stream;
  float max_dens;
  int64_t step;
  int64_t *dstep;     /* device copy of step, advanced by a kernel each step */
  int async_mode;     /* the step being recorded or run needs no host sync */
  cudaGraph_t graph;
  cudaGraphExec_t graph_exec;
  int64_t graph_launches; /* kernels in the captured step */
  int64_t launches;
  char err[512];

  /* canonical particles */
  float *px, *py, *pz, *vx, *vy, *vz, *dens;
  uint8_t *type;
  float *nx, *ny, *nz;

  /* cell lists */
  uint32_t *key, *rank, *perm, *cell_start, *cell_count;
  uint32_t *cell_mid; /* FAST arithmetic: first slot of each cell's upper z half
                         (k_sort.cu k_sort_fixup_halves) */
  float4 *spos;       /* world position, w = type */
  float4 *spg;        /* clamp(n*pos, 0, n), w = type (P2G) */
  float4 *svel;       /* velocity, w unused */
  float *sdens;
  bool cells_valid;   /* lists match the current positions */
  bool lists_exist;   /* some sort has run (lists of the last sort) */

  /* static wall lists (walls never move) */
  int nwall;
  uint32_t *wall_start;
  float4 *wall_pos;   /* w = unused */
  float4 *wall_nrm;

  /* grid */
  float *u[3], *us[3];
  uint8_t *A;
  float *L, *press, *div;

  /* solver */
  float *r, *z, *s, *s1, *w;
  /* mixed-precision refinement (FAST mode): the iterate is press + press_lo
   * (a double-float pair), ir_b the right-hand side and ir_e the correction
   * of the current inner FP32 solve */
  float *press_lo, *ir_b, *ir_e;
  int press_lo_valid; /* press_lo belongs to the current press (last solve refined) */
  float *w1, *pdir;   /* single-reduction CG: second w buffer, directions */
  /* flipgpu_step_host: transfers overlapped with the step on a second stream */
  cudaStream_t xstream;
  cudaEvent_t xev[3];
  int defer_vel, defer_gravity;   /* payload velocities after the upload */
  float *xfer_pos_out;            /* host destination of the positions, or null */
  /* MG preconditioner (k_pcg.cu mg_alloc): levels 1.. and level-0 scratch */
  int mg_nlev, mg_lb, mg_m[10];
  uint8_t *mg_flags[10];
  float *mg_diag[10], *mg_x[10], *mg_b[10], *mg_res[10];
  float *mg_p2, *mg_q;
  unsigned *chunk_off;  /* single-reduction CG: liquid flags of the 32-quad chunks, scanned */
  unsigned *chunk_list; /* ... and the indices of the chunks that hold liquid */
  double *P;          /* REF preconditioner diagonal (double, as the reference) */
  float *Pf;          /* FP32 preconditioner diagonal / IC factor */
  float *diag;        /* FP32 matvec diagonal (FAST mode) */
  double *partial;    /* per-block reduction partials */
  double *scal;       /* device scalars of the CG recurrence */
  int *iflags;        /* device flags/counters */
  unsigned *bar;      /* grid barrier of the persistent CG: count, generation */
  int cg_grid[CG_VARIANTS]; /* cooperative CG grids (0 = none): REF, FAST, FAST single-
                               reduction (small blocks), FAST IC, single-reduction (large),
                               FAST MG */
  int solve_blocks;   /* cap on the persistent solve's grid (0 = none; not the IC
                         wavefront), so that concurrent simulations' solves share the GPU */
  int solve_capacity; /* co-resident grid of the last solve's kernel */
  unsigned *ticket;   /* task ticket of the IC wavefront */
  /* IC(0)/MIC(0) line wavefront (k_pcg.cu ic_alloc) */
  int ic_njb, ic_tasks;              /* 32-j line blocks; tasks */
  unsigned *ic_order, *ic_line;      /* tasks in wavefront order; lines holding liquid */
  uint8_t *ic_cf;                    /* per cell: liquid flag, MIC(0) counts */
  float *ic_pf;                      /* skewed factor */
  unsigned long long *ic_psk, *ic_qsk, *ic_zsk; /* skewed tagged factor, q, z */
  float2 *ic_part;                   /* per-task q.q partials */
  unsigned *ic_ctr;                  /* tag counter of the word handoff */
  int npartial;

  /* reposition */
  uint8_t *flag;      /* per particle / per cell */
  uint32_t *scan_a, *scan_b, *scan_tmp;
  uint32_t *stuck_idx, *water_idx;
  uint32_t *repo_draw;       /* per stuck particle: shuffle draw */
  uint32_t *repo_cnt, *repo_start, *repo_list; /* shuffle steps listed by position */
  float4 *repo_res, *repo_old; /* per stuck particle: resampled / previous velocity */
  uint8_t *repo_state;       /* per stuck particle: resample round state */
  size_t scan_cap;

  float *stage;       /* AoS staging for downloads */
  MeshBufs *mesh;     /* mesher buffers, allocated by the first mesh call */
  struct ExportJob *exportjob; /* the mesh export in flight (export.cu) */

  /* learned warm start (k_unet.cu) */
  FlipUNet *warm;     /* network, or null for the previous-step guess */
  float *wdelta;      /* correction, A*correction, A*x0 (3 n^3) */
  double *wpart;
  cudaEvent_t wev[2];
  /* capture of the last solve's system for training data */
  int capture;
  float *cap_b, *cap_x0, *cap_r0;
  cudaEvent_t ev0, ev1;

  /* per-stage profiling */
  int prof_on;
  cudaEvent_t prof_ev[FLIPGPU_NSTAGES + 1];
  double prof_ms[FLIPGPU_NSTAGES];
  int64_t prof_calls[FLIPGPU_NSTAGES];
  /* per-kernel profiling of the main kernels (ktime_*): event pairs of the
   * launches not yet read, and the totals per kernel name */
  static constexpr int KT_SLOTS = 64, KT_NAMES = 24;
  cudaEvent_t kt_ev[2 * KT_SLOTS];
  const char *kt_pending[KT_SLOTS];
  int kt_n, kt_ready;
  const char *kt_name[KT_NAMES];
  double kt_ms[KT_NAMES];
  int64_t kt_calls[KT_NAMES];
  int kt_nnames;
};

/* Per-kernel clock of the profiling mode: events on the handle's stream
 * before and after one launch of the named kernel (a string literal);
 * ktime_flush waits for them and adds each launch's time to its kernel's
 * total. Does nothing unless profiling is on. */
void ktime_begin(FlipGpu *h, const char *name);
void ktime_end(FlipGpu *h);
void ktime_flush(FlipGpu *h);

/* Device scalar slots (FlipGpu::scal). */
enum {
  SC_A = 0,      /* z.r of the previous iteration */
  SC_ALPHA,
  SC_BETA,
  SC_ERR2,       /* float(r.r) */
  SC_EPS,
  SC_B2,
  SC_DOT,        /* scratch result of the last dot */
  SC_ERR2_0,
  SC_TRUE2,      /* FP64 r.r of b - A x after a FAST solve */
  SC_IR_B2,      /* refinement: b.b of the outer system */
  SC_IR_TOL,     /* refinement: relative tolerance of the next inner solve */
  SC_IR_PREV,    /* refinement: true r.r before the last inner solve */
  SC_COUNT
};
/* Device int slots (FlipGpu::iflags). */
enum {
  IF_DONE = 0,   /* CG converged */
  IF_ITERS,      /* iterations taken */
  IF_EXOTIC,     /* REF preconditioner has a diagonal entry equal to 1.0 */
  IF_NSTUCK,
  IF_NWATER,
  IF_NAN,
  IF_TIMEOUT,
  IF_REPO_LEFT,
  IF_IR_DONE,    /* refinement: 0 running, 1 converged, 2 non-finite, 3 no
                    convergence, 4 zero right-hand side (x = 0) */
  IF_IR_ITERS,   /* refinement: inner CG iterations of all passes */
  IF_IR_PASS,    /* refinement: inner solves run */
  IF_COUNT
};

SimConst make_const(const FlipGpu *h);

/* launchers (one per reference stage or sub-stage); return cudaError_t */
/* Sorted copies written by the sort's payload besides spos. A step leaves
 * out what it rewrites before reading (sdens: the density stage) or never
 * reads (after the reposition's sort: spg, sdens, and svel, which the
 * reposition refreshes); the lists then stop being valid at the step's
 * end, so later calls sort again. */
enum { PL_SPG = 1, PL_SVEL = 2, PL_SDENS = 4, PL_ALL = 7 };
cudaError_t launch_sort(FlipGpu *h, int apply_gravity, int fields = PL_ALL);
cudaError_t launch_payload(FlipGpu *h, int apply_gravity, int fields = PL_ALL);
/* the velocity half of the payload: the deferred one (FlipGpu::defer_vel)
 * or a refresh of the sorted velocities */
cudaError_t launch_payload_vel(FlipGpu *h, int apply_gravity);
/* flipgpu_step_host: download the corrected positions on the transfer
 * stream while the velocity resample runs (called between the two) */
cudaError_t xfer_positions_out(FlipGpu *h);
cudaError_t launch_density(FlipGpu *h);
cudaError_t launch_mark_water(FlipGpu *h);
cudaError_t launch_add_force(FlipGpu *h);
cudaError_t launch_p2g(FlipGpu *h, int enforce);
cudaError_t launch_g2p(FlipGpu *h);
cudaError_t launch_divergence(FlipGpu *h);
cudaError_t launch_gradient_enforce(FlipGpu *h, int enforce);
cudaError_t launch_extrapolate_delta(FlipGpu *h);
cudaError_t launch_flip_blend(FlipGpu *h);
cudaError_t launch_advect(FlipGpu *h);
/* launch_flip_blend + launch_advect in one kernel (one grid sample) */
cudaError_t launch_flip_advect(FlipGpu *h);
/* in_step: the step's own reposition, whose sort writes only spos (see
 * PL_*) */
cudaError_t launch_reposition(FlipGpu *h, int *stuck_host, bool in_step = false);
cudaError_t launch_correct(FlipGpu *h);
cudaError_t launch_fetch_points(FlipGpu *h, int count, const float *pts, float *out);
cudaError_t launch_resample_points(FlipGpu *h, int count, const float *pts, float *vel,
                                   float re);
int run_solve(FlipGpu *h, FlipGpuSolveStats *st);
/* out[c] = press + press_lo (the refined iterate) as double, device memory */
void launch_pressure_double(FlipGpu *h, double *out);
/* stats of the last solve read from the device (for steps run without a
 * host sync) */
int mesh_download_async(FlipGpu *h, double *vertices, double *normals, int32_t *faces,
                        int64_t *nv, int64_t *nf);
/* the asynchronous mesh export of export.cu: join and free */
int export_join(FlipGpu *h);
void export_free(FlipGpu *h);
int read_solve_stats(FlipGpu *h, FlipGpuSolveStats *st);
int cg_grid_size(int *out);
int mg_alloc(FlipGpu *h);  /* MG preconditioner buffers (idempotent) */
void mg_free(FlipGpu *h);
int ic_alloc(FlipGpu *h);
void ic_free(FlipGpu *h);
int particles_init_device();

/* device-wide exclusive scan of n uint32 (in may equal out) */
cudaError_t scan_exclusive(FlipGpu *h, const uint32_t *in, uint32_t *out,
                           size_t n);
/* the same with caller scratch of tmp_blocks entries (scan_tmp_blocks(n)) */
cudaError_t scan_exclusive_tmp(FlipGpu *h, const uint32_t *in, uint32_t *out, size_t n,
                               uint32_t *tmp, size_t tmp_blocks);
size_t scan_tmp_blocks(size_t n);
/* the same over the first *nlive + 1 entries only (a count on the device) */
cudaError_t scan_exclusive_live(FlipGpu *h, const uint32_t *in, uint32_t *out, size_t n,
                                const int *nlive);
/* ordered compactions: idx = ascending indices of the set particle flags /
 * of the deep-water cells, *count their number (device) */
cudaError_t compact_flags(FlipGpu *h, const uint8_t *flag, size_t n, uint32_t *idx, int *count);
cudaError_t compact_deep_water(FlipGpu *h, uint32_t *idx, int *count);

/* learned warm start (k_unet.cu): x0 += g*d before CG; out3 = {r0.r0 of
 * the previous-step guess, of the new guess, g} */
int warm_start_apply(FlipGpu *h, float inv_h2_f, double *out3, float *ms);
/* r = b - A x with the FAST-mode matrix (diag set by the solver's setup) */
cudaError_t launch_residual(FlipGpu *h, float inv_h2_f, const float *x, float *r);

/* mesher (k_mesh.cu) */
int mesh_run(FlipGpu *h, int64_t *nverts, int64_t *nfaces);
int mesh_get(FlipGpu *h, double *vertices, double *normals, int32_t *faces, float *phi);
cudaError_t launch_implicit_points(FlipGpu *h, int count, const float *pts, double *out);
void mesh_free(FlipGpu *h);

/* kernel-count bookkeeping */
#define FG_LAUNCHED(h, k) ((h)->launches += (k))

static inline unsigned grid_for(size_t n, int block) {
  return (unsigned)((n + block - 1) / block);
}

#endif
