/*
 * flipgpu.h — C ABI of the GB300 FLIP step (libflipgpu.so).
 *
 * One opaque handle holds one simulation resident in device memory: the
 * particle set (structure of arrays, in the caller's particle order), the
 * sorted cell lists, the MAC grid and the solver vectors. Each entry point
 * below replaces one function of the reference's per-step hot path and runs
 * on the handle's CUDA stream; none synchronises with the host unless it
 * returns data to host memory.
 *
 * Layouts (identical to the CPU oracle and the reference's arrays):
 *   particles   pos/vel/nrm float[count][3], type uint8 (1 fluid, 2 wall)
 *   cells       x-major (i*n + j)*n + k, k fastest (the reference's
 *               A[i][j][k] with k contiguous)
 *   faces       u0 (n+1)*n*n, u1 n*(n+1)*n, u2 n*n*(n+1), x-major
 *   cell lists  cell_start[n^3+1], perm[count]: the particles of cell c are
 *               perm[cell_start[c] .. cell_start[c+1]) in particle order,
 *               exactly the lists sorter::sort builds (FAST arithmetic lists
 *               the particles below the cell's mid-plane in z, (k + 0.5)/n,
 *               first, each half in particle order)
 *
 * Every call returns FLIPGPU_OK (0) or a negative FLIPGPU_E* code;
 * flipgpu_last_error() gives a message. Handles are not thread-safe, like
 * the reference's static state (src/flip3D.cpp:41-60).
 */
#ifndef FLIPGPU_H
#define FLIPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLIPGPU_OK 0
#define FLIPGPU_EINVAL -1      /* bad argument or size */
#define FLIPGPU_ECUDA -2       /* CUDA runtime error */
#define FLIPGPU_ENOMEM -3      /* device allocation failed */
#define FLIPGPU_ENOCONV -4     /* CG hit its iteration cap */
#define FLIPGPU_ENAN -5        /* non-finite residual */
#define FLIPGPU_ETIMEOUT -6    /* a bounded device wait expired */
#define FLIPGPU_ETOOBIG -7     /* input larger than a fixed scratch limit */

/* Preconditioners. REF reproduces the reference's buildPreconditioner/
 * applyPreconditioner as written (src/solver.cpp:119-180): its neighbour
 * terms only act on values equal to 1.0, so in practice it scales by the
 * diagonal. IC is the same lexicographic incomplete-Cholesky factor with the
 * neighbour test on the cell flag (mic_tau 0 = IC(0), 0.97 = MIC(0)),
 * applied as wavefronts. JACOBI is plain diagonal scaling in FP32. MG is
 * one symmetric geometric-multigrid V-cycle per iteration (red-black
 * Gauss-Seidel smoothing, coarse operators rediscretised on coarsened cell
 * flags); FAST mode with n % 4 == 0 and n >= 8 only. */
#define FLIPGPU_PRECOND_NONE 0
#define FLIPGPU_PRECOND_REF 1
#define FLIPGPU_PRECOND_IC 2
#define FLIPGPU_PRECOND_JACOBI 3
#define FLIPGPU_PRECOND_MG 4

/* Solver arithmetic. REF: the reference's promotions (double matvec sums,
 * float(r.r) stop test, power-of-4 relative tolerance, see rel_tol). FAST:
 * FP32 matvec and preconditioner, dot products with exact products summed
 * as double-float pairs (about 48 significant bits, fixed reduction order),
 * and mixed-precision iterative refinement on the true residual (see
 * refine_steps): stop on ||b - A x|| <= rel_tol*||b||. */
#define FLIPGPU_SOLVE_REF 0
#define FLIPGPU_SOLVE_FAST 1

/* Particle-gather arithmetic (density, P2G, FLIP blend, advection, the
 * corrector's spring and resample). REF: the reference's float expressions
 * and double promotions reproduced bit for bit (error-free transforms).
 * FAST: native FP32 with fused multiply-adds and the fast division
 * intrinsic; results agree with REF to FP32 rounding per step. FAST also
 * orders each cell's particles by z half (see the cell lists above), so a
 * sum over a cell runs in that order and the corrector's neighbour walk
 * starts and stops at half cells. The grid stages and the solver are
 * unaffected. */
#define FLIPGPU_ARITH_REF 0
#define FLIPGPU_ARITH_FAST 1

typedef struct FlipGpuParams {
  int n;              /* N: grid cells per axis (src/flip3D.cpp:25) */
  int max_particles;  /* capacity of the particle arrays */
  float density;      /* DENSITY 0.5: particle spacing in cells */
  double alpha;       /* ALPHA 0.95: FLIP fraction */
  double dt;          /* DT 0.006 */
  double gravity;     /* GRAVITY 9.8 */
  int subcell;        /* SUBCELL 1: ghost-fluid free surface */
  uint64_t seed;      /* seed of the keyed random draws */
  int solve_mode;     /* FLIPGPU_SOLVE_* */
  int precond;        /* FLIPGPU_PRECOND_* */
  double mic_tau;     /* IC modification weight */
  double rel_tol;     /* relative residual target; REF mode divides the
                         reference's absolute 1e-2*n^3 by 4^k until it is at
                         most rel_tol^2*b.b; 0 keeps the reference's own */
  double eps_abs;     /* REF mode: explicit absolute r.r bound if >= 0 */
  int max_iters;      /* CG iteration cap; <=0: n^3 like the reference
                         (1000 with the MG preconditioner) */
  int refine_steps;   /* FAST mode: mixed-precision iterative refinement with
                         at most refine_steps passes (default 4). The iterate
                         is a double-float pair (press holds its FP32
                         rounding; flipgpu_get_pressure returns the pair as
                         double); each pass evaluates the true residual
                         b - A x with error-free FP32 transforms (about 48
                         significant bits) and solves A e = r with the FP32
                         PCG to a loose tolerance; the solve stops when
                         ||b - A x|| <= rel_tol ||b|| and returns
                         FLIPGPU_ENOCONV if the passes run out or stall.
                         0: one FP32 PCG that stops on its recursive
                         residual; its true residual (stats r2_true) levels
                         off near the FP32 rounding of A x (about 1e-4 of
                         ||b|| at n=128). */
  int arith;          /* FLIPGPU_ARITH_*: particle-gather arithmetic */
  int mg_sweeps;      /* MG preconditioner: red-black Gauss-Seidel sweeps before
                         the coarse correction (mirrored after it) on every
                         level; <= 0: the library's default */
} FlipGpuParams;

typedef struct FlipGpuSolveStats {
  int iterations;     /* CG iterations of the last solve (all passes) */
  int status;         /* FLIPGPU_OK / ENOCONV / ENAN */
  double r2;          /* final r.r */
  double b2;          /* b.b */
  double ms;          /* device time of the solve (CUDA events), warm start included */
  int warm;           /* 1 when a learned warm start ran before CG */
  double r2_prev;     /* warm start: r.r of the previous-step guess */
  double r2_guess;    /* warm start: r.r of the guess CG started from */
  double gamma;       /* warm start: step taken along the network's correction */
  double warm_ms;     /* warm start: device time of network + step */
  double r2_true;     /* FAST mode: r.r of the true residual b - A x at the
                         end (the iterate of the refinement, or x in FP32
                         without it, whose recursive r2 is what CG's stop
                         test saw) */
  int refine_passes;  /* FAST mode with refinement: inner solves run; r2 is
                         then r2_true and iterations counts all passes */
} FlipGpuSolveStats;

typedef struct FlipUNet FlipUNet;

typedef struct FlipGpu FlipGpu;

/* Fill p with the reference's defaults for grid size n. */
void flipgpu_default_params(FlipGpuParams *p, int n, int max_particles);

int flipgpu_create(const FlipGpuParams *p, FlipGpu **out);
int flipgpu_destroy(FlipGpu *h);
const char *flipgpu_last_error(const FlipGpu *h);
/* Change the run parameters of a handle (everything except n and
 * max_particles, which must match). solver::setSubcell maps onto this. */
int flipgpu_set_params(FlipGpu *h, const FlipGpuParams *p);
/* Use an external stream (a cudaStream_t); NULL restores the handle's own. */
int flipgpu_set_stream(FlipGpu *h, void *stream);
int flipgpu_sync(FlipGpu *h);
int flipgpu_set_step(FlipGpu *h, int64_t step);

/* Particle state. Pointers are host memory unless on_device != 0. Any
 * pointer may be NULL to skip that array (set: keeps zeros/old values). */
/* A liquid object of a seeded scene: a lattice point belongs to the first
 * object containing it (pushParticle, src/flip3D.cpp:580-647). Boxes are
 * open intervals lo < p < hi; spheres |p - c| < r in float. */
#define FLIPGPU_SHAPE_BOX 0
#define FLIPGPU_SHAPE_SPHERE 1
typedef struct FlipSceneObject {
  int shape;          /* FLIPGPU_SHAPE_* */
  float lo[3], hi[3]; /* box corners */
  float c[3];         /* sphere centre */
  float r;            /* sphere radius */
  float vel[3];       /* initial velocity of the object's particles */
} FlipSceneObject;

/* flip3D::init's scene setup on the device (src/flip3D.cpp:649-777): a
 * lattice of spacing density cells in the interior, each point kept if it
 * lies in an object, jittered by +-jitter cell per axis with
 * flip_rand31(seed, FLIP_RNG_SEED stream, lattice index) and dropped if the
 * jitter moves it into a wall cell; then one wall particle per cell of the
 * outer layer with its face normal (compute_wall_normal,
 * src/flip3D.cpp:75-130) and the static wall lists. Replaces the particle
 * state; the particle order is liquid in lattice order, then walls in cell
 * order. At most 16 objects. */
int flipgpu_seed_scene(FlipGpu *h, const FlipSceneObject *objs, int nobj, uint64_t seed,
                       double density, double jitter);
/* The reference's checkpoint file (saveState/loadState,
 * src/flip3D.cpp:453-578), float build, native byte order:
 *   int nparticle; float max_dens; int pourTime; float pourPos[2];
 *   float pourRad; nparticle x 72-byte particle records (src/common.h:34-45:
 *   float p[3], u[3], n[3]; char type, visible, remove, thinparticle;
 *   float tmp[2][3], m, dens); press, n^3 floats with k fastest;
 *   wall_normal, n^3 x 4 floats (normal x, y, z and the perimeter flag).
 * Host arrays; n is not in the file (the reference's N is compiled in) and
 * fixes the grid sections' size. The writer stores remove = thinparticle = 0,
 * tmp = 0 (scratch in the reference, partly never initialised), m = 1 and
 * visible = (type == FLUID) when visible is null. */
typedef struct FlipCheckpoint {
  int n;
  int count;
  float max_dens;
  int pour_time;
  float pour_pos[2];
  float pour_rad;
  float *pos, *vel, *nrm; /* [count*3] */
  uint8_t *type;          /* [count] */
  uint8_t *visible;       /* [count], may be null */
  float *dens;            /* [count] */
  float *press;           /* [n^3] */
  float *wall_normal;     /* [n^3*4] */
} FlipCheckpoint;
int flipgpu_checkpoint_write(const char *path, const FlipCheckpoint *c);
/* particle count of a checkpoint for grid n (checks the file size) */
int flipgpu_checkpoint_count(const char *path, int n, int *count);
/* fills the caller's arrays (sized by flipgpu_checkpoint_count): c->count is
 * the capacity of every per-particle array given (FLIPGPU_EINVAL if
 * negative; FLIPGPU_ETOOBIG, with nothing read, if the file holds more
 * particles and any per-particle pointer is set); on return it holds the
 * file's particle count */
int flipgpu_checkpoint_read(const char *path, FlipCheckpoint *c);
/* The handle's state as a checkpoint: particles, pressure, max_dens, and
 * the wall-normal grid compute_wall_normal (src/flip3D.cpp:75-164) gives
 * for the current walls, computed on the device. pour_* are carried
 * through (the benchmark scenes do not pour). */
int flipgpu_save_state(FlipGpu *h, const char *path, int pour_time, const float *pour_pos,
                       float pour_rad);
/* Replace the handle's particles, pressure and max_dens from a checkpoint
 * (grid n of the handle); pour_* may be null. */
int flipgpu_load_state(FlipGpu *h, const char *path, int *pour_time, float *pour_pos,
                       float *pour_rad);
/* The files exporter::write3D writes for a mesh (src/exporter.cpp:70-167),
 * byte-identical text: write_obj's Wavefront OBJ (vertices
 * s*(v - wall_thick) with s = 1/(1 - 2 wall_thick), y and z swapped;
 * normals; faces 1-based as f a//a b//b c//c) and writeSunflow's scene file
 * (include template.sc; the mesh object with each vertex clamped to
 * [0.001, 0.999] after the wall offset and scaled by 100/(1 - 2 wall_thick);
 * 0-based triangles). Host arrays as flipgpu_get_mesh returns them. */
int flipgpu_write_obj(const char *path, const double *vertices, const double *normals,
                      int64_t n_vertices, const int32_t *faces, int64_t n_faces,
                      float wall_thick);
int flipgpu_write_sunflow(const char *path, const double *vertices, const double *normals,
                          int64_t n_vertices, const int32_t *faces, int64_t n_faces,
                          float wall_thick);
#define FLIPGPU_EXPORT_OBJ 1
#define FLIPGPU_EXPORT_SUNFLOW 2
/* Export the last flipgpu_mesh result as dir/obj/<frame>_scene.obj and/or
 * dir/sunflow/<frame>_scene.sc (plus dir/sunflow/template.sc when
 * sunflow_template is given). Returns once the download is enqueued; the
 * formatting and writing run on a host thread. flipgpu_export_wait joins it
 * and returns its status; the next export, or destroying the handle, joins
 * it too. */
int flipgpu_export_mesh(FlipGpu *h, const char *dir, int frame, float wall_thick, int formats,
                        const char *sunflow_template);
int flipgpu_export_wait(FlipGpu *h);
/* The reference's point-splat preview (write_frame, src/flip3D.cpp:1133-1192)
 * of the current particles as a width x height RGBA8 buffer (the reference
 * draws 1024 x 700): liquid particles rotated and projected, each blending
 * exp(-DENSITY*N/23) of (0.3, 0.5, 0.8) into 2x2 pixels; alpha 255.
 * rgba is host or device memory (on_device). */
int flipgpu_preview(FlipGpu *h, uint8_t *rgba, int width, int height, int on_device);
/* write_bmp (src/write_bmp.cpp): a 24-bit BMP of an RGBA8 buffer, rows in
 * buffer order. */
int flipgpu_write_bmp(const char *path, const uint8_t *rgba, int width, int height);
/* The launch-configuration autotuner: kernels whose results do not depend
 * on their tile shape or schedule (the U-Net's tcgen05 convolutions: lines
 * per unit and pipeline depth) time their candidates on first use per
 * problem size and keep the fastest. on = 0 turns tuning off (defaults run),
 * 1 on (the default; FLIPGPU_AUTOTUNE=0 in the environment starts it off),
 * -1 on and forgets the decisions made so far. The report is one line per
 * key: the choice and every candidate's median ms; returns its length. */
int flipgpu_set_autotune(int on);
int flipgpu_autotune_report(char *buf, int len);
/* particles currently in the handle (liquid and wall) */
int flipgpu_particle_count(const FlipGpu *h);

int flipgpu_set_particles(FlipGpu *h, int count, const float *pos,
                          const float *vel, const uint8_t *type,
                          const float *nrm, const float *dens, int on_device);
int flipgpu_get_particles(FlipGpu *h, float *pos, float *vel, float *dens,
                          uint8_t *type, int on_device);
int flipgpu_count(const FlipGpu *h);

/* Grid state, same host/device rule; NULL skips an array. */
int flipgpu_set_grid(FlipGpu *h, const float *u0, const float *u1,
                     const float *u2, const uint8_t *A, const float *L,
                     const float *press, const float *div, int on_device);
int flipgpu_get_grid(FlipGpu *h, float *u0, float *u1, float *u2, uint8_t *A,
                     float *L, float *press, float *div, int on_device);
/* The cell lists of the last sort. */
int flipgpu_get_cells(FlipGpu *h, uint32_t *cell_start, uint32_t *perm,
                      int on_device);

/* Density normalisation: set it, or compute it from the calibration
 * lattice of src/flip3D.cpp:689-709 with the density kernel. */
int flipgpu_set_max_density(FlipGpu *h, float max_dens);
int flipgpu_calibrate_max_density(FlipGpu *h, float *out);

/* ---- the hot path, one entry per reference function ------------------ */

/* sorter::sort (src/sorter.cpp:22-40): stable counting sort of particles
 * into cells. */
int flipgpu_sort(FlipGpu *h);
/* computeDensity (src/flip3D.cpp:166-190) on the current cell lists. */
int flipgpu_compute_density(FlipGpu *h);
/* sorter::markWater (src/sorter.cpp:83-93) into A, and sorter::levelset for
 * every cell into L (src/flip3D.cpp:824-826). */
int flipgpu_mark_water(FlipGpu *h);
/* add_ExtForce (src/flip3D.cpp:870-875). */
int flipgpu_add_force(FlipGpu *h);
/* mapper::mapP2G (src/mapper.cpp:17-88) into the face grids. */
int flipgpu_p2g(FlipGpu *h);
/* mapper::mapG2P (src/mapper.cpp:90-94): every particle's velocity = the
 * trilinear sample of the face grids at its position. */
int flipgpu_g2p(FlipGpu *h);
/* mapper::fetchVelocity (src/mapper.cpp:108-112) at count points: trilinear
 * samples of the handle's face grids. pts/out are float[count][3]. */
int flipgpu_fetch_velocity(FlipGpu *h, int count, const float *pts, float *out,
                           int on_device);
/* corrector::resample (src/corrector.cpp:15-47) at count points with kernel
 * radius re: the cell lists of the last sort over the particles' current
 * positions and velocities (the reference's sorter keeps particle pointers,
 * so it reads current data through old lists). vel holds the fallback
 * velocity on input and the resampled one on output. */
int flipgpu_resample(FlipGpu *h, int count, const float *pts, float *vel,
                     float re, int on_device);
/* implicit::implicit_func (src/implicit.cpp:14-38) at count points (float
 * [count][3]): distance to the nearest non-wall particle within the 5^3
 * cells around the point, capped at 8*density/n, minus density/n; the wall
 * value 4.5*density/n when a wall particle is closer than density/n. Reads
 * the lists of the last sort over current positions. out is double[count]. */
int flipgpu_implicit(FlipGpu *h, int count, const float *pts, double *out,
                     int on_device);
/* mesher::generateMesh (src/mesher.cpp:137-195) with mg = n+1, the way
 * write_mesh calls it after a step (src/flip3D.cpp:999-1004): the lists of
 * the last sort over current positions; the reference's A argument is
 * unused there and has no counterpart. Computes the mesh on the device and
 * returns its vertex and face counts; flipgpu_get_mesh copies it out. */
int flipgpu_mesh(FlipGpu *h, int64_t *n_vertices, int64_t *n_faces);
/* The last mesh: vertices and normals double[n_vertices][3], faces
 * int32[n_faces][3] (vertex indices), and optionally the field it meshed,
 * float[(n+1)^3] in the reference's dense_grid layout (x fastest, node
 * (x,y,z) at (z*(n+1) + y)*(n+1) + x, value = -implicit_func). Any pointer
 * may be NULL. */
int flipgpu_get_mesh(FlipGpu *h, double *vertices, double *normals,
                     int32_t *faces, float *field);
/* The pressure of the last solve as double[n^3]: with FAST-mode refinement
 * the double-float iterate the solver's tolerance was met on (the pressure
 * grid holds its FP32 rounding), otherwise the pressure grid itself. press is
 * host or device memory (on_device). */
int flipgpu_get_pressure(FlipGpu *h, double *press, int on_device);
/* solver::solve (src/solver.cpp:224-241) on the handle's A, L, pressure
 * (initial guess, overwritten) and divergence (negated, as the reference
 * does). */
int flipgpu_solve(FlipGpu *h, FlipGpuSolveStats *stats);
/* project (src/flip3D.cpp:807-868): divergence, solve, subcell gradient. */
int flipgpu_project(FlipGpu *h, FlipGpuSolveStats *stats);
/* solve_picflip (src/flip3D.cpp:1057-1103) after its sort. */
int flipgpu_picflip(FlipGpu *h, FlipGpuSolveStats *stats);
/* advect_particle (src/flip3D.cpp:877-969), including the wall constraint,
 * stuck-particle detection and reposition (src/flip3D.cpp:405-451). */
int flipgpu_advect(FlipGpu *h, int *stuck);
/* corrector::correct (src/corrector.cpp:49-115). */
int flipgpu_correct(FlipGpu *h);
/* simulateStep (src/flip3D.cpp:1194-1264) without preview and mesh I/O. */
int flipgpu_step(FlipGpu *h, FlipGpuSolveStats *stats);
/* One step on host data: the same results as flipgpu_put_state(pos_in,
 * vel_in) + flipgpu_step + flipgpu_get_particles(pos_out, vel_out), with
 * the transfers overlapped with the step on a second stream (the velocities
 * upload while the sort and density run; the positions download while the
 * corrector's velocity resample runs). Any pointer may be NULL (skipped);
 * in and out may be the same buffers. Host AoS float[np][3]; pinned memory
 * gives the full transfer rate. Returns after everything is done. */
int flipgpu_step_host(FlipGpu *h, const float *pos_in, const float *vel_in, float *pos_out,
                      float *vel_out, FlipGpuSolveStats *stats);

/* Replace positions and velocities of the current particle set (same count
 * and types as the last flipgpu_set_particles), host or device AoS. This is
 * the per-step upload of a host-side driver such as src/flip3D.cpp. */
int flipgpu_put_state(FlipGpu *h, const float *pos, const float *vel,
                      int on_device);

/* Number of kernels this library launched on the handle so far. */
int64_t flipgpu_launch_count(const FlipGpu *h);

/* Per-stage device time of flipgpu_step (CUDA events on the handle's
 * stream), the analogue of the reference's dumptime() stage prints
 * (src/flip3D.cpp:1219-1243). Stage ids index the FLIPGPU_STAGE_* list. */
#define FLIPGPU_STAGE_SORT 0       /* sort + payload (+ add_ExtForce) */
#define FLIPGPU_STAGE_DENSITY 1
#define FLIPGPU_STAGE_MARK 2       /* markWater + levelset */
#define FLIPGPU_STAGE_P2G 3
#define FLIPGPU_STAGE_DIV 4
#define FLIPGPU_STAGE_SOLVE 5
#define FLIPGPU_STAGE_GRAD 6       /* gradient + enforce_boundary */
#define FLIPGPU_STAGE_EXTRAP 7     /* extrapolate + subtract_grid */
#define FLIPGPU_STAGE_FLIP 8       /* G2P + FLIP blend; in flipgpu_step also
                                      advect_particle, fused with the blend */
#define FLIPGPU_STAGE_ADVECT 9     /* advect_particle (empty in flipgpu_step) */
#define FLIPGPU_STAGE_REPOSITION 10 /* stuck lists, placement, sort, resample */
#define FLIPGPU_STAGE_CORRECT 11
#define FLIPGPU_NSTAGES 12
int flipgpu_set_profiling(FlipGpu *h, int on);
/* ms[i] and calls[i] accumulated since profiling was switched on. */
int flipgpu_get_profile(FlipGpu *h, double *ms, int64_t *calls, int max);
/* The main kernels' own device time since profiling was switched on (CUDA
 * events around each launch on the handle's stream): one line per kernel,
 * "name<TAB>ms<TAB>launches". The persistent solve (k_cg_mg, k_cg_cg1,
 * k_cg_ic, k_cg), the FAST gathers (k_density, k_p2g_cells,
 * k_spring_inline, k_resample_inline) and k_flip_advect are timed. Writes
 * at most len - 1 characters and a terminating zero; returns the length of
 * the whole text. */
int flipgpu_get_kernel_profile(FlipGpu *h, char *buf, int len);

/* Testing aid (no reference counterpart): set the counter from which the
 * IC(0)/MIC(0) wavefront's solves take the tags of their words (each solve
 * advances it by two per preconditioner application). A value near the end
 * of the 32-bit range makes the next solve clear the tagged buffers and
 * start again at 0, which a test checks gives the same result. Allocates
 * the wavefront buffers if needed; runs on the handle's stream. */
int flipgpu_set_ic_tag_counter(FlipGpu *h, unsigned value);
/* its current value (synchronises) */
int flipgpu_get_ic_tag_counter(FlipGpu *h, unsigned *value);

/* Cell sort that allocates no device memory. It has no counterpart in the
 * reference. It is for callers that may not allocate on the GPU, such as a
 * plugin inside a host application that owns all device memory, or a frame
 * loop that cannot take the device-wide stall of cudaMalloc/cudaFree. It
 * writes the same cell_start[n^3+1] / perm[count] as flipgpu_sort from a
 * device AoS position buffer pos[count][3]; every pointer is device memory
 * the caller owns. Its working memory is one fixed array per device, alive
 * until the process exits, sized for at most FLIPGPU_NOALLOC_MAX_CELLS cells
 * (n <= 64) and FLIPGPU_NOALLOC_MAX_PARTICLES particles (about 5.3 MB);
 * larger inputs return FLIPGPU_ETOOBIG. The first call on a device looks that
 * array up (with the device current); make it before any stream capture.
 * Calls share the array: calls that overlap on the GPU race and give
 * undefined results. stream is a cudaStream_t (NULL = default stream). */
#define FLIPGPU_NOALLOC_MAX_CELLS (64 * 64 * 64)
#define FLIPGPU_NOALLOC_MAX_PARTICLES (1 << 20)
int flipgpu_sort_cells_noalloc(int n, int count, const float *pos,
                               uint32_t *cell_start, uint32_t *perm,
                               void *stream);

/* ---------------------------------------------------------------------------
 * Steps without host synchronisation, CUDA graphs and batches of scenes (no
 * counterpart in the reference, which runs one scene per process).
 *
 * flipgpu_step_async is flipgpu_step with nothing waiting for the device
 * (FAST solver only; no warm start, no profiling): the solve's statistics
 * stay on the device until flipgpu_last_solve_stats reads them.
 * flipgpu_capture_step records one such step as a CUDA graph (the step
 * counter that keys the random draws lives on the device, so replays
 * advance it) and flipgpu_step_graph replays it. */
int flipgpu_step_async(FlipGpu *h);
int flipgpu_capture_step(FlipGpu *h);
int flipgpu_step_graph(FlipGpu *h);
int flipgpu_last_solve_stats(FlipGpu *h, FlipGpuSolveStats *stats);

/* A batch advances independent simulations together: each handle keeps its
 * own stream, so the steps of different scenes overlap on the GPU and the
 * host does not wait between them. The batch does not own the handles. */
typedef struct FlipBatch FlipBatch;
int flipbatch_create(FlipBatch **out);
int flipbatch_destroy(FlipBatch *b);
int flipbatch_add(FlipBatch *b, FlipGpu *h);
/* record every member's step as a graph; later flipbatch_step calls replay */
int flipbatch_capture(FlipBatch *b);
/* one step of every member (graphs if captured, else asynchronous steps) */
int flipbatch_step(FlipBatch *b);
int flipbatch_sync(FlipBatch *b);
/* Share the GPU between the members' pressure solves. Member i's
 * persistent solve gets max(1, share * C_i * cells_i / cells of all
 * members) blocks, C_i its solve kernel's co-resident grid (at share 1 all
 * members' solves fit side by side). The tuner times the candidate shares
 * (uncapped, 0.5, 1, 2, 4, 8, 16) on every member's current system, solved by
 * all members at once from the saved warm start, keeps the fastest and
 * puts each member's pressure back as its last step left it; the decision
 * appears in flipgpu_autotune_report. Every member must have stepped at
 * least once. Captured graphs are re-recorded with the new grids. The
 * grids change the order of the solve's sums, so a member's bits then
 * match a lone handle with the same flipgpu_set_solve_blocks. share_out
 * (optional) receives the chosen share, 0 for uncapped; flipgpu_last_solve_stats
 * then reports the last trial. */
int flipbatch_tune(FlipBatch *b, double *share_out);
/* cap on the persistent pressure solve's grid (0 = none, the default): a
 * simulation that shares the GPU with others leaves them SMs. The IC(0)
 * wavefront keeps its full grid. */
int flipgpu_set_solve_blocks(FlipGpu *h, int blocks);
int flipgpu_get_solve_blocks(const FlipGpu *h, int *blocks);

/* ---------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference; the reference starts
 * CG from the previous step's pressure, src/flip3D.cpp:679 and
 * src/solver.cpp:224).
 *
 * A 3D U-Net (4 levels, 16/32/48/64 channels, BF16 activations, FP32
 * accumulation, tensor-core implicit-GEMM convolutions) maps (liquid mask,
 * b, previous pressure x0 and its residual r0 = b - A x0) to a correction d
 * (an approximation of A^-1 r0). With a network attached, a
 * FAST-mode solve starts from x0 + g d, where g = (Ad).r0 / (Ad).(Ad)
 * minimises the residual along d (so the starting residual is never above
 * the previous-step guess's: g = 0 is on the line; FLIPGPU_WARM_STEP=anorm
 * in the environment selects g = d.r0 / d.Ad, the least A-norm error
 * instead) and CG still runs to the same relative residual. Grids must be a multiple
 * of 8 cells per axis. All array arguments of the flipunet_* calls are
 * device pointers to batch systems of n^3 cells each, concatenated. */
int64_t flipunet_param_count(void);
int flipunet_create(uint64_t seed, FlipUNet **out);
int flipunet_destroy(FlipUNet *u);
const char *flipunet_last_error(const FlipUNet *u);
int flipunet_set_stream(FlipUNet *u, void *stream);
/* FP32 master parameters (host arrays of flipunet_param_count() floats);
 * setting them resets the optimiser state. */
int flipunet_get_params(FlipUNet *u, float *params);
int flipunet_set_params(FlipUNet *u, const float *params);
/* Forward 3x3x3 convolutions on the tcgen05 tensor cores (TMEM
 * accumulators, 1, the default) or on the mma.sync path (0). Backward-data
 * and weight-gradient convolutions always use mma.sync. */
int flipunet_set_tensor_path(FlipUNet *u, int tcgen05);
/* Coarsened warm start (levels 0..3, default 0): the 16 input features are
 * computed on the solver's grid n, average-pooled `levels` times, the
 * network runs on the (n >> levels)^3 grid and its output is prolonged
 * trilinearly back to n before the step along it. Training targets
 * are the liquid-cell averages of x and x0 over each coarse cell. n must be
 * a multiple of 8 << levels. */
int flipunet_set_coarsening(FlipUNet *u, int levels);
int flipunet_get_coarsening(const FlipUNet *u);
/* delta = the correction for systems (A, b, x0, r0), zero off the liquid. */
int flipunet_predict(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                     const float *x0, const float *r0, float *delta);
/* Mean squared error over liquid cells between the network output and
 * (x - x0)/s (s = RMS of r0 over the liquid times h^2), its gradient (host
 * array, may be NULL) and no update. */
int flipunet_gradients(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                       const float *x0, const float *r0, const float *x, double *loss,
                       float *grad);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on that loss. */
int flipunet_train_step(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                        const float *x0, const float *r0, const float *x, float lr,
                        double *loss);
/* Attach a network to a simulation's FAST-mode solves (NULL detaches). */
int flipgpu_set_warm_start(FlipGpu *h, FlipUNet *u);
/* Keep a copy of each solve's system: flipgpu_get_solve_system returns A,
 * L (the levelset of the subcell diagonal), b (the solver's right-hand side,
 * already negated as solver::solve does), x0 (the initial guess before any
 * warm start), r0 = b - A x0 (FAST mode) and x (the solution) of the last
 * solve. Any pointer may be NULL. To solve such a system again,
 * set_grid(A, L, press = x0, div = -b). */
int flipgpu_set_capture(FlipGpu *h, int on);
int flipgpu_get_solve_system(FlipGpu *h, uint8_t *A, float *L, float *b, float *x0, float *r0,
                             float *x, int on_device);

#ifdef __cplusplus
}
#endif
#endif /* FLIPGPU_H */
