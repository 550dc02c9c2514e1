/*
 * noalloc_sort.cu — the cell sort for callers that must not allocate device
 * memory.
 *
 * Some callers cannot call cudaMalloc: a plugin inside a host application
 * that owns the GPU's memory and hands its guests only the buffers it
 * allocated itself, or a per-frame loop that cannot afford the implicit
 * device-wide synchronisation of cudaFree or the latency of a first-touch
 * allocation. flipgpu_sort_cells_noalloc serves them: it builds the same cell
 * lists as flipgpu_sort from a caller-owned position buffer into caller-owned
 * outputs, and keeps its working memory (per-cell counters, per-particle
 * tickets, scan partials) in the fixed array below, which exists once per
 * device for the lifetime of the process.
 *
 * The order inside each cell is made by one thread per cell for the usual
 * handful of particles (insertion sort, at most 32), and for crowded cells by
 * one block each: the block marks the cell's particle indices in a bitmap in
 * shared memory (indices are below 2^20, so the bitmap of one cell's index
 * range fits in 128 KB) and writes them back in bit order. The work is
 * linear in the particles of a cell, so a degenerate input (every position
 * clamped into one corner cell) costs about a millisecond, not a quadratic
 * number of moves.
 *
 * Rules of use:
 *   - at most FLIPGPU_NOALLOC_MAX_CELLS cells (n <= 64) and
 *     FLIPGPU_NOALLOC_MAX_PARTICLES particles; larger inputs are rejected
 *     with FLIPGPU_ETOOBIG before anything runs;
 *   - the first call on a device looks up the array's device address (with
 *     that device current) and caches it; make that first call before any
 *     stream capture;
 *   - every call on a device shares the one array and leaves its contents
 *     behind; each call clears the counters it needs, but two calls that
 *     overlap on the GPU (different streams, no ordering between them) race
 *     on it and both results are then undefined.
 */
#include <mutex>

#include "devcommon.cuh"

namespace {

constexpr int NA_BLOCK = 256;
constexpr int NA_ITEMS = 16;
constexpr int NA_TILE = NA_BLOCK * NA_ITEMS;
constexpr int NA_MAX_N = 64; /* cube root of FLIPGPU_NOALLOC_MAX_CELLS */
static_assert(NA_MAX_N * NA_MAX_N * NA_MAX_N == FLIPGPU_NOALLOC_MAX_CELLS, "cell limit");
constexpr size_t NA_COUNTS = (size_t)FLIPGPU_NOALLOC_MAX_CELLS + 1;
constexpr size_t NA_PARTIALS = (NA_COUNTS + NA_TILE - 1) / NA_TILE + 1;
/* cells with more than NA_SMALL particles are ordered by a block each */
constexpr uint32_t NA_SMALL = 32;
constexpr size_t NA_CROWDED = (size_t)FLIPGPU_NOALLOC_MAX_PARTICLES / (NA_SMALL + 1) + 1;
constexpr int NA_CROWD_BLOCK = 1024;
constexpr int NA_CROWD_GRID = 152;
/* bitmap over one cell's particle-index range: every index is below 2^20 */
constexpr uint32_t NA_BITMAP_WORDS = (uint32_t)FLIPGPU_NOALLOC_MAX_PARTICLES / 32;
constexpr size_t NA_CROWD_SMEM = (size_t)NA_BITMAP_WORDS * sizeof(uint32_t);
constexpr size_t NA_WORDS =
    NA_COUNTS + (size_t)FLIPGPU_NOALLOC_MAX_PARTICLES + NA_PARTIALS + 1 + NA_CROWDED;

/* counters [NA_COUNTS] | tickets [MAX_PARTICLES] | scan partials |
 * crowded-cell count [1] | crowded cells [NA_CROWDED] */
static __device__ __align__(256) uint32_t g_noalloc_scratch[NA_WORDS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mutex;
uint32_t *g_scratch_dev[NA_MAX_DEVICES] = {};

__device__ __forceinline__ uint32_t na_key(const float *__restrict__ pos, int p, int n, float fn) {
  int i = cell_clamp(pos[3 * (size_t)p], fn, n);
  int j = cell_clamp(pos[3 * (size_t)p + 1], fn, n);
  int k = cell_clamp(pos[3 * (size_t)p + 2], fn, n);
  return (uint32_t)cell_id(n, i, j, k);
}

__global__ void na_zero(uint32_t *__restrict__ a, size_t n, uint32_t *__restrict__ crowd_count) {
  size_t i = (size_t)blockIdx.x * NA_BLOCK + threadIdx.x;
  if (i < n) a[i] = 0u;
  if (i == 0) *crowd_count = 0u;
}

__global__ void na_count(const float *__restrict__ pos, int np, int n, float fn,
                         uint32_t *__restrict__ counts, uint32_t *__restrict__ ticket) {
  int p = blockIdx.x * NA_BLOCK + threadIdx.x;
  if (p >= np) return;
  ticket[p] = atomicAdd(&counts[na_key(pos, p, n, fn)], 1u);
}

__device__ __forceinline__ uint32_t na_block_scan(uint32_t v, uint32_t &total) {
  __shared__ uint32_t warp_tot[NA_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = (lane < NA_BLOCK / 32) ? warp_tot[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NA_BLOCK / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  uint32_t off = wid ? warp_tot[wid - 1] : 0u;
  total = warp_tot[NA_BLOCK / 32 - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void na_scan_reduce(const uint32_t *__restrict__ in, size_t n,
                               uint32_t *__restrict__ part) {
  size_t base = (size_t)blockIdx.x * NA_TILE + (size_t)threadIdx.x * NA_ITEMS;
  uint32_t s = 0;
  for (int i = 0; i < NA_ITEMS; i++)
    if (base + i < n) s += in[base + i];
  uint32_t tot = block_sum_u32<NA_BLOCK>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void na_scan_spine(uint32_t *__restrict__ part, size_t nb) {
  uint32_t carry = 0;
  for (size_t base = 0; base < nb; base += NA_BLOCK) {
    size_t i = base + threadIdx.x;
    uint32_t v = (i < nb) ? part[i] : 0u;
    uint32_t tot;
    uint32_t ex = na_block_scan(v, tot);
    if (i < nb) part[i] = carry + ex;
    carry += tot;
  }
}

__global__ void na_scan_down(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                             size_t n, const uint32_t *__restrict__ part) {
  size_t base = (size_t)blockIdx.x * NA_TILE + (size_t)threadIdx.x * NA_ITEMS;
  uint32_t v[NA_ITEMS];
  uint32_t s = 0;
  for (int i = 0; i < NA_ITEMS; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t run = na_block_scan(s, tot) + part[blockIdx.x];
  for (int i = 0; i < NA_ITEMS; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

__global__ void na_scatter(const float *__restrict__ pos, int np, int n, float fn,
                           const uint32_t *__restrict__ ticket,
                           const uint32_t *__restrict__ cell_start,
                           uint32_t *__restrict__ perm) {
  int p = blockIdx.x * NA_BLOCK + threadIdx.x;
  if (p >= np) return;
  perm[cell_start[na_key(pos, p, n, fn)] + ticket[p]] = (uint32_t)p;
}

/* Particle order inside each cell (the tickets were taken in any order):
 * insertion sort for at most NA_SMALL entries; crowded cells are listed for
 * na_order_crowded. */
__global__ void na_order(size_t nc, const uint32_t *__restrict__ cell_start,
                         uint32_t *__restrict__ perm, uint32_t *__restrict__ crowd_count,
                         uint32_t *__restrict__ crowd) {
  size_t c = (size_t)blockIdx.x * NA_BLOCK + threadIdx.x;
  if (c >= nc) return;
  uint32_t s = cell_start[c], e = cell_start[c + 1];
  if (e - s > NA_SMALL) {
    /* at most count / (NA_SMALL + 1) < NA_CROWDED such cells */
    crowd[atomicAdd(crowd_count, 1u)] = (uint32_t)c;
    return;
  }
  for (uint32_t i = s + 1; i < e; i++) {
    uint32_t v = perm[i];
    uint32_t j = i;
    while (j > s && perm[j - 1] > v) {
      perm[j] = perm[j - 1];
      j--;
    }
    perm[j] = v;
  }
}

/* One block per crowded cell (grid-stride over the list): the cell's
 * particle indices, all distinct and below 2^20, are marked in a shared
 * bitmap over [lowest, highest] and written back in increasing order. */
__global__ void __launch_bounds__(NA_CROWD_BLOCK)
na_order_crowded(const uint32_t *__restrict__ cell_start, uint32_t *__restrict__ perm,
                 const uint32_t *__restrict__ crowd_count, const uint32_t *__restrict__ crowd) {
  extern __shared__ uint32_t bm[];
  __shared__ uint32_t s_lo, s_hi;
  __shared__ uint32_t warp_tot[NA_CROWD_BLOCK / 32];
  const uint32_t ncrowd = *crowd_count;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t e = blockIdx.x; e < ncrowd; e += gridDim.x) {
    const uint32_t c = crowd[e];
    const uint32_t s = cell_start[c], t = cell_start[c + 1];
    if (threadIdx.x == 0) {
      s_lo = 0xffffffffu;
      s_hi = 0u;
    }
    __syncthreads();
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (uint32_t i = s + threadIdx.x; i < t; i += NA_CROWD_BLOCK) {
      const uint32_t v = perm[i];
      lo = min(lo, v);
      hi = max(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) {
      atomicMin(&s_lo, lo);
      atomicMax(&s_hi, hi);
    }
    __syncthreads();
    const uint32_t base = s_lo;
    /* indices are below 2^20, so the range fits NA_BITMAP_WORDS words */
    const uint32_t words = ((s_hi - base) >> 5) + 1;
    for (uint32_t w = threadIdx.x; w < words; w += NA_CROWD_BLOCK) bm[w] = 0u;
    __syncthreads();
    for (uint32_t i = s + threadIdx.x; i < t; i += NA_CROWD_BLOCK) {
      const uint32_t d = perm[i] - base;
      atomicOr(&bm[d >> 5], 1u << (d & 31));
    }
    __syncthreads();
    /* each thread owns a contiguous run of words; an exclusive scan of the
     * runs' bit counts gives each run's first output slot */
    const uint32_t per = (words + NA_CROWD_BLOCK - 1) / NA_CROWD_BLOCK;
    const uint32_t w0 = min(words, threadIdx.x * per), w1 = min(words, w0 + per);
    uint32_t mine = 0;
    for (uint32_t w = w0; w < w1; w++) mine += __popc(bm[w]);
    uint32_t x = mine;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t v = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      warp_tot[lane] = v;
    }
    __syncthreads();
    uint32_t out = s + (wid ? warp_tot[wid - 1] : 0u) + x - mine;
    for (uint32_t w = w0; w < w1; w++) {
      uint32_t bits = bm[w];
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        perm[out++] = base + (w << 5) + (uint32_t)b;
      }
    }
    __syncthreads();
  }
}

/* Device address of the scratch array on the current device, looked up once
 * per device. */
cudaError_t scratch_for_current_device(uint32_t **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_dev[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(na_order_crowded, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)NA_CROWD_SMEM);
    if (e != cudaSuccess) return e;
    g_scratch_dev[dev] = (uint32_t *)ptr;
  }
  *out = g_scratch_dev[dev];
  return cudaSuccess;
}

} // namespace

extern "C" int flipgpu_sort_cells_noalloc(int n, int count, const float *pos,
                                          uint32_t *cell_start, uint32_t *perm,
                                          void *stream) {
  if (n < 1 || count < 0 || !cell_start || (count > 0 && (!pos || !perm)))
    return FLIPGPU_EINVAL;
  /* n itself is bounded first: n^3 of a large n would wrap */
  if (n > NA_MAX_N || count > FLIPGPU_NOALLOC_MAX_PARTICLES) return FLIPGPU_ETOOBIG;
  const size_t nc = (size_t)n * n * n;
  uint32_t *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return FLIPGPU_ECUDA;
  uint32_t *counts = scratch;
  uint32_t *ticket = scratch + NA_COUNTS;
  uint32_t *part = ticket + FLIPGPU_NOALLOC_MAX_PARTICLES;
  uint32_t *crowd_count = part + NA_PARTIALS;
  uint32_t *crowd = crowd_count + 1;
  cudaStream_t s = (cudaStream_t)stream;
  const float fn = (float)n;
  const size_t ncount = nc + 1; /* the extra zero makes cell_start[nc] = count */
  na_zero<<<grid_for(ncount, NA_BLOCK), NA_BLOCK, 0, s>>>(counts, ncount, crowd_count);
  if (count > 0)
    na_count<<<grid_for(count, NA_BLOCK), NA_BLOCK, 0, s>>>(pos, count, n, fn, counts, ticket);
  const size_t nb = (ncount + NA_TILE - 1) / NA_TILE;
  na_scan_reduce<<<(unsigned)nb, NA_BLOCK, 0, s>>>(counts, ncount, part);
  na_scan_spine<<<1, NA_BLOCK, 0, s>>>(part, nb);
  na_scan_down<<<(unsigned)nb, NA_BLOCK, 0, s>>>(counts, cell_start, ncount, part);
  if (count > 0) {
    na_scatter<<<grid_for(count, NA_BLOCK), NA_BLOCK, 0, s>>>(pos, count, n, fn, ticket,
                                                              cell_start, perm);
    na_order<<<grid_for(nc, NA_BLOCK), NA_BLOCK, 0, s>>>(nc, cell_start, perm, crowd_count,
                                                         crowd);
    na_order_crowded<<<NA_CROWD_GRID, NA_CROWD_BLOCK, NA_CROWD_SMEM, s>>>(cell_start, perm,
                                                                          crowd_count, crowd);
  }
  return cudaGetLastError() == cudaSuccess ? FLIPGPU_OK : FLIPGPU_ECUDA;
}
