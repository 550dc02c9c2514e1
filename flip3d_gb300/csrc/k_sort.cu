/*
 * k_sort.cu — sorter::sort (src/sorter.cpp:22-40) as a stable counting sort.
 *
 *   count    key = cell of the clamped position (the reference's clamp),
 *            rank = atomic ticket within the cell (integer atomics: the
 *            counts are deterministic, the tickets are not)
 *   scan     cell_start = exclusive prefix sum of the counts
 *   scatter  perm[cell_start[key] + rank] = particle
 *   fixup    each cell's slots sorted by particle index, which makes the
 *            lists identical to the reference's push_back order (FAST
 *            arithmetic: by the z half of the cell first, then by index)
 *   payload  sorted copies of position / clamped grid position / velocity
 *            for the gather stages (optionally applying add_ExtForce)
 *
 * Also the device-wide exclusive scan used by the sort and the reposition
 * compactions.
 */
#include "devcommon.cuh"

namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

/* Exclusive block scan of one value per thread; returns the block total. */
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &total) {
  __shared__ uint32_t warp_tot[SCAN_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = (lane < SCAN_BLOCK / 32) ? warp_tot[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_BLOCK / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  uint32_t warp_off = wid ? warp_tot[wid - 1] : 0u;
  total = warp_tot[SCAN_BLOCK / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

/* nlive (optional): only the first *nlive + 1 entries are scanned; the
 * tiles past them write a zero block sum and nothing else. */
__device__ __forceinline__ size_t scan_len(size_t n, const int *nlive) {
  if (!nlive) return n;
  const size_t m = (size_t)max(*nlive, 0) + 1;
  return m < n ? m : n;
}

__global__ void k_scan_reduce(const uint32_t *__restrict__ in, size_t n,
                              uint32_t *__restrict__ bsum, const int *__restrict__ nlive) {
  n = scan_len(n, nlive);
  if ((size_t)blockIdx.x * SCAN_TILE >= n) {
    if (threadIdx.x == 0) bsum[blockIdx.x] = 0u;
    return;
  }
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++)
    if (base + i < n) s += in[base + i];
  uint32_t tot = block_sum_u32<SCAN_BLOCK>(s);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

/* One block scans the block sums in chunks, carrying the running total. */
__global__ void k_scan_spine(uint32_t *__restrict__ bsum, size_t nb) {
  uint32_t carry = 0;
  for (size_t base = 0; base < nb; base += SCAN_BLOCK) {
    size_t i = base + threadIdx.x;
    uint32_t v = (i < nb) ? bsum[i] : 0u;
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(v, tot);
    if (i < nb) bsum[i] = carry + ex;
    carry += tot;
  }
}

__global__ void k_scan_down(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                            size_t n, const uint32_t *__restrict__ bsum,
                            const int *__restrict__ nlive) {
  n = scan_len(n, nlive);
  if ((size_t)blockIdx.x * SCAN_TILE >= n) return;
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t run = block_exclusive_scan(s, tot) + bsum[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

/* key = the particle's cell; with HALVES (FAST arithmetic) bit 31 also
 * marks a particle at or above its cell's mid-plane in z, (k + 0.5) h, and
 * the scatter carries that bit into perm for k_sort_fixup_halves (cell ids
 * stay below 2^30, as flipgpu_create allows n <= 1024, and particle
 * indices below 2^31). */
template <bool HALVES>
__global__ void k_sort_count(SimConst c, const float *__restrict__ px,
                             const float *__restrict__ py, const float *__restrict__ pz,
                             uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                             uint32_t *__restrict__ count) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.np) return;
  const float z = pz[p];
  int i = cell_clamp(px[p], c.fn, c.n);
  int j = cell_clamp(py[p], c.fn, c.n);
  int k = cell_clamp(z, c.fn, c.n);
  uint32_t kk = (uint32_t)cell_id(c.n, i, j, k);
  const bool up = HALVES && z >= ((float)k + 0.5f) * c.h;
  key[p] = kk | (up ? 0x80000000u : 0u);
  rank[p] = atomicAdd(&count[kk], 1u);
}

__global__ void k_sort_scatter(int np, const uint32_t *__restrict__ key,
                               const uint32_t *__restrict__ rank,
                               const uint32_t *__restrict__ cell_start,
                               uint32_t *__restrict__ perm) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const uint32_t kk = key[p];
  perm[cell_start[kk & 0x7fffffffu] + rank[p]] = (uint32_t)p | (kk & 0x80000000u);
}

/* Order each cell's slots by particle index: insertion sort for the usual
 * handful, heapsort for crowded cells. */
__global__ void k_sort_fixup(size_t nc, const uint32_t *__restrict__ cell_start,
                             uint32_t *__restrict__ perm) {
  size_t cidx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cidx >= nc) return;
  uint32_t s = cell_start[cidx], e = cell_start[cidx + 1];
  uint32_t len = e - s;
  if (len < 2) return;
  uint32_t *a = perm + s;
  if (len <= 32) {
    for (uint32_t i = 1; i < len; i++) {
      uint32_t v = a[i];
      uint32_t j = i;
      while (j > 0 && a[j - 1] > v) {
        a[j] = a[j - 1];
        j--;
      }
      a[j] = v;
    }
    return;
  }
  auto sift = [&](uint32_t root, uint32_t end) {
    while (true) {
      uint32_t child = 2 * root + 1;
      if (child >= end) break;
      if (child + 1 < end && a[child] < a[child + 1]) child++;
      if (a[root] >= a[child]) break;
      uint32_t t = a[root];
      a[root] = a[child];
      a[child] = t;
      root = child;
    }
  };
  for (uint32_t i = len / 2; i-- > 0;) sift(i, len);
  for (uint32_t end = len - 1; end > 0; end--) {
    uint32_t t = a[0];
    a[0] = a[end];
    a[end] = t;
    sift(0, end);
  }
}

/* FAST arithmetic: each cell's slots ordered by (z half, particle index),
 * the particles below the cell's mid-plane (k + 0.5) h first, and
 * cell_mid[c] the slot where the upper half starts, so that a walk along a
 * row of cells can start or stop at half a cell. The half arrives in bit
 * 31 of each slot (k_sort_count<true>, k_sort_scatter), which makes it the
 * leading sort key; the bit is cleared at the end. */
__global__ void k_sort_fixup_halves(size_t nc, const uint32_t *__restrict__ cell_start,
                                    uint32_t *__restrict__ perm,
                                    uint32_t *__restrict__ cell_mid) {
  size_t cidx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cidx >= nc) return;
  const uint32_t s = cell_start[cidx], e = cell_start[cidx + 1];
  const uint32_t len = e - s;
  uint32_t *a = perm + s;
  uint32_t low = 0;
  for (uint32_t i = 0; i < len; i++) low += a[i] >> 31 ? 0u : 1u;
  cell_mid[cidx] = s + low;
  if (len >= 2) {
    if (len <= 32) {
      for (uint32_t i = 1; i < len; i++) {
        uint32_t v = a[i];
        uint32_t j = i;
        while (j > 0 && a[j - 1] > v) {
          a[j] = a[j - 1];
          j--;
        }
        a[j] = v;
      }
    } else {
      auto sift = [&](uint32_t root, uint32_t end) {
        while (true) {
          uint32_t child = 2 * root + 1;
          if (child >= end) break;
          if (child + 1 < end && a[child] < a[child + 1]) child++;
          if (a[root] >= a[child]) break;
          uint32_t t = a[root];
          a[root] = a[child];
          a[child] = t;
          root = child;
        }
      };
      for (uint32_t i = len / 2; i-- > 0;) sift(i, len);
      for (uint32_t end = len - 1; end > 0; end--) {
        uint32_t t = a[0];
        a[0] = a[end];
        a[end] = t;
        sift(0, end);
      }
    }
  }
  for (uint32_t i = low; i < len; i++) a[i] &= 0x7fffffffu;
}

/* Sorted payload; with apply_gravity also add_ExtForce (src/flip3D.cpp:
 * 870-875) on the fluid velocities, canonical and sorted. */
/* The sorted copies a caller needs (spos always): PL_SPG, PL_SVEL, PL_SDENS
 * (flipgpu_impl.h). add_ExtForce updates the canonical velocity whichever
 * copies are written. */
template <int FIELDS>
__global__ void k_payload(SimConst c, int apply_gravity, const uint32_t *__restrict__ perm,
                          const float *__restrict__ px, const float *__restrict__ py,
                          const float *__restrict__ pz, float *__restrict__ vx,
                          float *__restrict__ vy, float *__restrict__ vz,
                          const uint8_t *__restrict__ type, const float *__restrict__ dens,
                          float4 *__restrict__ spos, float4 *__restrict__ spg,
                          float4 *__restrict__ svel, float *__restrict__ sdens) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= c.np) return;
  uint32_t p = perm[a];
  float x = px[p], y = py[p], z = pz[p];
  uint8_t t = type[p];
  float tw = pack_type(t);
  spos[a] = make_float4(x, y, z, tw);
  if (FIELDS & PL_SPG)
    /* FLOAT x = fmax(0, fmin(gn, gn*p)) (src/mapper.cpp:28-30) */
    spg[a] = make_float4(fmaxf(0.0f, fminf(c.fn, c.fn * x)), fmaxf(0.0f, fminf(c.fn, c.fn * y)),
                         fmaxf(0.0f, fminf(c.fn, c.fn * z)), tw);
  if ((FIELDS & PL_SVEL) || apply_gravity) {
    float ux = vx[p], uy = vy[p], uz = vz[p];
    if (apply_gravity && t == CELL_FLUID) {
      uy = refmath::add_fd(uy, c.grav_h, c.grav_l, c.grav);
      vy[p] = uy;
    }
    if (FIELDS & PL_SVEL) svel[a] = make_float4(ux, uy, uz, 0.0f);
  }
  if (FIELDS & PL_SDENS) sdens[a] = dens[p];
}

/* The payload in two parts, for steps whose velocities arrive while the
 * sort runs: positions, grid positions and densities first, the velocities
 * (with add_ExtForce) once they are on the device. Same values as k_payload. */
template <bool SDENS>
__global__ void k_payload_pos(SimConst c, const uint32_t *__restrict__ perm,
                              const float *__restrict__ px, const float *__restrict__ py,
                              const float *__restrict__ pz, const uint8_t *__restrict__ type,
                              const float *__restrict__ dens, float4 *__restrict__ spos,
                              float4 *__restrict__ spg, float *__restrict__ sdens) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= c.np) return;
  uint32_t p = perm[a];
  float x = px[p], y = py[p], z = pz[p];
  float tw = pack_type(type[p]);
  spos[a] = make_float4(x, y, z, tw);
  spg[a] = make_float4(fmaxf(0.0f, fminf(c.fn, c.fn * x)), fmaxf(0.0f, fminf(c.fn, c.fn * y)),
                       fmaxf(0.0f, fminf(c.fn, c.fn * z)), tw);
  if (SDENS) sdens[a] = dens[p];
}

__global__ void k_payload_vel(SimConst c, int apply_gravity, const uint32_t *__restrict__ perm,
                              float *__restrict__ vx, float *__restrict__ vy,
                              float *__restrict__ vz, const uint8_t *__restrict__ type,
                              float4 *__restrict__ svel) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= c.np) return;
  uint32_t p = perm[a];
  float ux = vx[p], uy = vy[p], uz = vz[p];
  if (apply_gravity && type[p] == CELL_FLUID) {
    uy = refmath::add_fd(uy, c.grav_h, c.grav_l, c.grav);
    vy[p] = uy;
  }
  svel[a] = make_float4(ux, uy, uz, 0.0f);
}

/* Ordered compaction over tiles of SCAN_TILE: count each tile's selected
 * elements, scan the tile counts (k_scan_spine), then each tile writes its
 * selected indices in ascending order at its offset. Reads the predicate's
 * inputs twice and writes only the list. */
template <class Pred>
__global__ void k_cmp_count(size_t n, Pred pred, uint32_t *__restrict__ tile_cnt) {
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++)
    if (base + i < n && pred(base + i)) s++;
  const uint32_t tot = block_sum_u32<SCAN_BLOCK>(s);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = tot;
}

template <class Pred>
__global__ void k_cmp_write(size_t n, Pred pred, const uint32_t *__restrict__ tile_off,
                            uint32_t *__restrict__ idx, int *__restrict__ count) {
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t bits = 0, s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++)
    if (base + i < n && pred(base + i)) {
      bits |= 1u << i;
      s++;
    }
  uint32_t tot;
  uint32_t off = block_exclusive_scan(s, tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++)
    if (bits & (1u << i)) idx[off++] = (uint32_t)(base + i);
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *count = (int)(tile_off[blockIdx.x] + tot);
}

/* a particle flag set */
struct PredFlag {
  const uint8_t *f;
  __device__ __forceinline__ bool operator()(size_t i) const { return f[i] != 0; }
};

/* a deep-water cell: FLUID with its six in-grid neighbours FLUID
 * (src/flip3D.cpp:409-421) */
struct PredDeepWater {
  int n;
  const uint8_t *A;
  __device__ __forceinline__ bool operator()(size_t c) const {
    if (A[c] != CELL_FLUID) return false;
    int i, j, k;
    decode_index(c, n, n, i, j, k);
    if (i > 0 && A[cell_id(n, i - 1, j, k)] != CELL_FLUID) return false;
    if (i < n - 1 && A[cell_id(n, i + 1, j, k)] != CELL_FLUID) return false;
    if (j > 0 && A[cell_id(n, i, j - 1, k)] != CELL_FLUID) return false;
    if (j < n - 1 && A[cell_id(n, i, j + 1, k)] != CELL_FLUID) return false;
    if (k > 0 && A[cell_id(n, i, j, k - 1)] != CELL_FLUID) return false;
    if (k < n - 1 && A[cell_id(n, i, j, k + 1)] != CELL_FLUID) return false;
    return true;
  }
};

template <class Pred>
cudaError_t compact(FlipGpu *h, size_t n, Pred pred, uint32_t *idx, int *count) {
  if (n == 0) return cudaMemsetAsync(count, 0, sizeof(int), h->stream);
  const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb > h->scan_cap) return cudaErrorInvalidValue;
  k_cmp_count<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(n, pred, h->scan_tmp);
  k_scan_spine<<<1, SCAN_BLOCK, 0, h->stream>>>(h->scan_tmp, nb);
  k_cmp_write<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(n, pred, h->scan_tmp, idx, count);
  FG_LAUNCHED(h, 3);
  return cudaGetLastError();
}

} // namespace

cudaError_t compact_flags(FlipGpu *h, const uint8_t *flag, size_t n, uint32_t *idx, int *count) {
  return compact(h, n, PredFlag{flag}, idx, count);
}

cudaError_t compact_deep_water(FlipGpu *h, uint32_t *idx, int *count) {
  return compact(h, h->nc, PredDeepWater{h->n, h->A}, idx, count);
}

cudaError_t scan_exclusive_live(FlipGpu *h, const uint32_t *in, uint32_t *out, size_t n,
                                const int *nlive) {
  if (n == 0) return cudaSuccess;
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb > h->scan_cap) return cudaErrorInvalidValue;
  k_scan_reduce<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(in, n, h->scan_tmp, nlive);
  k_scan_spine<<<1, SCAN_BLOCK, 0, h->stream>>>(h->scan_tmp, nb);
  k_scan_down<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(in, out, n, h->scan_tmp, nlive);
  FG_LAUNCHED(h, 3);
  return cudaGetLastError();
}

cudaError_t scan_exclusive_tmp(FlipGpu *h, const uint32_t *in, uint32_t *out, size_t n,
                               uint32_t *tmp, size_t tmp_blocks) {
  if (n == 0) return cudaSuccess;
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb > tmp_blocks) return cudaErrorInvalidValue;
  k_scan_reduce<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(in, n, tmp, nullptr);
  k_scan_spine<<<1, SCAN_BLOCK, 0, h->stream>>>(tmp, nb);
  k_scan_down<<<(unsigned)nb, SCAN_BLOCK, 0, h->stream>>>(in, out, n, tmp, nullptr);
  FG_LAUNCHED(h, 3);
  return cudaGetLastError();
}

cudaError_t scan_exclusive(FlipGpu *h, const uint32_t *in, uint32_t *out, size_t n) {
  return scan_exclusive_tmp(h, in, out, n, h->scan_tmp, h->scan_cap);
}

size_t scan_tmp_blocks(size_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

cudaError_t launch_payload(FlipGpu *h, int apply_gravity, int fields) {
  SimConst c = make_const(h);
  if (h->np == 0) return cudaSuccess;
  const unsigned g = grid_for(h->np, 256);
  if (h->defer_vel) {
    /* the velocities are still being uploaded (flipgpu_step_host) */
    if (fields & PL_SDENS)
      k_payload_pos<true><<<g, 256, 0, h->stream>>>(c, h->perm, h->px, h->py, h->pz, h->type,
                                                    h->dens, h->spos, h->spg, h->sdens);
    else
      k_payload_pos<false><<<g, 256, 0, h->stream>>>(c, h->perm, h->px, h->py, h->pz, h->type,
                                                     h->dens, h->spos, h->spg, h->sdens);
    FG_LAUNCHED(h, 1);
    h->defer_gravity = apply_gravity;
    return cudaGetLastError();
  }
#define PAYLOAD(F)                                                                            \
  k_payload<F><<<g, 256, 0, h->stream>>>(c, apply_gravity, h->perm, h->px, h->py, h->pz, h->vx, \
                                         h->vy, h->vz, h->type, h->dens, h->spos, h->spg,       \
                                         h->svel, h->sdens)
  if (fields == PL_ALL)
    PAYLOAD(PL_ALL);
  else if (fields == (PL_SPG | PL_SVEL))
    PAYLOAD(PL_SPG | PL_SVEL);
  else if (fields == 0)
    PAYLOAD(0);
  else
    return cudaErrorInvalidValue;
#undef PAYLOAD
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_payload_vel(FlipGpu *h, int apply_gravity) {
  SimConst c = make_const(h);
  if (h->np == 0) return cudaSuccess;
  k_payload_vel<<<grid_for(h->np, 256), 256, 0, h->stream>>>(
      c, apply_gravity, h->perm, h->vx, h->vy, h->vz, h->type, h->svel);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}

cudaError_t launch_sort(FlipGpu *h, int apply_gravity, int fields) {
  SimConst c = make_const(h);
  cudaError_t e = cudaMemsetAsync(h->cell_count, 0, (h->nc + 1) * sizeof(uint32_t), h->stream);
  if (e != cudaSuccess) return e;
  if (h->np > 0) {
    if (h->prm.arith == FLIPGPU_ARITH_FAST)
      k_sort_count<true><<<grid_for(h->np, 256), 256, 0, h->stream>>>(
          c, h->px, h->py, h->pz, h->key, h->rank, h->cell_count);
    else
      k_sort_count<false><<<grid_for(h->np, 256), 256, 0, h->stream>>>(
          c, h->px, h->py, h->pz, h->key, h->rank, h->cell_count);
    FG_LAUNCHED(h, 1);
  }
  /* cell_count has nc+1 entries (last = 0), so cell_start[nc] = np. */
  e = scan_exclusive(h, h->cell_count, h->cell_start, h->nc + 1);
  if (e != cudaSuccess) return e;
  if (h->np > 0) {
    k_sort_scatter<<<grid_for(h->np, 256), 256, 0, h->stream>>>(h->np, h->key, h->rank,
                                                                h->cell_start, h->perm);
    if (h->prm.arith == FLIPGPU_ARITH_FAST)
      k_sort_fixup_halves<<<grid_for(h->nc, 256), 256, 0, h->stream>>>(
          h->nc, h->cell_start, h->perm, h->cell_mid);
    else
      k_sort_fixup<<<grid_for(h->nc, 256), 256, 0, h->stream>>>(h->nc, h->cell_start, h->perm);
    FG_LAUNCHED(h, 2);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_payload(h, apply_gravity, fields);
  h->cells_valid = true;
  h->lists_exist = true;
  return e;
}
