/*
 * k_unet.cu — learned warm start for the pressure solve.
 *
 * A 3D U-Net maps, per cell, (liquid mask, right-hand side b, previous
 * pressure x0) to a correction d of the initial guess; the solve then
 * starts from x0 + g*d, where g minimises the residual over that line
 * (g = (Ad).r0 / (Ad).(Ad) with r0 = b - A x0; or, with
 * FLIPGPU_WARM_STEP=anorm, the A-norm error: g = d.r0 / d.Ad). The line
 * contains x0 (g = 0), so the starting residual is never above the
 * previous-step guess's, and CG still iterates to the same relative
 * residual: the answer is the plain method's answer.
 *
 * Network: 4 levels (16/32/48/64 channels), two 3x3x3 convolutions with
 * ReLU per level and side, 2x2x2 average pooling down, nearest upsampling
 * and channel concatenation up, a 1x1x1 head. Activations are BF16 with
 * the channels of a cell contiguous ([sample][cell][channel], cells
 * x-major like the solver's grids); weights are FP32 masters with BF16
 * copies laid out as tensor-core fragments.
 *
 * Every 3x3x3 convolution is an implicit GEMM on the tensor cores. The
 * forward convolutions run on tcgen05 with TMEM accumulators
 * (k_conv_tc.cu). Backward-data (the same convolution on flipped, transposed
 * weights), weight gradients and the mma.sync forward path (selectable for
 * comparison) use mma.sync m16n8k16 BF16 -> FP32: a block stages a 4x8x8-cell
 * output tile's input halo in shared memory and each warp accumulates 32
 * cells x up to 64 output channels over 27 taps x Cin/16 chunks, loading A
 * fragments with ldmatrix. Weight gradients reduce over
 * cells in fixed-size chunks whose partial sums are added in a fixed order,
 * so training is deterministic. Adam updates the FP32 masters.
 */
#include <cstdlib>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "conv_tc.h"
#include "devcommon.cuh"
#include "flipgpu_impl.h"

typedef __nv_bfloat16 bf16;

namespace {

constexpr int NCONV = 14;
struct ConvSpec {
  int cin, cout, level;
};
/* forward order: 0a 0b 1a 1b 2a 2b 3a 3b 2c 2d 1c 1d 0c 0d */
constexpr ConvSpec kConv[NCONV] = {{16, 16, 0},  {16, 16, 0}, {16, 32, 1}, {32, 32, 1},
                                   {32, 48, 2},  {48, 48, 2}, {48, 64, 3}, {64, 64, 3},
                                   {112, 48, 2}, {48, 48, 2}, {80, 32, 1}, {32, 32, 1},
                                   {48, 16, 0},  {16, 16, 0}};
constexpr int IN_CH = 4; /* real input channels (padded to 16) */

constexpr int TI = 4, TJ = 8, TK = 8, TV = TI * TJ * TK;
constexpr int HI = TI + 2, HJ = TJ + 2, HK = TK + 2, HV = HI * HJ * HK;
constexpr int CTHREADS = 256;
constexpr int EBLK = 256;
constexpr int RB = 256; /* reduction blocks per sample */
constexpr int WG_SUB = 64; /* cells staged per weight-gradient step */

__host__ __device__ inline int tiles_of(int n, int t) { return (n + t - 1) / t; }

/* --------------------------------------------------------------- tensor-core helpers */

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                        uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1,
                                          uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t addr, uint32_t &r0, uint32_t &r1) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float *d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* ------------------------------------------------------------------ convolution */

/* Y[s][v][co] = (relu)(sum_{tap, ci} X[s][v + off(tap)][ci] W[tap][ci][co] + bias[co])
 * over the block's output channels [blockIdx.y*NB, +NB). Cells outside the
 * grid read as zero. frag holds W as B fragments: for (tap, 16-channel chunk
 * c, 8-column tile nt) 32 lanes x {W[2t..2t+1][g], W[2t+8..2t+9][g]}. */
template <int NB>
__global__ void __launch_bounds__(CTHREADS, 1)
    k_conv3(int n, int cin, int cout, const bf16 *__restrict__ X, const uint2 *__restrict__ frag,
            const float *__restrict__ bias, bf16 *__restrict__ Y, int relu) {
  extern __shared__ __align__(16) unsigned char smraw[];
  bf16 *sm = reinterpret_cast<bf16 *>(smraw);
  const int stride = cin + 8; /* bf16 per staged cell (padded against bank conflicts) */
  const int tj_n = tiles_of(n, TJ), tk_n = tiles_of(n, TK);
  const int tile = blockIdx.x;
  const int i0 = (tile / (tj_n * tk_n)) * TI, j0 = ((tile / tk_n) % tj_n) * TJ,
            k0 = (tile % tk_n) * TK;
  const size_t n3 = (size_t)n * n * n;
  const bf16 *Xs = X + (size_t)blockIdx.z * n3 * cin;
  /* stage the halo */
  const int q8 = cin / 8;
  for (int idx = threadIdx.x; idx < HV * q8; idx += CTHREADS) {
    const int hv = idx / q8, q = idx % q8;
    const int hi = hv / (HJ * HK), hj = (hv / HK) % HJ, hk = hv % HK;
    const int gi = i0 - 1 + hi, gj = j0 - 1 + hj, gk = k0 - 1 + hk;
    uint4 val = make_uint4(0, 0, 0, 0);
    if (gi >= 0 && gi < n && gj >= 0 && gj < n && gk >= 0 && gk < n)
      val = *reinterpret_cast<const uint4 *>(Xs + (((size_t)gi * n + gj) * n + gk) * cin + q * 8);
    *reinterpret_cast<uint4 *>(sm + hv * stride + q * 8) = val;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  constexpr int NT = NB / 8;
  float acc[2][NT][4];
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int j = 0; j < NT; j++) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
  /* the halo cell each lane addresses for its ldmatrix row, per m-tile */
  int base_row[2];
#pragma unroll
  for (int m = 0; m < 2; m++) {
    const int e = (warp * 2 + m) * 16 + (lane & 15);
    const int ei = e / (TJ * TK), ej = (e / TK) % TJ, ek = e % TK;
    base_row[m] = (ei * HJ + ej) * HK + ek;
  }
  const uint32_t sbase = smem_u32(sm) + (uint32_t)((lane >> 4) * 16);
  const int nchunk = cin / 16, ntile_all = cout / 8;
  const int nt0 = blockIdx.y * NT;
  for (int tap = 0; tap < 27; tap++) {
    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
    const int toff = (dz * HJ + dy) * HK + dx;
    for (int c = 0; c < nchunk; c++) {
      uint32_t a[2][4];
#pragma unroll
      for (int m = 0; m < 2; m++)
        ldsm_x4(sbase + (uint32_t)(((base_row[m] + toff) * stride + c * 16) * 2), a[m][0], a[m][1],
                a[m][2], a[m][3]);
      const uint2 *fb = frag + ((size_t)(tap * nchunk + c) * ntile_all + nt0) * 32 + lane;
#pragma unroll
      for (int j = 0; j < NT; j++) {
        const uint2 b = __ldg(fb + j * 32);
        mma_bf16(acc[0][j], a[0][0], a[0][1], a[0][2], a[0][3], b.x, b.y);
        mma_bf16(acc[1][j], a[1][0], a[1][1], a[1][2], a[1][3], b.x, b.y);
      }
    }
  }
  bf16 *Ys = Y + (size_t)blockIdx.z * n3 * cout;
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int e = (warp * 2 + m) * 16 + g + h * 8;
      const int gi = i0 + e / (TJ * TK), gj = j0 + (e / TK) % TJ, gk = k0 + e % TK;
      if (gi >= n || gj >= n || gk >= n) continue;
      bf16 *yrow = Ys + (((size_t)gi * n + gj) * n + gk) * cout;
#pragma unroll
      for (int j = 0; j < NT; j++) {
        const int co = (nt0 + j) * 8 + 2 * t;
        float v0 = acc[m][j][2 * h], v1 = acc[m][j][2 * h + 1];
        if (bias) {
          v0 += bias[co];
          v1 += bias[co + 1];
        }
        if (relu) {
          v0 = fmaxf(v0, 0.0f);
          v1 = fmaxf(v1, 0.0f);
        }
        *reinterpret_cast<__nv_bfloat162 *>(yrow + co) = __floats2bfloat162_rn(v0, v1);
      }
    }
}

/* Weight gradient of one tap over one chunk of cells:
 * part[chunk][tap][ci][co] = sum_{v in chunk} X[v + off(tap)][ci] dZ[v][co],
 * and for the centre tap the bias gradient part_b[chunk][co] = sum dZ[v][co].
 * GEMM with M = ci, N = co, K = cells: A = X^T and B = dZ come from shared
 * memory through transposing ldmatrix. Each warp owns 16x8 output tiles
 * w, w+8, ... */
__global__ void __launch_bounds__(CTHREADS)
    k_wgrad(int n, int cin, int cout, int cps, int ch, const bf16 *__restrict__ X,
            const bf16 *__restrict__ dZ, float *__restrict__ part, float *__restrict__ part_b) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int xs = cin + 8, zs = cout + 8;
  bf16 *sx = reinterpret_cast<bf16 *>(smraw);
  bf16 *sz = sx + WG_SUB * xs;
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const size_t n3 = (size_t)n * n * n;
  /* chunk blockIdx.x: sample s, cells [cb, cb + chunk_cells) of that sample */
  const size_t s = blockIdx.x / cps;
  const size_t cb = (size_t)(blockIdx.x % cps) * ch;
  const int chunk_cells = (int)((cb + ch <= n3) ? ch : n3 - cb);
  const size_t c0 = s * n3 + cb; /* flat cell over the batch */
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt_n = cin / 16, nt_n = cout / 8, tiles = mt_n * nt_n;
  constexpr int MAXT = 7; /* 112/16 x 64/8 = 56 tiles over 8 warps */
  float acc[MAXT][4];
#pragma unroll
  for (int q = 0; q < MAXT; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
  float bsum = 0.0f;
  const bool centre = tap == 13;
  for (int sub = 0; sub < chunk_cells; sub += WG_SUB) {
    __syncthreads();
    /* stage X at the shifted cells and dZ at the cells */
    for (int idx = threadIdx.x; idx < WG_SUB * (cin / 8); idx += CTHREADS) {
      const int r = idx / (cin / 8), q = idx % (cin / 8);
      uint4 val = make_uint4(0, 0, 0, 0);
      if (sub + r < chunk_cells) {
        const size_t v = (c0 + sub + r) - s * n3;
        const int i = (int)(v / ((size_t)n * n)) + dz, j = (int)((v / n) % n) + dy,
                  k = (int)(v % n) + dx;
        if (i >= 0 && i < n && j >= 0 && j < n && k >= 0 && k < n)
          val = *reinterpret_cast<const uint4 *>(
              X + (s * n3 + ((size_t)i * n + j) * n + k) * cin + q * 8);
      }
      *reinterpret_cast<uint4 *>(sx + r * xs + q * 8) = val;
    }
    for (int idx = threadIdx.x; idx < WG_SUB * (cout / 8); idx += CTHREADS) {
      const int r = idx / (cout / 8), q = idx % (cout / 8);
      uint4 val = make_uint4(0, 0, 0, 0);
      if (sub + r < chunk_cells)
        val = *reinterpret_cast<const uint4 *>(dZ + (c0 + sub + r) * cout + q * 8);
      *reinterpret_cast<uint4 *>(sz + r * zs + q * 8) = val;
    }
    __syncthreads();
    if (centre && threadIdx.x < cout)
      for (int r = 0; r < WG_SUB; r++) bsum += __bfloat162float(sz[r * zs + threadIdx.x]);
    for (int kk = 0; kk < WG_SUB; kk += 16) {
#pragma unroll
      for (int q = 0; q < MAXT; q++) {
        const int tile = warp + q * 8;
        if (tile >= tiles) break;
        const int mi = tile / nt_n, ni = tile % nt_n;
        uint32_t a0, a1, a2, a3, b0, b1;
        const int vr = (lane & 7) + (lane >> 4) * 8, cio = ((lane >> 3) & 1) * 8;
        ldsm_x4_t(smem_u32(sx + (kk + vr) * xs + mi * 16 + cio), a0, a1, a2, a3);
        const int vb = (lane & 7) + ((lane >> 3) & 1) * 8;
        ldsm_x2_t(smem_u32(sz + (kk + vb) * zs + ni * 8), b0, b1);
        mma_bf16(acc[q], a0, a1, a2, a3, b0, b1);
      }
    }
  }
  const int g = lane >> 2, t = lane & 3;
  float *dst = part + ((size_t)blockIdx.x * 27 + tap) * cin * cout;
#pragma unroll
  for (int q = 0; q < MAXT; q++) {
    const int tile = warp + q * 8;
    if (tile >= tiles) break;
    const int mi = tile / nt_n, ni = tile % nt_n;
    const int ci = mi * 16 + g, co = ni * 8 + 2 * t;
    dst[ci * cout + co] = acc[q][0];
    dst[ci * cout + co + 1] = acc[q][1];
    dst[(ci + 8) * cout + co] = acc[q][2];
    dst[(ci + 8) * cout + co + 1] = acc[q][3];
  }
  if (centre && threadIdx.x < cout) part_b[(size_t)blockIdx.x * cout + threadIdx.x] = bsum;
}

/* grad W[tap][ci][co] = sum over chunks in order; grad b likewise */
__global__ void k_wgrad_reduce(int nchunks, int wcount, int cout, const float *__restrict__ part,
                               const float *__restrict__ part_b, float *__restrict__ gw,
                               float *__restrict__ gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < wcount) {
    float s = 0.0f;
    for (int c = 0; c < nchunks; c++) s += part[(size_t)c * wcount + i];
    gw[i] = s;
  } else if (i < wcount + cout) {
    const int co = i - wcount;
    float s = 0.0f;
    for (int c = 0; c < nchunks; c++) s += part_b[(size_t)c * cout + co];
    gb[co] = s;
  }
}

/* ------------------------------------------------------------------ elementwise */

/* per sample and block: sums over liquid cells of b^2, r0^2, x0^2 and the
 * liquid count; each thread sums its cells in FP32 (FP64 arithmetic is a
 * small fraction of FP32's on this GPU), the block tree is FP64 */
__global__ void k_sample_sums(size_t n3, const uint8_t *__restrict__ A, const float *__restrict__ b,
                              const float *__restrict__ r0, const float *__restrict__ x0,
                              double *__restrict__ part) {
  __shared__ double sh[EBLK][4];
  const size_t s = blockIdx.y;
  float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  for (size_t v = (size_t)blockIdx.x * EBLK + threadIdx.x; v < n3; v += (size_t)RB * EBLK) {
    const size_t i = s * n3 + v;
    if (A[i] != CELL_FLUID) continue;
    const float bb = b[i], rr = r0[i], xx = x0[i];
    a[0] = fmaf(bb, bb, a[0]);
    a[1] = fmaf(rr, rr, a[1]);
    a[2] = fmaf(xx, xx, a[2]);
    a[3] += 1.0f;
  }
  for (int q = 0; q < 4; q++) sh[threadIdx.x][q] = (double)a[q];
  __syncthreads();
  for (int w = EBLK / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 4; q++) sh[threadIdx.x][q] += sh[threadIdx.x + w][q];
    __syncthreads();
  }
  if (threadIdx.x < 4) part[4 * (s * RB + blockIdx.x) + threadIdx.x] = sh[0][threadIdx.x];
}

/* per sample: RMS over the liquid of b, r0 and x0 (1 where zero), and the
 * target scale s_r h^2 (the size of A^-1 r0 for a residual of RMS s_r);
 * scale[4s + 0..3] = {s_b, s_r, s_x, s_t} */
__global__ void k_sample_scale(int batch, int n, const double *__restrict__ part,
                               float *__restrict__ scale, double *__restrict__ count) {
  /* block s: a fixed tree over the RB block partials of sample s */
  __shared__ double sh[RB][4];
  const int s = blockIdx.x;
  for (int q = 0; q < 4; q++) sh[threadIdx.x][q] = part[4 * (s * RB + threadIdx.x) + q];
  __syncthreads();
  for (int w = RB / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 4; q++) sh[threadIdx.x][q] += sh[threadIdx.x + w][q];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double c = sh[0][3];
  double rms[3];
  for (int q = 0; q < 3; q++) rms[q] = (c > 0.0 && sh[0][q] > 0.0) ? sqrt(sh[0][q] / c) : 1.0;
  scale[4 * s + 0] = (float)rms[0];
  scale[4 * s + 1] = (float)rms[1];
  scale[4 * s + 2] = (float)rms[2];
  scale[4 * s + 3] = (float)(rms[1] / ((double)n * n));
  count[s] = c;
}

/* input channels: liquid mask, r0/s_r, b/s_b, x0/s_x (zero off the liquid),
 * the rest zero */
__global__ void k_features(size_t n3, int batch, const uint8_t *__restrict__ A,
                           const float *__restrict__ b, const float *__restrict__ r0,
                           const float *__restrict__ x0, const float *__restrict__ scale,
                           bf16 *__restrict__ X0) {
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= n3 * batch) return;
  const size_t s = idx / n3;
  const bool fl = A[idx] == CELL_FLUID;
  __align__(16) bf16 row[16];
  row[0] = __float2bfloat16(fl ? 1.0f : 0.0f);
  row[1] = __float2bfloat16(fl ? r0[idx] / scale[4 * s + 1] : 0.0f);
  row[2] = __float2bfloat16(fl ? b[idx] / scale[4 * s + 0] : 0.0f);
  row[3] = __float2bfloat16(fl ? x0[idx] / scale[4 * s + 2] : 0.0f);
#pragma unroll
  for (int c = 4; c < 16; c++) row[c] = __float2bfloat16(0.0f);
  uint4 *dst = reinterpret_cast<uint4 *>(X0 + idx * 16);
  dst[0] = reinterpret_cast<uint4 *>(row)[0];
  dst[1] = reinterpret_cast<uint4 *>(row)[1];
}

/* 2x2x2 average: coarse cell p of an n/2 grid from its eight children */
__global__ void k_pool(int nc_, int C, int batch, const bf16 *__restrict__ X, bf16 *__restrict__ P) {
  const int n = 2 * nc_;
  const size_t nc3 = (size_t)nc_ * nc_ * nc_, n3 = (size_t)n * n * n;
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  const size_t total = nc3 * batch * (C / 2);
  if (idx >= total) return;
  const int cp = (int)(idx % (C / 2));
  const size_t pc = idx / (C / 2);
  const size_t s = pc / nc3, p = pc % nc3;
  const int I = (int)(p / ((size_t)nc_ * nc_)), J = (int)((p / nc_) % nc_), K = (int)(p % nc_);
  float a = 0.0f, bb = 0.0f;
  for (int q = 0; q < 8; q++) {
    const int i = 2 * I + (q >> 2), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q & 1);
    const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(
        X + (s * n3 + ((size_t)i * n + j) * n + k) * C + 2 * cp);
    a += __bfloat162float(v.x);
    bb += __bfloat162float(v.y);
  }
  *reinterpret_cast<__nv_bfloat162 *>(P + (s * nc3 + p) * C + 2 * cp) =
      __floats2bfloat162_rn(a * 0.125f, bb * 0.125f);
}

/* dX[child][c] = dP[parent][c]/8 + skip[child][c] (skip: a channel slice of
 * width C at offset off in rows of width ws; null for none) */
__global__ void k_pool_bwd(int n, int C, int batch, const bf16 *__restrict__ dP,
                           const bf16 *__restrict__ skip, int ws, int off, bf16 *__restrict__ dX) {
  const int nc_ = n / 2;
  const size_t n3 = (size_t)n * n * n, nc3 = (size_t)nc_ * nc_ * nc_;
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= n3 * batch * C) return;
  const int c = (int)(idx % C);
  const size_t vc = idx / C;
  const size_t s = vc / n3, v = vc % n3;
  const int i = (int)(v / ((size_t)n * n)), j = (int)((v / n) % n), k = (int)(v % n);
  const size_t p = ((size_t)(i / 2) * nc_ + j / 2) * nc_ + k / 2;
  float g = __bfloat162float(dP[(s * nc3 + p) * C + c]) * 0.125f;
  if (skip) g += __bfloat162float(skip[(s * n3 + v) * ws + off + c]);
  dX[idx] = __float2bfloat16(g);
}

/* U[v] = [coarse[parent(v)] (C1) | skip[v] (C2)]; one thread per 8 channels
 * of a cell, 32-bit index arithmetic (n^3 * batch * C/8 < 2^32) */
__global__ void k_up_cat(int n, int C1, int C2, int batch, const bf16 *__restrict__ coarse,
                         const bf16 *__restrict__ skip, bf16 *__restrict__ U) {
  const unsigned nc_ = (unsigned)n / 2, C = (unsigned)(C1 + C2), C8 = C / 8, un = (unsigned)n;
  const unsigned n3 = un * un * un, nc3 = nc_ * nc_ * nc_;
  const unsigned idx = blockIdx.x * EBLK + threadIdx.x;
  if (idx >= n3 * (unsigned)batch * C8) return;
  const unsigned q = idx % C8, vc = idx / C8;
  const unsigned s = vc / n3, v = vc - s * n3;
  uint4 val;
  if (q * 8 < (unsigned)C1) {
    const unsigned k = v % un, t = v / un, j = t % un, i = t / un;
    const unsigned p = ((i / 2) * nc_ + j / 2) * nc_ + k / 2;
    val = *reinterpret_cast<const uint4 *>(coarse + ((size_t)s * nc3 + p) * C1 + q * 8);
  } else {
    val = *reinterpret_cast<const uint4 *>(skip + ((size_t)s * n3 + v) * C2 + (q * 8 - C1));
  }
  *reinterpret_cast<uint4 *>(U + ((size_t)s * n3 + v) * C + q * 8) = val;
}

/* dCoarse[p][c] = sum over the eight children of dU[child][c], c < C1 */
__global__ void k_up_bwd(int n, int C1, int C, int batch, const bf16 *__restrict__ dU,
                         bf16 *__restrict__ dC) {
  const int nc_ = n / 2;
  const size_t n3 = (size_t)n * n * n, nc3 = (size_t)nc_ * nc_ * nc_;
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= nc3 * batch * C1) return;
  const int c = (int)(idx % C1);
  const size_t pc = idx / C1;
  const size_t s = pc / nc3, p = pc % nc3;
  const int I = (int)(p / ((size_t)nc_ * nc_)), J = (int)((p / nc_) % nc_), K = (int)(p % nc_);
  float a = 0.0f;
  for (int q = 0; q < 8; q++) {
    const int i = 2 * I + (q >> 2), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q & 1);
    a += __bfloat162float(dU[(s * n3 + ((size_t)i * n + j) * n + k) * C + c]);
  }
  dC[idx] = __float2bfloat16(a);
}

/* dst[v][c] = src[v][off + c], c < width (rows of ws channels), 8 per thread */
__global__ void k_slice(size_t cells, int ws, int off, int width, const bf16 *__restrict__ src,
                        bf16 *__restrict__ dst) {
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  const int q8 = width / 8;
  if (idx >= cells * q8) return;
  const size_t v = idx / q8;
  const int q = (int)(idx % q8);
  *reinterpret_cast<uint4 *>(dst + v * width + q * 8) =
      *reinterpret_cast<const uint4 *>(src + v * ws + off + q * 8);
}

/* dZ = dY where Y > 0 (ReLU backward), 8 channels per thread */
__global__ void k_relu_bwd(size_t count8, const bf16 *__restrict__ dY, const bf16 *__restrict__ Y,
                           bf16 *__restrict__ dZ) {
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= count8) return;
  uint4 gy = reinterpret_cast<const uint4 *>(dY)[idx];
  const uint4 yy = reinterpret_cast<const uint4 *>(Y)[idx];
  const bf16 *y = reinterpret_cast<const bf16 *>(&yy);
  bf16 *d = reinterpret_cast<bf16 *>(&gy);
#pragma unroll
  for (int c = 0; c < 8; c++)
    if (!(__bfloat162float(y[c]) > 0.0f)) d[c] = __float2bfloat16(0.0f);
  reinterpret_cast<uint4 *>(dZ)[idx] = gy;
}

/* head: O[v] = sum_c D[v][c] wh[c] + bh (FP32) */
__global__ void k_head(size_t cells, const bf16 *__restrict__ D, const float *__restrict__ wh,
                       float *__restrict__ O) {
  const size_t v = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (v >= cells) return;
  float a = wh[16];
  const bf16 *d = D + v * 16;
#pragma unroll
  for (int c = 0; c < 16; c++) a += __bfloat162float(d[c]) * wh[c];
  O[v] = a;
}

/* loss = sum over liquid cells of (O - T)^2 / count, T = (x - x0)/scale;
 * dO = 2 (O - T) / count on liquid cells; dD[v][c] = dO wh[c]; partial
 * sums of the loss and of the head's gradients per block */
__global__ void k_loss_head_bwd(size_t n3, int batch, const uint8_t *__restrict__ A,
                                const float *__restrict__ x, const float *__restrict__ x0,
                                const float *__restrict__ scale, double inv_count,
                                const float *__restrict__ O, const bf16 *__restrict__ D,
                                const float *__restrict__ wh, bf16 *__restrict__ dD,
                                double *__restrict__ part) {
  __shared__ double sh[EBLK][18];
  const size_t v = (size_t)blockIdx.x * EBLK + threadIdx.x;
  double l = 0.0, gw[17];
#pragma unroll
  for (int c = 0; c < 17; c++) gw[c] = 0.0;
  if (v < n3 * batch) {
    const size_t s = v / n3;
    float g = 0.0f;
    if (A[v] == CELL_FLUID) {
      const float T = (x[v] - x0[v]) / scale[4 * s + 3];
      const float e = O[v] - T;
      l = (double)e * e * inv_count;
      g = (float)(2.0 * e * inv_count);
    }
    const bf16 *d = D + v * 16;
    __align__(16) bf16 row[16];
#pragma unroll
    for (int c = 0; c < 16; c++) {
      row[c] = __float2bfloat16(g * wh[c]);
      gw[c] = (double)g * __bfloat162float(d[c]);
    }
    gw[16] = g;
    uint4 *dst = reinterpret_cast<uint4 *>(dD + v * 16);
    dst[0] = reinterpret_cast<uint4 *>(row)[0];
    dst[1] = reinterpret_cast<uint4 *>(row)[1];
  }
  sh[threadIdx.x][0] = l;
#pragma unroll
  for (int c = 0; c < 17; c++) sh[threadIdx.x][c + 1] = gw[c];
  __syncthreads();
  for (int w = EBLK / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 18; c++) sh[threadIdx.x][c] += sh[threadIdx.x + w][c];
    __syncthreads();
  }
  if (threadIdx.x < 18) part[(size_t)blockIdx.x * 18 + threadIdx.x] = sh[0][threadIdx.x];
}

__global__ void k_head_reduce(int nblocks, const double *__restrict__ part, float *__restrict__ gh,
                              double *__restrict__ loss) {
  const int c = threadIdx.x;
  if (c >= 18) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; b++) s += part[(size_t)b * 18 + c];
  if (c == 0) *loss = s;
  else gh[c - 1] = (float)s;
}

/* out = scale_x * O (the correction in pressure units), zero off the liquid */
__global__ void k_delta_out(size_t n3, int batch, const uint8_t *__restrict__ A,
                            const float *__restrict__ O, const float *__restrict__ scale,
                            float *__restrict__ delta) {
  const size_t v = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (v >= n3 * batch) return;
  delta[v] = A[v] == CELL_FLUID ? O[v] * scale[4 * (v / n3) + 3] : 0.0f;
}

/* Coarsened warm start: the network runs on the grid pooled c times
 * (factor f = 2^c per axis). Training targets on that grid: per coarse
 * cell, the liquid flag (any liquid child) and the averages of x and x0
 * over its liquid children. */
__global__ void k_pool_target(int nc_, int f, int batch, const uint8_t *__restrict__ A,
                              const float *__restrict__ x, const float *__restrict__ x0,
                              uint8_t *__restrict__ Ac, float *__restrict__ xc,
                              float *__restrict__ x0c) {
  const size_t nc3 = (size_t)nc_ * nc_ * nc_;
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= nc3 * batch) return;
  const int n = nc_ * f;
  const size_t s = idx / nc3, p = idx % nc3, n3 = (size_t)n * n * n;
  const int I = (int)(p / ((size_t)nc_ * nc_)), J = (int)((p / nc_) % nc_), K = (int)(p % nc_);
  int cnt = 0;
  float sx = 0.0f, sx0 = 0.0f;
  for (int a = 0; a < f; a++)
    for (int b = 0; b < f; b++)
      for (int c = 0; c < f; c++) {
        const size_t v = s * n3 + ((size_t)(I * f + a) * n + (J * f + b)) * n + (K * f + c);
        if (A[v] != CELL_FLUID) continue;
        cnt++;
        sx += x[v];
        sx0 += x0[v];
      }
  Ac[idx] = cnt ? (uint8_t)CELL_FLUID : (uint8_t)0;
  xc[idx] = cnt ? sx / (float)cnt : 0.0f;
  x0c[idx] = cnt ? sx0 / (float)cnt : 0.0f;
}

/* count[s] = liquid cells of sample s (integer-valued, so the atomic
 * double sums are exact and order-independent) */
__global__ void k_count_fluid(size_t n3, const uint8_t *__restrict__ A, double *__restrict__ count) {
  __shared__ int sh[EBLK];
  const size_t s = blockIdx.y;
  int c = 0;
  for (size_t v = (size_t)blockIdx.x * EBLK + threadIdx.x; v < n3; v += (size_t)gridDim.x * EBLK)
    c += A[s * n3 + v] == CELL_FLUID;
  sh[threadIdx.x] = c;
  __syncthreads();
  for (int w = EBLK / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0 && sh[0]) atomicAdd(count + s, (double)sh[0]);
}

/* trilinear prolongation of a cell-centred field from nc^3 to (nc f)^3,
 * clamped at the boundary */
__global__ void k_prolong(int nc_, int f, int batch, const float *__restrict__ O,
                          float *__restrict__ Of) {
  const int n = nc_ * f;
  const size_t n3 = (size_t)n * n * n, nc3 = (size_t)nc_ * nc_ * nc_;
  const size_t idx = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (idx >= n3 * batch) return;
  const size_t s = idx / n3, v = idx % n3;
  const int ii[3] = {(int)(v / ((size_t)n * n)), (int)((v / n) % n), (int)(v % n)};
  int lo[3], hi[3];
  float w[3];
  for (int d = 0; d < 3; d++) {
    const float xc = ((float)ii[d] + 0.5f) / (float)f - 0.5f;
    const float fl = floorf(xc);
    w[d] = xc - fl;
    lo[d] = min(max((int)fl, 0), nc_ - 1);
    hi[d] = min(max((int)fl + 1, 0), nc_ - 1);
  }
  const float *o = O + s * nc3;
  float acc = 0.0f;
  for (int q = 0; q < 8; q++) {
    const int a = (q >> 2) & 1, b = (q >> 1) & 1, c = q & 1;
    const float wt = (a ? w[0] : 1.0f - w[0]) * (b ? w[1] : 1.0f - w[1]) * (c ? w[2] : 1.0f - w[2]);
    acc += wt * o[((size_t)(a ? hi[0] : lo[0]) * nc_ + (b ? hi[1] : lo[1])) * nc_ +
                  (c ? hi[2] : lo[2])];
  }
  Of[idx] = acc;
}

/* BF16 fragments of W (fwd) and of the flipped, transposed W (bwd-data). */
__global__ void k_pack(int cin, int cout, const float *__restrict__ W, uint2 *__restrict__ ffwd,
                       uint2 *__restrict__ fbwd) {
  const int nfw = 27 * (cin / 16) * (cout / 8) * 32;
  const int nbw = 27 * (cout / 16) * (cin / 8) * 32;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  auto pack2 = [](float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
  };
  if (idx < nfw) {
    const int lane = idx % 32, rest = idx / 32;
    const int nt = rest % (cout / 8), c = (rest / (cout / 8)) % (cin / 16),
              tap = rest / ((cout / 8) * (cin / 16));
    const int g = lane >> 2, t = lane & 3;
    const int co = nt * 8 + g, ci = c * 16 + 2 * t;
    auto w = [&](int ci_) { return W[((size_t)tap * cin + ci_) * cout + co]; };
    ffwd[idx] = make_uint2(pack2(w(ci), w(ci + 1)), pack2(w(ci + 8), w(ci + 9)));
  } else if (fbwd && idx < nfw + nbw) {
    const int j = idx - nfw;
    const int lane = j % 32, rest = j / 32;
    /* convolution with Cin' = cout, Cout' = cin, tap' = 26 - tap */
    const int nt = rest % (cin / 8), c = (rest / (cin / 8)) % (cout / 16),
              tapb = rest / ((cin / 8) * (cout / 16));
    const int tap = 26 - tapb;
    const int g = lane >> 2, t = lane & 3;
    const int ci = nt * 8 + g, co = c * 16 + 2 * t;
    auto w = [&](int co_) { return W[((size_t)tap * cin + ci) * cout + co_]; };
    fbwd[j] = make_uint2(pack2(w(co), w(co + 1)), pack2(w(co + 8), w(co + 9)));
  }
}

__global__ void k_adam(size_t count, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const size_t i = (size_t)blockIdx.x * EBLK + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

/* ------------------------------------------------------------------ warm start */

/* FAST-mode matvec (the solver's): (diag x - sum of liquid neighbours) / h^2 */
__global__ void k_wm_matvec(int n, float inv_h2, const uint8_t *__restrict__ A,
                            const float *__restrict__ diag, const float *__restrict__ x,
                            float *__restrict__ out) {
  const size_t c = (size_t)blockIdx.x * EBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  if (A[c] != CELL_FLUID) {
    out[c] = 0.0f;
    return;
  }
  const int i = (int)(c / ((size_t)n * n)), j = (int)((c / n) % n), k = (int)(c % n);
  float acc = diag[c] * x[c];
  const size_t sj = n, si = (size_t)n * n;
  if (i + 1 < n && A[c + si] == CELL_FLUID) acc -= x[c + si];
  if (i > 0 && A[c - si] == CELL_FLUID) acc -= x[c - si];
  if (j + 1 < n && A[c + sj] == CELL_FLUID) acc -= x[c + sj];
  if (j > 0 && A[c - sj] == CELL_FLUID) acc -= x[c - sj];
  if (k + 1 < n && A[c + 1] == CELL_FLUID) acc -= x[c + 1];
  if (k > 0 && A[c - 1] == CELL_FLUID) acc -= x[c - 1];
  out[c] = acc * inv_h2;
}

/* r0 = b - A x0 on the liquid (zero elsewhere) */
__global__ void k_wm_residual(int n, float inv_h2, const uint8_t *__restrict__ A,
                              const float *__restrict__ diag, const float *__restrict__ b,
                              const float *__restrict__ x, float *__restrict__ r) {
  const size_t c = (size_t)blockIdx.x * EBLK + threadIdx.x;
  const size_t nc = (size_t)n * n * n;
  if (c >= nc) return;
  if (A[c] != CELL_FLUID) {
    r[c] = 0.0f;
    return;
  }
  const int i = (int)(c / ((size_t)n * n)), j = (int)((c / n) % n), k = (int)(c % n);
  float acc = diag[c] * x[c];
  const size_t sj = n, si = (size_t)n * n;
  if (i + 1 < n && A[c + si] == CELL_FLUID) acc -= x[c + si];
  if (i > 0 && A[c - si] == CELL_FLUID) acc -= x[c - si];
  if (j + 1 < n && A[c + sj] == CELL_FLUID) acc -= x[c + sj];
  if (j > 0 && A[c - sj] == CELL_FLUID) acc -= x[c - sj];
  if (k + 1 < n && A[c + 1] == CELL_FLUID) acc -= x[c + 1];
  if (k > 0 && A[c - 1] == CELL_FLUID) acc -= x[c - 1];
  r[c] = b[c] - acc * inv_h2;
}

/* partial sums over liquid cells: d.r, d.w, r.r, r.w, w.w with r = r0 */
__global__ void k_wm_dots(size_t nc, const uint8_t *__restrict__ A, const float *__restrict__ r0,
                          const float *__restrict__ d, const float *__restrict__ w,
                          double *__restrict__ part) {
  __shared__ double sh[EBLK][5];
  double a[5] = {0, 0, 0, 0, 0};
  for (size_t c = (size_t)blockIdx.x * EBLK + threadIdx.x; c < nc; c += (size_t)RB * EBLK) {
    if (A[c] != CELL_FLUID) continue;
    const double r = r0[c];
    const double dd = d[c], ww = w[c];
    a[0] += dd * r;
    a[1] += dd * ww;
    a[2] += r * r;
    a[3] += r * ww;
    a[4] += ww * ww;
  }
  for (int q = 0; q < 5; q++) sh[threadIdx.x][q] = a[q];
  __syncthreads();
  for (int s = EBLK / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < 5; q++) sh[threadIdx.x][q] += sh[threadIdx.x + s][q];
    __syncthreads();
  }
  if (threadIdx.x < 5) part[blockIdx.x * 5 + threadIdx.x] = sh[0][threadIdx.x];
}

/* minres: g = r.w / w.w, the step along d that minimises the residual
 * ||r0 - g A d|| (never above ||r0||); else g = d.r / d.w, the step that
 * minimises the A-norm error. 0 when not finite. x0 += g d; res = the
 * squared residual norms before and after */
__global__ void k_wm_apply(size_t nc, const uint8_t *__restrict__ A, const double *__restrict__ part,
                           const float *__restrict__ d, float *__restrict__ x0,
                           double *__restrict__ res, int minres) {
  __shared__ double tot[5];
  if (threadIdx.x < 5) {
    double s = 0.0;
    for (int b = 0; b < RB; b++) s += part[b * 5 + threadIdx.x];
    tot[threadIdx.x] = s;
  }
  __syncthreads();
  double g = 0.0;
  if (minres) {
    if (tot[4] > 0.0 && isfinite(tot[3] / tot[4])) g = tot[3] / tot[4];
  } else if (tot[1] > 0.0 && isfinite(tot[0] / tot[1])) {
    g = tot[0] / tot[1];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    res[0] = tot[2];
    res[1] = tot[2] - 2.0 * g * tot[3] + g * g * tot[4];
    res[2] = g;
  }
  const float gf = (float)g;
  for (size_t c = (size_t)blockIdx.x * EBLK + threadIdx.x; c < nc; c += (size_t)gridDim.x * EBLK)
    if (A[c] == CELL_FLUID) x0[c] += gf * d[c];
}

} // namespace

/* ====================================================================== host side */

struct FlipUNet {
  cudaStream_t stream = nullptr;
  int64_t nparam = 0;
  int64_t woff[NCONV], boff[NCONV], hoff = 0; /* offsets in the parameter vector */
  float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
  uint2 *ffrag[NCONV] = {}, *bfrag[NCONV] = {};
  bf16 *tcw[NCONV] = {};  /* weights in the tcgen05 B-operand layout */
  int tc = 1;             /* forward convolutions on tcgen05 where they fit */
  int coarse = 0;         /* the network runs on the grid pooled this many times */
  int *tc_err = nullptr;
  int64_t adam_t = 0;
  bool frags_fresh = false;
  /* workspace */
  int ws_n = 0, ws_b = 0;
  bf16 *X0 = nullptr, *A0 = nullptr, *E0 = nullptr, *P1 = nullptr, *A1 = nullptr, *E1 = nullptr,
       *P2 = nullptr, *A2 = nullptr, *E2 = nullptr, *P3 = nullptr, *A3 = nullptr, *E3 = nullptr,
       *U2 = nullptr, *B2 = nullptr, *D2 = nullptr, *U1 = nullptr, *B1 = nullptr, *D1 = nullptr,
       *U0 = nullptr, *B0 = nullptr, *D0 = nullptr;
  bf16 *G1 = nullptr, *G2 = nullptr, *G3 = nullptr, *S0 = nullptr, *S1 = nullptr, *S2 = nullptr;
  float *O = nullptr, *scale = nullptr;
  double *red = nullptr, *count = nullptr, *loss = nullptr;
  float *part = nullptr, *part_b = nullptr;
  size_t part_cap = 0, partb_cap = 0;
  double *hpart = nullptr;
  size_t hpart_cap = 0;
  /* fine-grid buffers of the coarsened warm start */
  int fw_n = 0, fw_b = 0;
  bf16 *XF = nullptr, *XP = nullptr; /* fine features, one pooling step */
  uint8_t *Ac = nullptr;
  float *xc = nullptr, *x0c = nullptr, *Of = nullptr;
  char err[256] = {};
};

namespace {

#define UCK(x)                                                              \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) {                                                \
      snprintf(u->err, sizeof u->err, "%s: %s", #x, cudaGetErrorString(e_)); \
      return FLIPGPU_ECUDA;                                                 \
    }                                                                       \
  } while (0)

template <class T> cudaError_t ualloc(T *&p, size_t n) {
  if (p) cudaFree(p);
  p = nullptr;
  return cudaMalloc(&p, (n ? n : 1) * sizeof(T));
}

size_t conv_smem(int cin) { return (size_t)HV * (cin + 8) * sizeof(bf16); }
size_t wgrad_smem(int cin, int cout) {
  return (size_t)WG_SUB * ((cin + 8) + (cout + 8)) * sizeof(bf16);
}

int unet_init_device() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  const int big = (int)conv_smem(112);
  if (cudaFuncSetAttribute(k_conv3<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ||
      cudaFuncSetAttribute(k_conv3<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ||
      cudaFuncSetAttribute(k_conv3<48>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ||
      cudaFuncSetAttribute(k_conv3<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ||
      conv_tc_init_device() != 0)
    return -1;
  done[dev] = true;
  return 0;
}

/* conv with output-channel blocks of up to 64 */
cudaError_t conv(FlipUNet *u, int n, int batch, int cin, int cout, const bf16 *X, const uint2 *frag,
                 const float *bias, bf16 *Y, int relu) {
  const int tiles = tiles_of(n, TI) * tiles_of(n, TJ) * tiles_of(n, TK);
  const size_t smem = conv_smem(cin);
  const int nb = (cout % 64 == 0) ? 64 : (cout % 48 == 0) ? 48 : (cout % 32 == 0) ? 32 : 16;
  dim3 grid(tiles, cout / nb, batch);
  switch (nb) {
  case 64: k_conv3<64><<<grid, CTHREADS, smem, u->stream>>>(n, cin, cout, X, frag, bias, Y, relu); break;
  case 48: k_conv3<48><<<grid, CTHREADS, smem, u->stream>>>(n, cin, cout, X, frag, bias, Y, relu); break;
  case 32: k_conv3<32><<<grid, CTHREADS, smem, u->stream>>>(n, cin, cout, X, frag, bias, Y, relu); break;
  default: k_conv3<16><<<grid, CTHREADS, smem, u->stream>>>(n, cin, cout, X, frag, bias, Y, relu); break;
  }
  return cudaGetLastError();
}

/* forward convolution l: tcgen05 where it fits, mma.sync otherwise */
cudaError_t conv_fwd(FlipUNet *u, int l, int n, int batch, const bf16 *X, bf16 *Y) {
  const int cin = kConv[l].cin, cout = kConv[l].cout;
  const float *bias = u->P + u->boff[l];
  if (u->tc && conv_tc_supported(n, cin, cout))
    return conv_tc_launch(u->stream, n, batch, cin, cout, X, u->tcw[l], bias, Y, 1, u->tc_err);
  return conv(u, n, batch, cin, cout, X, u->ffrag[l], bias, Y, 1);
}

int lvl_n(int n, int level) { return n >> level; }

int ensure_workspace(FlipUNet *u, int n, int batch) {
  if (u->ws_n == n && u->ws_b >= batch) return FLIPGPU_OK;
  const size_t B = (size_t)batch;
  const size_t V0 = (size_t)n * n * n, V1 = V0 / 8, V2 = V1 / 8, V3 = V2 / 8;
  UCK(ualloc(u->X0, 16 * V0 * B));
  UCK(ualloc(u->A0, 16 * V0 * B));
  UCK(ualloc(u->E0, 16 * V0 * B));
  UCK(ualloc(u->P1, 16 * V1 * B));
  UCK(ualloc(u->A1, 32 * V1 * B));
  UCK(ualloc(u->E1, 32 * V1 * B));
  UCK(ualloc(u->P2, 32 * V2 * B));
  UCK(ualloc(u->A2, 48 * V2 * B));
  UCK(ualloc(u->E2, 48 * V2 * B));
  UCK(ualloc(u->P3, 48 * V3 * B));
  UCK(ualloc(u->A3, 64 * V3 * B));
  UCK(ualloc(u->E3, 64 * V3 * B));
  UCK(ualloc(u->U2, 112 * V2 * B));
  UCK(ualloc(u->B2, 48 * V2 * B));
  UCK(ualloc(u->D2, 48 * V2 * B));
  UCK(ualloc(u->U1, 80 * V1 * B));
  UCK(ualloc(u->B1, 32 * V1 * B));
  UCK(ualloc(u->D1, 32 * V1 * B));
  UCK(ualloc(u->U0, 48 * V0 * B));
  UCK(ualloc(u->B0, 16 * V0 * B));
  UCK(ualloc(u->D0, 16 * V0 * B));
  size_t gmax = 48 * V0 * B;
  UCK(ualloc(u->G1, gmax));
  UCK(ualloc(u->G2, gmax));
  UCK(ualloc(u->G3, gmax));
  UCK(ualloc(u->S0, 16 * V0 * B));
  UCK(ualloc(u->S1, 32 * V1 * B));
  UCK(ualloc(u->S2, 48 * V2 * B));
  UCK(ualloc(u->O, V0 * B));
  UCK(ualloc(u->scale, 4 * B));
  UCK(ualloc(u->red, 4 * RB * B + 64));
  UCK(ualloc(u->count, B));
  UCK(ualloc(u->loss, 4));
  /* weight-gradient partials: chunks x 27 x cin x cout over all layers */
  size_t pc = 0, pb = 0;
  for (int l = 0; l < NCONV; l++) {
    const size_t V = (size_t)lvl_n(n, kConv[l].level) * lvl_n(n, kConv[l].level) *
                     lvl_n(n, kConv[l].level);
    const size_t chunks = (V + 4095) / 4096 * B;
    pc = std::max(pc, chunks * 27 * kConv[l].cin * kConv[l].cout);
    pb = std::max(pb, chunks * kConv[l].cout);
  }
  UCK(ualloc(u->part, pc));
  UCK(ualloc(u->part_b, pb));
  u->part_cap = pc;
  u->partb_cap = pb;
  const size_t hb = (V0 * B + EBLK - 1) / EBLK;
  UCK(ualloc(u->hpart, hb * 18));
  u->hpart_cap = hb;
  u->ws_n = n;
  u->ws_b = batch;
  return FLIPGPU_OK;
}

int refresh_frags(FlipUNet *u) {
  if (u->frags_fresh) return FLIPGPU_OK;
  for (int l = 0; l < NCONV; l++) {
    const int cin = kConv[l].cin, cout = kConv[l].cout;
    const int nf = 27 * (cin / 16) * (cout / 8) * 32, nb = 27 * (cout / 16) * (cin / 8) * 32;
    k_pack<<<(nf + nb + EBLK - 1) / EBLK, EBLK, 0, u->stream>>>(cin, cout, u->P + u->woff[l],
                                                               u->ffrag[l], u->bfrag[l]);
    if (u->tc) UCK(conv_tc_pack(u->stream, cin, cout, u->P + u->woff[l], u->tcw[l]));
  }
  UCK(cudaGetLastError());
  u->frags_fresh = true;
  return FLIPGPU_OK;
}

/* features and per-sample scales of a batch of systems */
unsigned eg(size_t count) { return (unsigned)((count + EBLK - 1) / EBLK); }

/* fine-grid buffers of the coarsened warm start (grid n, network on n >> c) */
int ensure_fine(FlipUNet *u, int n, int batch) {
  if (!u->coarse || (u->fw_n == n && u->fw_b >= batch)) return FLIPGPU_OK;
  const size_t B = (size_t)batch, V = (size_t)n * n * n, Vc = V >> (3 * u->coarse);
  UCK(ualloc(u->XF, 16 * V * B));
  UCK(ualloc(u->XP, 16 * (V / 8 + V / 64) * B));
  UCK(ualloc(u->Ac, Vc * B));
  UCK(ualloc(u->xc, Vc * B));
  UCK(ualloc(u->x0c, Vc * B));
  UCK(ualloc(u->Of, V * B));
  u->fw_n = n;
  u->fw_b = batch;
  return FLIPGPU_OK;
}

/* per-sample scales and the 16-channel input on the fine grid n; with
 * coarsening c the features are average-pooled c times into X0 */
int prepare_inputs(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                   const float *x0, const float *r0) {
  const size_t n3 = (size_t)n * n * n;
  const int c = u->coarse;
  k_sample_sums<<<dim3(RB, batch), EBLK, 0, u->stream>>>(n3, A, b, r0, x0, u->red);
  k_sample_scale<<<batch, RB, 0, u->stream>>>(batch, n, u->red, u->scale, u->count);
  k_features<<<(unsigned)((n3 * batch + EBLK - 1) / EBLK), EBLK, 0, u->stream>>>(
      n3, batch, A, b, r0, x0, u->scale, c ? u->XF : u->X0);
  const bf16 *src = u->XF;
  bf16 *tmp[2] = {u->XP, u->XP + 16 * (n3 / 8) * batch};
  for (int k = 1; k <= c; k++) {
    const int nk = n >> k;
    bf16 *dst = k == c ? u->X0 : tmp[k - 1];
    k_pool<<<eg((size_t)nk * nk * nk * batch * 8), EBLK, 0, u->stream>>>(nk, 16, batch, src, dst);
    src = dst;
  }
  UCK(cudaGetLastError());
  return FLIPGPU_OK;
}

int forward(FlipUNet *u, int n, int batch) {
  const int B = batch;
  const int n1 = n / 2, n2 = n / 4, n3l = n / 8;
  const size_t V0 = (size_t)n * n * n, V1 = V0 / 8, V2 = V1 / 8, V3 = V2 / 8;
  UCK(conv_fwd(u, 0, n, B, u->X0, u->A0));
  UCK(conv_fwd(u, 1, n, B, u->A0, u->E0));
  k_pool<<<eg(V1 * B * 8), EBLK, 0, u->stream>>>(n1, 16, B, u->E0, u->P1);
  UCK(conv_fwd(u, 2, n1, B, u->P1, u->A1));
  UCK(conv_fwd(u, 3, n1, B, u->A1, u->E1));
  k_pool<<<eg(V2 * B * 16), EBLK, 0, u->stream>>>(n2, 32, B, u->E1, u->P2);
  UCK(conv_fwd(u, 4, n2, B, u->P2, u->A2));
  UCK(conv_fwd(u, 5, n2, B, u->A2, u->E2));
  k_pool<<<eg(V3 * B * 24), EBLK, 0, u->stream>>>(n3l, 48, B, u->E2, u->P3);
  UCK(conv_fwd(u, 6, n3l, B, u->P3, u->A3));
  UCK(conv_fwd(u, 7, n3l, B, u->A3, u->E3));
  k_up_cat<<<eg(V2 * B * 14), EBLK, 0, u->stream>>>(n2, 64, 48, B, u->E3, u->E2, u->U2);
  UCK(conv_fwd(u, 8, n2, B, u->U2, u->B2));
  UCK(conv_fwd(u, 9, n2, B, u->B2, u->D2));
  k_up_cat<<<eg(V1 * B * 10), EBLK, 0, u->stream>>>(n1, 48, 32, B, u->D2, u->E1, u->U1);
  UCK(conv_fwd(u, 10, n1, B, u->U1, u->B1));
  UCK(conv_fwd(u, 11, n1, B, u->B1, u->D1));
  k_up_cat<<<eg(V0 * B * 6), EBLK, 0, u->stream>>>(n, 32, 16, B, u->D1, u->E0, u->U0);
  UCK(conv_fwd(u, 12, n, B, u->U0, u->B0));
  UCK(conv_fwd(u, 13, n, B, u->B0, u->D0));
  k_head<<<eg(V0 * B), EBLK, 0, u->stream>>>(V0 * B, u->D0, u->P + u->hoff, u->O);
  UCK(cudaGetLastError());
  return FLIPGPU_OK;
}

/* weight gradient of conv l: input X at level n, output gradient dZ */
int wgrad(FlipUNet *u, int l, int n, int batch, const bf16 *X, const bf16 *dZ) {
  const int cin = kConv[l].cin, cout = kConv[l].cout;
  const size_t V = (size_t)n * n * n;
  const int cps = (int)((V + 4095) / 4096);
  const int ch = (int)((V + cps - 1) / cps);
  const size_t chunks = (size_t)cps * batch;
  k_wgrad<<<dim3((unsigned)chunks, 27), CTHREADS, wgrad_smem(cin, cout), u->stream>>>(
      n, cin, cout, cps, ch, X, dZ, u->part, u->part_b);
  const int wc = 27 * cin * cout;
  k_wgrad_reduce<<<(wc + cout + EBLK - 1) / EBLK, EBLK, 0, u->stream>>>(
      (int)chunks, wc, cout, u->part, u->part_b, u->G + u->woff[l], u->G + u->boff[l]);
  UCK(cudaGetLastError());
  return FLIPGPU_OK;
}

/* one conv's backward: dZ = dY where the output was positive (into G2),
 * its weight gradient, and dX = the transposed convolution of dZ (skipped
 * when dX is null) */
int conv_bwd(FlipUNet *u, int l, int n, int batch, const bf16 *dY, const bf16 *Xin,
             const bf16 *Yout, bf16 *dX) {
  const int cin = kConv[l].cin, cout = kConv[l].cout;
  const size_t V = (size_t)n * n * n * batch;
  k_relu_bwd<<<eg(V * cout / 8), EBLK, 0, u->stream>>>(V * cout / 8, dY, Yout, u->G2);
  int r = wgrad(u, l, n, batch, Xin, u->G2);
  if (r != FLIPGPU_OK) return r;
  if (dX) UCK(conv(u, n, batch, cout, cin, u->G2, u->bfrag[l], nullptr, dX, 0));
  return FLIPGPU_OK;
}

int backward(FlipUNet *u, int n, int batch, const uint8_t *A, const float *x, const float *x0) {
  const int B = batch;
  const int n1 = n / 2, n2 = n / 4;
  const size_t V0 = (size_t)n * n * n, V1 = V0 / 8, V2 = V1 / 8;
  int r;
  /* loss over the batch's liquid cells and the head's backward */
  double cnt_host[64];
  UCK(cudaMemcpyAsync(cnt_host, u->count, sizeof(double) * B, cudaMemcpyDeviceToHost, u->stream));
  UCK(cudaStreamSynchronize(u->stream));
  double total = 0.0;
  for (int s = 0; s < B; s++) total += cnt_host[s];
  const double inv = total > 0.0 ? 1.0 / total : 0.0;
  const unsigned hb = eg(V0 * B);
  k_loss_head_bwd<<<hb, EBLK, 0, u->stream>>>(V0, B, A, x, x0, u->scale, inv, u->O, u->D0,
                                              u->P + u->hoff, u->G1, u->hpart);
  k_head_reduce<<<1, 32, 0, u->stream>>>((int)hb, u->hpart, u->G + u->hoff, u->loss);
  UCK(cudaGetLastError());
  /* decoder, level 0 */
  if ((r = conv_bwd(u, 13, n, B, u->G1, u->B0, u->D0, u->G3))) return r;
  if ((r = conv_bwd(u, 12, n, B, u->G3, u->U0, u->B0, u->G1))) return r;  /* dU0: 48 */
  k_slice<<<eg(V0 * B * 2), EBLK, 0, u->stream>>>(V0 * B, 48, 32, 16, u->G1, u->S0);
  k_up_bwd<<<eg(V1 * B * 32), EBLK, 0, u->stream>>>(n, 32, 48, B, u->G1, u->G3);
  /* level 1 */
  if ((r = conv_bwd(u, 11, n1, B, u->G3, u->B1, u->D1, u->G1))) return r;
  if ((r = conv_bwd(u, 10, n1, B, u->G1, u->U1, u->B1, u->G3))) return r; /* dU1: 80 */
  k_slice<<<eg(V1 * B * 4), EBLK, 0, u->stream>>>(V1 * B, 80, 48, 32, u->G3, u->S1);
  k_up_bwd<<<eg(V2 * B * 48), EBLK, 0, u->stream>>>(n1, 48, 80, B, u->G3, u->G1);
  /* level 2 */
  if ((r = conv_bwd(u, 9, n2, B, u->G1, u->B2, u->D2, u->G3))) return r;
  if ((r = conv_bwd(u, 8, n2, B, u->G3, u->U2, u->B2, u->G1))) return r;  /* dU2: 112 */
  k_slice<<<eg(V2 * B * 6), EBLK, 0, u->stream>>>(V2 * B, 112, 64, 48, u->G1, u->S2);
  k_up_bwd<<<eg(V2 / 8 * B * 64), EBLK, 0, u->stream>>>(n2, 64, 112, B, u->G1, u->G3);
  /* bottleneck */
  if ((r = conv_bwd(u, 7, n2 / 2, B, u->G3, u->A3, u->E3, u->G1))) return r;
  if ((r = conv_bwd(u, 6, n2 / 2, B, u->G1, u->P3, u->A3, u->G3))) return r; /* dP3: 48 */
  /* encoder */
  k_pool_bwd<<<eg(V2 * B * 48), EBLK, 0, u->stream>>>(n2, 48, B, u->G3, u->S2, 48, 0, u->G1);
  if ((r = conv_bwd(u, 5, n2, B, u->G1, u->A2, u->E2, u->G3))) return r;
  if ((r = conv_bwd(u, 4, n2, B, u->G3, u->P2, u->A2, u->G1))) return r;  /* dP2: 32 */
  k_pool_bwd<<<eg(V1 * B * 32), EBLK, 0, u->stream>>>(n1, 32, B, u->G1, u->S1, 32, 0, u->G3);
  if ((r = conv_bwd(u, 3, n1, B, u->G3, u->A1, u->E1, u->G1))) return r;
  if ((r = conv_bwd(u, 2, n1, B, u->G1, u->P1, u->A1, u->G3))) return r;  /* dP1: 16 */
  k_pool_bwd<<<eg(V0 * B * 16), EBLK, 0, u->stream>>>(n, 16, B, u->G3, u->S0, 16, 0, u->G1);
  if ((r = conv_bwd(u, 1, n, B, u->G1, u->A0, u->E0, u->G3))) return r;
  if ((r = conv_bwd(u, 0, n, B, u->G3, u->X0, u->A0, nullptr))) return r;
  UCK(cudaGetLastError());
  return FLIPGPU_OK;
}

} // namespace

/* ====================================================================== C ABI */

namespace {

uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* He-normal weights (std sqrt(2/fan_in), Box-Muller on keyed uniforms),
 * zero biases; the first convolution's padded input channels stay zero. */
void init_params(FlipUNet *u, uint64_t seed, std::vector<float> &p) {
  p.assign((size_t)u->nparam, 0.0f);
  uint64_t ctr = 0;
  auto unif = [&]() {
    uint64_t r = mix64(seed * 0x2545f4914f6cdd1dull + (ctr++));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  auto normal = [&]() {
    const double a = unif(), b = unif();
    return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
  };
  for (int l = 0; l < NCONV; l++) {
    const int cin = kConv[l].cin, cout = kConv[l].cout;
    const int real_in = l == 0 ? IN_CH : cin;
    const double sd = sqrt(2.0 / (27.0 * real_in));
    for (int tap = 0; tap < 27; tap++)
      for (int ci = 0; ci < cin; ci++)
        for (int co = 0; co < cout; co++) {
          const double w = normal() * sd;
          if (ci < real_in) p[u->woff[l] + ((size_t)tap * cin + ci) * cout + co] = (float)w;
        }
  }
  const double sd = 0.1 * sqrt(1.0 / 16.0); /* small head: the first guesses stay near x0 */
  for (int c = 0; c < 16; c++) p[u->hoff + c] = (float)(normal() * sd);
}

} // namespace

extern "C" {

int64_t flipunet_param_count(void) {
  int64_t n = 0;
  for (int l = 0; l < NCONV; l++) n += 27LL * kConv[l].cin * kConv[l].cout + kConv[l].cout;
  return n + 17;
}

const char *flipunet_last_error(const FlipUNet *u) { return u ? u->err : "null network"; }

int flipunet_destroy(FlipUNet *u) {
  if (!u) return FLIPGPU_EINVAL;
  if (u->stream) cudaStreamSynchronize(u->stream);
  else cudaDeviceSynchronize();
  void *ptrs[] = {u->P,  u->G,  u->M,  u->V,  u->X0, u->A0, u->E0, u->P1, u->A1, u->E1,
                  u->P2, u->A2, u->E2, u->P3, u->A3, u->E3, u->U2, u->B2, u->D2, u->U1,
                  u->B1, u->D1, u->U0, u->B0, u->D0, u->G1, u->G2, u->G3, u->S0, u->S1,
                  u->S2, u->O,  u->scale, u->red, u->count, u->loss, u->part, u->part_b,
                  u->hpart, u->XF, u->XP, u->Ac, u->xc, u->x0c, u->Of};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int l = 0; l < NCONV; l++) {
    if (u->ffrag[l]) cudaFree(u->ffrag[l]);
    if (u->bfrag[l]) cudaFree(u->bfrag[l]);
    if (u->tcw[l]) cudaFree(u->tcw[l]);
  }
  if (u->tc_err) cudaFree(u->tc_err);
  delete u;
  return FLIPGPU_OK;
}

int flipunet_create(uint64_t seed, FlipUNet **out) {
  if (!out) return FLIPGPU_EINVAL;
  *out = nullptr;
  if (unet_init_device() != 0) return FLIPGPU_ECUDA;
  FlipUNet *u = new FlipUNet;
  int64_t off = 0;
  for (int l = 0; l < NCONV; l++) {
    u->woff[l] = off;
    off += 27LL * kConv[l].cin * kConv[l].cout;
    u->boff[l] = off;
    off += kConv[l].cout;
  }
  u->hoff = off;
  off += 17;
  u->nparam = off;
  const size_t np = (size_t)off;
  if (ualloc(u->P, np) || ualloc(u->G, np) || ualloc(u->M, np) || ualloc(u->V, np)) {
    flipunet_destroy(u);
    return FLIPGPU_ENOMEM;
  }
  for (int l = 0; l < NCONV; l++) {
    const size_t nf = 27 * (kConv[l].cin / 16) * (kConv[l].cout / 8) * 32;
    const size_t nb = 27 * (kConv[l].cout / 16) * (kConv[l].cin / 8) * 32;
    if (ualloc(u->ffrag[l], nf) || ualloc(u->bfrag[l], nb) ||
        ualloc(u->tcw[l], (size_t)27 * kConv[l].cin * kConv[l].cout)) {
      flipunet_destroy(u);
      return FLIPGPU_ENOMEM;
    }
  }
  if (ualloc(u->tc_err, 1) || cudaMemset(u->tc_err, 0, sizeof(int)) != cudaSuccess) {
    flipunet_destroy(u);
    return FLIPGPU_ENOMEM;
  }
  std::vector<float> p;
  init_params(u, seed, p);
  if (cudaMemcpy(u->P, p.data(), np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(u->M, 0, np * sizeof(float)) != cudaSuccess ||
      cudaMemset(u->V, 0, np * sizeof(float)) != cudaSuccess ||
      cudaMemset(u->G, 0, np * sizeof(float)) != cudaSuccess) {
    flipunet_destroy(u);
    return FLIPGPU_ECUDA;
  }
  *out = u;
  return FLIPGPU_OK;
}

int flipunet_set_stream(FlipUNet *u, void *stream) {
  if (!u) return FLIPGPU_EINVAL;
  u->stream = (cudaStream_t)stream;
  return FLIPGPU_OK;
}

int flipunet_get_params(FlipUNet *u, float *params) {
  if (!u || !params) return FLIPGPU_EINVAL;
  UCK(cudaMemcpyAsync(params, u->P, u->nparam * sizeof(float), cudaMemcpyDeviceToHost, u->stream));
  UCK(cudaStreamSynchronize(u->stream));
  return FLIPGPU_OK;
}

int flipunet_set_params(FlipUNet *u, const float *params) {
  if (!u || !params) return FLIPGPU_EINVAL;
  UCK(cudaMemcpyAsync(u->P, params, u->nparam * sizeof(float), cudaMemcpyHostToDevice, u->stream));
  UCK(cudaMemsetAsync(u->M, 0, u->nparam * sizeof(float), u->stream));
  UCK(cudaMemsetAsync(u->V, 0, u->nparam * sizeof(float), u->stream));
  UCK(cudaStreamSynchronize(u->stream));
  u->adam_t = 0;
  u->frags_fresh = false;
  return FLIPGPU_OK;
}

static int check_shape(FlipUNet *u, int n, int batch) {
  const int q = 8 << u->coarse;
  if (n < q || n % q != 0 || batch < 1 || batch > 64) {
    snprintf(u->err, sizeof u->err,
             "grid size must be a multiple of %d (8 << coarsening) and batch 1..64", q);
    return FLIPGPU_EINVAL;
  }
  return FLIPGPU_OK;
}

int flipunet_predict(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                     const float *x0, const float *r0, float *delta) {
  if (!u || !A || !b || !x0 || !r0 || !delta) return FLIPGPU_EINVAL;
  int r;
  const int nn = n >> u->coarse;
  if ((r = check_shape(u, n, batch)) || (r = ensure_workspace(u, nn, batch)) ||
      (r = ensure_fine(u, n, batch)) || (r = refresh_frags(u)) ||
      (r = prepare_inputs(u, n, batch, A, b, x0, r0)) || (r = forward(u, nn, batch)))
    return r;
  const size_t n3 = (size_t)n * n * n;
  const float *O = u->O;
  if (u->coarse) {
    k_prolong<<<eg(n3 * batch), EBLK, 0, u->stream>>>(nn, 1 << u->coarse, batch, u->O, u->Of);
    O = u->Of;
  }
  k_delta_out<<<eg(n3 * batch), EBLK, 0, u->stream>>>(n3, batch, A, O, u->scale, delta);
  UCK(cudaGetLastError());
  if (u->tc) {
    int e = 0;
    UCK(cudaMemcpyAsync(&e, u->tc_err, sizeof(int), cudaMemcpyDeviceToHost, u->stream));
    UCK(cudaStreamSynchronize(u->stream));
    if (e) {
      snprintf(u->err, sizeof u->err, "tcgen05 convolution: a bounded wait expired");
      return FLIPGPU_ETIMEOUT;
    }
  }
  return FLIPGPU_OK;
}

int flipunet_set_coarsening(FlipUNet *u, int levels) {
  if (!u || levels < 0 || levels > 3) return FLIPGPU_EINVAL;
  u->coarse = levels;
  u->fw_n = 0; /* fine buffers are sized per coarsening */
  return FLIPGPU_OK;
}

int flipunet_get_coarsening(const FlipUNet *u) { return u ? u->coarse : -1; }

int flipunet_set_tensor_path(FlipUNet *u, int tcgen05) {
  if (!u) return FLIPGPU_EINVAL;
  u->tc = tcgen05 ? 1 : 0;
  u->frags_fresh = false;
  return FLIPGPU_OK;
}

static int grads(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                 const float *x0, const float *r0, const float *x, double *loss) {
  int r;
  const int nn = n >> u->coarse;
  if ((r = check_shape(u, n, batch)) || (r = ensure_workspace(u, nn, batch)) ||
      (r = ensure_fine(u, n, batch)) || (r = refresh_frags(u)) ||
      (r = prepare_inputs(u, n, batch, A, b, x0, r0)) || (r = forward(u, nn, batch)))
    return r;
  if (u->coarse) {
    /* targets, liquid flags and liquid counts on the network's grid */
    const size_t nc3 = (size_t)nn * nn * nn;
    k_pool_target<<<eg(nc3 * batch), EBLK, 0, u->stream>>>(nn, 1 << u->coarse, batch, A, x, x0,
                                                           u->Ac, u->xc, u->x0c);
    UCK(cudaMemsetAsync(u->count, 0, sizeof(double) * batch, u->stream));
    k_count_fluid<<<dim3(64, batch), EBLK, 0, u->stream>>>(nc3, u->Ac, u->count);
    UCK(cudaGetLastError());
    A = u->Ac;
    x = u->xc;
    x0 = u->x0c;
  }
  if ((r = backward(u, nn, batch, A, x, x0))) return r;
  if (loss) {
    UCK(cudaMemcpyAsync(loss, u->loss, sizeof(double), cudaMemcpyDeviceToHost, u->stream));
    UCK(cudaStreamSynchronize(u->stream));
  }
  return FLIPGPU_OK;
}

int flipunet_gradients(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                       const float *x0, const float *r0, const float *x, double *loss,
                       float *grad_host) {
  if (!u || !A || !b || !x0 || !r0 || !x) return FLIPGPU_EINVAL;
  int r = grads(u, n, batch, A, b, x0, r0, x, loss);
  if (r) return r;
  if (grad_host) {
    UCK(cudaMemcpyAsync(grad_host, u->G, u->nparam * sizeof(float), cudaMemcpyDeviceToHost,
                        u->stream));
    UCK(cudaStreamSynchronize(u->stream));
  }
  return FLIPGPU_OK;
}

int flipunet_train_step(FlipUNet *u, int n, int batch, const uint8_t *A, const float *b,
                        const float *x0, const float *r0, const float *x, float lr,
                        double *loss) {
  if (!u || !A || !b || !x0 || !r0 || !x) return FLIPGPU_EINVAL;
  int r = grads(u, n, batch, A, b, x0, r0, x, loss);
  if (r) return r;
  u->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = (float)(1.0 - pow(0.9, (double)u->adam_t));
  const float c2 = (float)(1.0 - pow(0.999, (double)u->adam_t));
  k_adam<<<eg((size_t)u->nparam), EBLK, 0, u->stream>>>((size_t)u->nparam, u->P, u->G, u->M, u->V,
                                                       lr, b1, b2, 1e-8f, c1, c2);
  UCK(cudaGetLastError());
  u->frags_fresh = false;
  return FLIPGPU_OK;
}

} // extern "C"

/* The solver's warm start (FAST mode): x0 += g d with d the network's
 * correction and g the least-residual step along d (k_wm_apply). */
int warm_start_apply(FlipGpu *h, float inv_h2_f, double *out3, float *ms) {
  FlipUNet *u = h->warm;
  cudaStream_t keep = u->stream;
  u->stream = h->stream;
  const int n = h->n;
  const size_t nc = h->nc;
  int r = FLIPGPU_OK;
  if (!h->wdelta) {
    if (cudaMalloc(&h->wdelta, 3 * nc * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&h->wpart, (RB * 5 + 4) * sizeof(double)) != cudaSuccess ||
        cudaEventCreate(&h->wev[0]) != cudaSuccess || cudaEventCreate(&h->wev[1]) != cudaSuccess) {
      u->stream = keep;
      return FLIPGPU_ENOMEM;
    }
  }
  cudaEventRecord(h->wev[0], h->stream);
  float *d = h->wdelta, *w = h->wdelta + nc, *rr = h->wdelta + 2 * nc;
  k_wm_residual<<<eg(nc), EBLK, 0, h->stream>>>(n, inv_h2_f, h->A, h->diag, h->div, h->press, rr);
  FG_LAUNCHED(h, 1);
  r = flipunet_predict(u, n, 1, h->A, h->div, h->press, rr, d);
  if (r == FLIPGPU_OK) {
    k_wm_matvec<<<eg(nc), EBLK, 0, h->stream>>>(n, inv_h2_f, h->A, h->diag, d, w);
    k_wm_dots<<<RB, EBLK, 0, h->stream>>>(nc, h->A, rr, d, w, h->wpart);
    const char *ev = getenv("FLIPGPU_WARM_STEP");
    const int minres = !(ev && strcmp(ev, "anorm") == 0);
    k_wm_apply<<<RB, EBLK, 0, h->stream>>>(nc, h->A, h->wpart, d, h->press, h->wpart + RB * 5,
                                           minres);
    FG_LAUNCHED(h, 3);
    cudaEventRecord(h->wev[1], h->stream);
    if (cudaMemcpyAsync(out3, h->wpart + RB * 5, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      r = FLIPGPU_ECUDA;
    cudaEventElapsedTime(ms, h->wev[0], h->wev[1]);
  } else {
    snprintf(h->err, sizeof h->err, "warm start: %s", u->err);
  }
  u->stream = keep;
  return r;
}

/* r = b - A x with the solver's FAST-mode matrix (after its setup) */
cudaError_t launch_residual(FlipGpu *h, float inv_h2_f, const float *x, float *r) {
  k_wm_residual<<<eg(h->nc), EBLK, 0, h->stream>>>(h->n, inv_h2_f, h->A, h->diag, h->div, x, r);
  FG_LAUNCHED(h, 1);
  return cudaGetLastError();
}
