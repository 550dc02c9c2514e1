/*
 * k_conv_tc.cu — the U-Net's forward 3x3x3 convolution on the 5th-generation
 * tensor cores: tcgen05.mma (BF16 x BF16 -> FP32) with the accumulators in
 * tensor memory, operands staged by the tensor memory accelerator (TMA).
 *
 * Padded slots. A CTA's unit of work is R output k-lines j0 .. j0+R-1 of
 * one (sample s, plane i, k-segment of Lk = min(n, 128) cells). For each
 * input plane i+di-1 one TMA copy per 8-channel plane brings the R+2 lines
 * j0-1 .. j0+R, each with one cell of k halo on both sides, as P = Lk+2
 * slots per line; cells outside the grid arrive as zeros (the copy's
 * out-of-bounds fill), so no boundary case reaches the MMA. In that slab
 * the input of output slot u = r*P + k' (line r, cell k'-1) for tap
 * (dj, dk) is slot u + dj*P + dk - 1: every tap reads the same run of slots,
 * shifted, so each tap's A operand is a shared-memory descriptor at a
 * tap-dependent start and nothing is copied per tap. One M=128 MMA tile is
 * 128 consecutive slots: a whole 128-cell segment when n >= 128, else a run
 * across line ends whose halo-slot rows are computed and dropped.
 *
 * Shared-memory layout (K-major, no swizzle, core matrices 8 rows x 16 B):
 * a slab plane is [line][slot][8 channels], rows 16 B apart (SBO = 128 B
 * per 8 rows); the two 8-channel halves of a 16-channel K step are one
 * plane apart (LBO). The weights of one (di, 16-channel chunk) stage are
 * 9 taps x Cout x 16 channels in the same layout (LBO = Cout/8 core
 * matrices, SBO = 128 B).
 *
 * Issue rate. A tcgen05.mma of M=128, N<=64, K=16 occupies its issuing
 * warp for about 55 cycles and the tensor core for about 40, so the narrow
 * N of these layers makes the convolution issue-bound: the MMAs of a stage
 * are fully unrolled over the tile count T (a template parameter) with
 * descriptors formed by one 64-bit add each, and two warps issue them, each
 * for its own tiles and accumulators.
 *
 * Pipeline, one CTA of 7 warps per SM, persistent over units, a ring of up
 * to 6 stages (di, 16-channel chunk):
 *   warp 0     producer (one thread): two TMA tile copies (one per 8-channel
 *              plane) and one bulk copy of the stage's weights, completion
 *              counted in bytes on full[stage];
 *   warps 1-2  MMA issuers (one thread each): 9 taps x its tiles, M=128,
 *              N=Cout, K=16; tcgen05.commit releases the stage
 *              (empty[stage], two arrivals) and, after a unit's last stage,
 *              hands the accumulator buffer to the epilogue (acc_full);
 *   warps 3-6  epilogue: tcgen05.ld of the warp's 32-lane quarter, bias,
 *              ReLU, BF16, stores of the valid rows; acc_empty hands the
 *              buffer back.
 * Two accumulator buffers let one unit's epilogue overlap the next unit's
 * MMAs. Planes i+di-1 outside the grid contribute nothing and are skipped
 * by producer and issuers alike. Every wait is bounded: an expired wait sets
 * a flag that ends every role's loop; the CTA then waits (bounded) for its
 * own copies and MMAs in flight, frees its tensor memory and sets *err.
 */
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>

#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "autotune.h"
#include "conv_tc.h"

typedef __nv_bfloat16 bf16;

namespace {

constexpr int TC_THREADS = 224;
constexpr int TC_STAGES = 6;
constexpr unsigned TC_SPIN = 1u << 22;
constexpr uint32_t TC_GUARD = 2304;       /* slots read past a slab by dropped rows */
constexpr size_t TC_SMEM_MAX = 225 * 1024;
constexpr size_t TC_SMEM_MIN = 120 * 1024; /* keeps one CTA per SM: its TMEM is never contended */

struct TcShape {
  int n, cin, cout, batch;
  int lk, segs, P, R, T, nslab, stages;
  uint32_t plane_stride, a_tx, w_bytes, stage_bytes, ncols;
};

struct TcCtl {
  uint64_t full[TC_STAGES], empty[TC_STAGES], acc_full[2], acc_empty[2], done[2];
  float bias[64];
  uint32_t tmem;
  int fail, produced, consumed;
};

__device__ __forceinline__ uint32_t su32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* shared-memory matrix descriptor: start, LBO, SBO (all >> 4), version 1,
 * no swizzle. The start field is the low 14 bits, so adding (bytes >> 4)
 * to a descriptor moves its start while it stays below 256 KB. */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t b, uint32_t parity) {
  uint32_t done;
  asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
               "selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(done)
               : "r"(b), "r"(parity)
               : "memory");
  return done != 0;
}
/* bounded wait; returns early (false) once another role has failed */
__device__ __forceinline__ bool tc_wait(uint32_t b, uint32_t parity, volatile int *fail) {
  for (unsigned spin = 0; spin < TC_SPIN; spin++) {
    if (mbar_try(b, parity)) return true;
    if ((spin & 255u) == 255u) {
      if (*fail) return false;
      __nanosleep(32);
    }
  }
  *fail = 1;
  return false;
}
/* bounded wait that ignores the failure flag (draining after a failure) */
__device__ __forceinline__ bool tc_wait_drain(uint32_t b, uint32_t parity) {
  for (unsigned spin = 0; spin < TC_SPIN; spin++) {
    if (mbar_try(b, parity)) return true;
    if ((spin & 255u) == 255u) __nanosleep(32);
  }
  return false;
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(b) : "memory");
}
__device__ __forceinline__ void tma_tile_5d(uint32_t dst, const void *map, int c0, int c1, int c2,
                                            int c3, int c4, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
               "[%3];\n" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
      : "memory");
}
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t accum) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
               "l"(a), "l"(b), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
               "%12,%13,%14,%15}, [%16];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                 "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
}

__device__ __forceinline__ void tc_unit(const TcShape &sh, int unit, int &s, int &i, int &seg,
                                        int &j0) {
  const int slab = unit % sh.nslab;
  int t = unit / sh.nslab;
  seg = t % sh.segs;
  t /= sh.segs;
  i = t % sh.n;
  s = t / sh.n;
  j0 = slab * sh.R;
}
/* first slot of MMA tile t within a unit */
__device__ __forceinline__ int tc_tile_start(const TcShape &sh, int t) {
  return sh.lk == 128 ? t * sh.P + 1 : 1 + 128 * t;
}

/* T: MMA tiles per unit; issuer 0 owns tiles [0, H), issuer 1 [H, T) */
template <int T>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv_tc(const __grid_constant__ CUtensorMap xmap, const TcShape sh,
              const bf16 *__restrict__ Wtc, const float *__restrict__ bias, bf16 *__restrict__ Y,
              int relu, int *__restrict__ err) {
  constexpr int H = (T + 1) / 2;
  extern __shared__ __align__(1024) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = sh.stages, nch = sh.cin / 16, cout = sh.cout, P = sh.P, n = sh.n;
  const int kst_n = 3 * nch;
  TcCtl *ctl = reinterpret_cast<TcCtl *>(smraw + (size_t)S * sh.stage_bytes + TC_GUARD);
  volatile int *fail = &ctl->fail;
  if (threadIdx.x == 0) {
    ctl->fail = 0;
    ctl->produced = 0;
    ctl->consumed = 0;
    for (int q = 0; q < TC_STAGES; q++) {
      mbar_init(&ctl->full[q], 1);
      mbar_init(&ctl->empty[q], 2);
    }
    for (int q = 0; q < 2; q++) {
      mbar_init(&ctl->acc_full[q], 2);
      mbar_init(&ctl->acc_empty[q], 4);
      mbar_init(&ctl->done[q], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (threadIdx.x < 64) ctl->bias[threadIdx.x] = (bias && threadIdx.x < cout) ? bias[threadIdx.x] : 0.f;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     su32(&ctl->tmem)),
                 "r"(sh.ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = ctl->tmem;
  const int units = sh.batch * n * sh.segs * sh.nslab;
  const uint32_t sbase = su32(smraw);

  if (warp == 0) {
    /* ---------------- producer */
    int produced = 0;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
      int s, i, seg, j0;
      tc_unit(sh, unit, s, i, seg, j0);
      for (int kst = 0; kst < kst_n; kst++) {
        const int di = kst / nch, c = kst - di * nch;
        if (i + di - 1 < 0 || i + di - 1 >= n) continue;
        const int slot = produced % S;
        const bool ok =
            tc_wait(su32(&ctl->empty[slot]), ((uint32_t)(produced / S) & 1u) ^ 1u, fail);
        if (!__all_sync(0xffffffffu, ok)) goto producer_end;
        if (lane == 0) {
          const uint32_t fb = su32(&ctl->full[slot]);
          const uint32_t a = sbase + (uint32_t)slot * sh.stage_bytes;
          mbar_expect_tx(fb, sh.a_tx + sh.w_bytes);
          tma_tile_5d(a, &xmap, 16 * c, seg * sh.lk - 1, j0 - 1, i + di - 1, s, fb);
          tma_tile_5d(a + sh.plane_stride, &xmap, 16 * c + 8, seg * sh.lk - 1, j0 - 1, i + di - 1,
                      s, fb);
          bulk_copy(a + 2 * sh.plane_stride, Wtc + (size_t)((di * nch + c) * 9) * cout * 16,
                    sh.w_bytes, fb);
        }
        __syncwarp();
        produced++;
      }
    }
  producer_end:
    if (lane == 0) ctl->produced = produced;
  } else if (warp <= 2) {
    /* ---------------- MMA issuers: warp 1 tiles [0, H), warp 2 tiles [H, T) */
    const int me = warp - 1;
    const int t_lo = me ? H : 0, t_hi = me ? T : H;
    int consumed = 0, acc = 0;
    uint32_t aphase = 0;
    /* D f32, A and B bf16, both K-major, N = cout, M = 128 */
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(cout >> 3) << 17) |
                           ((uint32_t)(128 >> 4) << 24);
    /* per-tap start offsets of each tile's A operand, in 16-byte units */
    uint32_t aoff[9][H];
#pragma unroll
    for (int t9 = 0; t9 < 9; t9++)
#pragma unroll
      for (int q = 0; q < H; q++) {
        const int t = t_lo + q < T ? t_lo + q : t_lo; /* unused slot when T is odd */
        aoff[t9][q] = (uint32_t)(tc_tile_start(sh, t) + (t9 / 3) * P + (t9 % 3) - 1);
      }
    const uint64_t wstep = (uint64_t)(cout * 32) >> 4;
    const uint32_t lbo_b = (uint32_t)(cout / 8) * 128u;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
      int s, i, seg, j0;
      tc_unit(sh, unit, s, i, seg, j0);
      bool ok = tc_wait(su32(&ctl->acc_empty[acc]), aphase ^ 1u, fail);
      if (!__all_sync(0xffffffffu, ok)) goto mma_end;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      {
        const uint32_t dbase = tmem + (uint32_t)(acc * T * cout);
        uint32_t accum = 0;
        for (int kst = 0; kst < kst_n; kst++) {
          const int di = kst / nch;
          if (i + di - 1 < 0 || i + di - 1 >= n) continue;
          const int slot = consumed % S;
          ok = tc_wait(su32(&ctl->full[slot]), (uint32_t)(consumed / S) & 1u, fail);
          if (!__all_sync(0xffffffffu, ok)) goto mma_end;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          if (lane == 0) {
            const uint32_t a = sbase + (uint32_t)slot * sh.stage_bytes;
            const uint64_t da = sdesc(a, sh.plane_stride, 128);
            const uint64_t db = sdesc(a + 2 * sh.plane_stride, lbo_b, 128);
#pragma unroll
            for (int t9 = 0; t9 < 9; t9++) {
#pragma unroll
              for (int q = 0; q < H; q++)
                if (t_lo + q < t_hi)
                  umma(dbase + (uint32_t)((t_lo + q) * cout), da + aoff[t9][q],
                       db + (uint64_t)t9 * wstep, idesc, accum | (uint32_t)t9);
            }
            umma_commit(su32(&ctl->empty[slot]));
          }
          __syncwarp();
          accum = 1;
          consumed++;
        }
      }
      if (lane == 0) umma_commit(su32(&ctl->acc_full[acc]));
      __syncwarp();
      if (++acc == 2) {
        acc = 0;
        aphase ^= 1u;
      }
    }
  mma_end:
    if (lane == 0 && me == 0) ctl->consumed = consumed;
  } else {
    /* ---------------- epilogue (warps 3-6): warp w reads TMEM lanes 32*(w%4) .. +31 */
    const int q = warp & 3, m = q * 32 + lane;
    int acc = 0;
    uint32_t aphase = 0;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
      int s, i, seg, j0;
      tc_unit(sh, unit, s, i, seg, j0);
      const bool ok = tc_wait(su32(&ctl->acc_full[acc]), aphase, fail);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * T * cout);
#pragma unroll 1
      for (int t = 0; t < T; t++) {
        const int u = tc_tile_start(sh, t) + m;
        const int r = u / P, kp = u - r * P, j = j0 + r;
        const bool valid = r < sh.R && kp >= 1 && kp <= sh.lk && j < n;
        bf16 *yrow = nullptr;
        if (valid)
          yrow = Y + ((((size_t)s * n + i) * n + j) * n + (size_t)seg * sh.lk + kp - 1) * cout;
        for (int c0 = 0; c0 < cout; c0 += 16) {
          uint32_t v[16];
          tmem_ld16(tb + (uint32_t)(t * cout + c0), v);
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          if (valid) {
            __align__(16) bf16 o[16];
#pragma unroll
            for (int e = 0; e < 16; e++) {
              float x = __uint_as_float(v[e]) + ctl->bias[c0 + e];
              if (relu) x = fmaxf(x, 0.0f);
              o[e] = __float2bfloat16(x);
            }
            reinterpret_cast<uint4 *>(yrow + c0)[0] = reinterpret_cast<const uint4 *>(o)[0];
            reinterpret_cast<uint4 *>(yrow + c0)[1] = reinterpret_cast<const uint4 *>(o)[1];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(su32(&ctl->acc_empty[acc]));
      if (++acc == 2) {
        acc = 0;
        aphase ^= 1u;
      }
    }
  }

  /* ---------------- teardown */
  __syncthreads();
  const bool failed = *fail != 0;
  if (threadIdx.x == 0 && failed) {
    /* copies issued for stages no MMA consumed: let them land */
    for (int k = ctl->consumed; k < ctl->produced; k++)
      tc_wait_drain(su32(&ctl->full[k % S]), (uint32_t)(k / S) & 1u);
  }
  if (warp == 1 || warp == 2) {
    /* every MMA this issuer started has completed before the memory is freed */
    if (lane == 0) umma_commit(su32(&ctl->done[warp - 1]));
    __syncwarp();
    tc_wait_drain(su32(&ctl->done[warp - 1]), 0);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  }
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(sh.ncols));
  }
  if (failed && threadIdx.x == 0) atomicExch(err, 1);
}

/* W[tap][ci][co] FP32 -> per stage (di, chunk c) and tap t9 = dj*3 + dk a
 * block of cout*32 bytes: two K-halves of cout/8 core matrices (8 output
 * channels x 8 input channels, 16-byte rows). */
__global__ void k_conv_tc_pack(int cin, int cout, const float *__restrict__ W,
                               bf16 *__restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 27 * cin * cout) return;
  const int co = idx % cout, ci = (idx / cout) % cin, tap = idx / (cout * cin);
  const int di = tap / 9, t9 = tap % 9;
  const int c = ci / 16, kk = ci % 16, h = kk / 8, col = kk % 8, g = co / 8, r = co % 8;
  const size_t byte = (size_t)((di * (cin / 16) + c) * 9 + t9) * cout * 32 +
                      (size_t)(h * (cout / 8) + g) * 128 + r * 16 + col * 2;
  out[byte / 2] = __float2bfloat16(W[idx]);
}

/* R_req / S_req > 0 ask for that many lines per unit / pipeline stages
 * (false if they do not fit); 0 takes the default */
bool tc_plan(int n, int cin, int cout, int batch, TcShape &sh, size_t &smem, int R_req = 0,
             int S_req = 0) {
  if (n < 2 || batch < 1 || cin < 16 || cin % 16 || cout < 16 || cout % 16 || cout > 64)
    return false;
  sh = TcShape{};
  sh.n = n;
  sh.cin = cin;
  sh.cout = cout;
  sh.batch = batch;
  sh.lk = n >= 128 ? 128 : n;
  if (n % sh.lk) return false;
  sh.segs = n / sh.lk;
  sh.P = sh.lk + 2;
  int R = 0, T = 0;
  auto tiles = [&](int r) { return sh.lk == 128 ? r : (r * sh.P - 2 + 127) / 128; };
  auto fits = [&](int r) {
    const int t = tiles(r);
    return r >= 1 && r <= n && n % r == 0 && t <= 5 && 2 * t * cout <= 512;
  };
  if (R_req > 0) {
    if (!fits(R_req)) return false;
    R = R_req;
  } else if (sh.lk == 128) {
    R = 4;
  } else {
    for (int r = 16; r >= 1; r >>= 1)
      if (fits(r)) {
        R = r;
        break;
      }
  }
  if (!R) return false;
  T = tiles(R);
  sh.R = R;
  sh.T = T;
  sh.nslab = (n + R - 1) / R;
  const uint32_t plane = (uint32_t)sh.P * (uint32_t)(R + 2) * 16u;
  sh.plane_stride = (plane + 127u) & ~127u;
  sh.a_tx = 2u * plane;
  sh.w_bytes = 9u * (uint32_t)cout * 32u;
  sh.stage_bytes = 2u * sh.plane_stride + ((sh.w_bytes + 127u) & ~127u);
  const size_t fixed = TC_GUARD + sizeof(TcCtl) + 128;
  int S = S_req > 0 ? S_req : TC_STAGES;
  if (S_req > 0 && (S_req < 2 || S_req > TC_STAGES)) return false;
  while (S_req <= 0 && S > 2 && (size_t)S * sh.stage_bytes + fixed > TC_SMEM_MAX) S--;
  if ((size_t)S * sh.stage_bytes + fixed > TC_SMEM_MAX) return false;
  sh.stages = S;
  uint32_t nc = 32;
  while (nc < 2u * (uint32_t)T * (uint32_t)cout) nc <<= 1;
  if (nc > 512) return false;
  sh.ncols = nc;
  smem = std::max((size_t)S * sh.stage_bytes + fixed, TC_SMEM_MIN);
  return true;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

template <int T> cudaError_t set_smem_limit() {
  return cudaFuncSetAttribute(k_conv_tc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)TC_SMEM_MAX);
}

} // namespace

bool conv_tc_supported(int n, int cin, int cout) {
  TcShape sh;
  size_t smem;
  return tc_plan(n, cin, cout, 1, sh, smem);
}

cudaError_t conv_tc_pack(cudaStream_t st, int cin, int cout, const float *W, bf16 *out) {
  const int total = 27 * cin * cout;
  k_conv_tc_pack<<<(total + 255) / 256, 256, 0, st>>>(cin, cout, W, out);
  return cudaGetLastError();
}

int conv_tc_init_device() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  if (set_smem_limit<1>() || set_smem_limit<2>() || set_smem_limit<3>() || set_smem_limit<4>() ||
      set_smem_limit<5>())
    return -1;
  done[dev] = true;
  return 0;
}

namespace {

/* the plan's (lines per unit, stages) choices for the autotuner; the
 * default first */
std::vector<std::pair<int, int>> tc_candidates(int n, int cin, int cout, int batch) {
  std::vector<std::pair<int, int>> out;
  TcShape sh;
  size_t smem;
  if (!tc_plan(n, cin, cout, batch, sh, smem)) return out;
  out.push_back({sh.R, sh.stages});
  const int rs[] = {1, 2, 4, 8, 16};
  const int ss[] = {3, 4, 6};
  for (int r : rs)
    for (int s : ss) {
      if (r == sh.R && s == sh.stages) continue;
      TcShape c;
      if (tc_plan(n, cin, cout, batch, c, smem, r, s)) out.push_back({r, s});
    }
  return out;
}

cudaError_t tc_launch_one(cudaStream_t st, int n, int batch, int cin, int cout, const bf16 *X,
                          const bf16 *Wtc, const float *bias, bf16 *Y, int relu, int *err,
                          int R, int S) {
  TcShape sh;
  size_t smem;
  if (!tc_plan(n, cin, cout, batch, sh, smem, R, S)) return cudaErrorInvalidValue;
  if (conv_tc_init_device() != 0) return cudaErrorInvalidDeviceFunction;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  /* X as a 5-D tensor {channel, k, j, i, sample}; the box is one 8-channel
   * plane of R+2 lines of P slots */
  CUtensorMap map;
  const cuuint64_t c2 = (cuuint64_t)cin * 2, nn = (cuuint64_t)n;
  const cuuint64_t dims[5] = {(cuuint64_t)cin, nn, nn, nn, (cuuint64_t)batch};
  const cuuint64_t strides[4] = {c2, c2 * nn, c2 * nn * nn, c2 * nn * nn * nn};
  const cuuint32_t box[5] = {8u, (cuuint32_t)sh.P, (cuuint32_t)(sh.R + 2), 1u, 1u};
  const cuuint32_t es[5] = {1u, 1u, 1u, 1u, 1u};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(X), dims, strides, box, es,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int units = batch * n * sh.segs * sh.nslab;
  const int grid = std::min(units, sms);
  switch (sh.T) {
  case 1: k_conv_tc<1><<<grid, TC_THREADS, smem, st>>>(map, sh, Wtc, bias, Y, relu, err); break;
  case 2: k_conv_tc<2><<<grid, TC_THREADS, smem, st>>>(map, sh, Wtc, bias, Y, relu, err); break;
  case 3: k_conv_tc<3><<<grid, TC_THREADS, smem, st>>>(map, sh, Wtc, bias, Y, relu, err); break;
  case 4: k_conv_tc<4><<<grid, TC_THREADS, smem, st>>>(map, sh, Wtc, bias, Y, relu, err); break;
  default: k_conv_tc<5><<<grid, TC_THREADS, smem, st>>>(map, sh, Wtc, bias, Y, relu, err); break;
  }
  return cudaGetLastError();
}

} // namespace

/* lines per unit (the tile shape) and pipeline depth picked by the
 * autotuner per (n, cin, cout, batch); the result does not depend on them */
cudaError_t conv_tc_launch(cudaStream_t st, int n, int batch, int cin, int cout, const bf16 *X,
                           const bf16 *Wtc, const float *bias, bf16 *Y, int relu, int *err) {
  const auto cands = tc_candidates(n, cin, cout, batch);
  if (cands.empty()) return cudaErrorInvalidValue;
  std::vector<std::string> names;
  char buf[64];
  for (const auto &c : cands) {
    snprintf(buf, sizeof buf, "R=%d S=%d", c.first, c.second);
    names.push_back(buf);
  }
  snprintf(buf, sizeof buf, "conv_tc n=%d cin=%d cout=%d batch=%d", n, cin, cout, batch);
  const int pick = autotune::choose(buf, names, st, [&](int i) {
    return tc_launch_one(st, n, batch, cin, cout, X, Wtc, bias, Y, relu, err, cands[i].first,
                         cands[i].second);
  });
  return tc_launch_one(st, n, batch, cin, cout, X, Wtc, bias, Y, relu, err, cands[pick].first,
                       cands[pick].second);
}
