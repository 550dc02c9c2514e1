/*
 * flip_rng.h — counter-based random numbers shared by the CUDA kernels, the
 * CPU oracle, the reference harness and the Python scene builder.
 *
 * The reference draws rand() inside OpenMP loops (src/corrector.cpp:74-76),
 * in reposition (src/flip3D.cpp:438-440) and through random_shuffle
 * (src/utility.cpp:28-30), so its results depend on thread scheduling and on
 * the libc generator. Every implementation here instead derives each draw
 * from a key (seed, stream, a, b) with no shared state, so a draw is the same
 * on any thread, on the GPU and on the host. The mixing function is the
 * public SplitMix64 finaliser.
 *
 * Streams (the top byte of `stream` selects the use, the rest carries the
 * step and the component):
 *   FLIP_RNG_SEED    scene seeding jitter       a = lattice index, b = 0
 *   FLIP_RNG_KICK    corrector close-pair kick  a = particle, b = neighbour
 *   FLIP_RNG_PLACE   reposition placement       a = ordinal of the draw
 *   FLIP_RNG_SHUFFLE reposition shuffle         a = swap position
 */
#ifndef FLIP_RNG_H
#define FLIP_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define FLIP_RNG_FN static __host__ __device__ __forceinline__
#else
#define FLIP_RNG_FN static inline
#endif

#define FLIP_RNG_SEED 1ull
#define FLIP_RNG_KICK 2ull
#define FLIP_RNG_PLACE 3ull
#define FLIP_RNG_SHUFFLE 4ull

FLIP_RNG_FN uint64_t flip_mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}

/* stream = (use << 56) | (step << 8) | component */
FLIP_RNG_FN uint64_t flip_stream(uint64_t use, uint64_t step, uint64_t comp) {
  return (use << 56) | ((step & 0xffffffffffull) << 8) | (comp & 0xffull);
}

/* 31-bit non-negative draw, the range of glibc rand(). */
FLIP_RNG_FN uint32_t flip_rand31(uint64_t seed, uint64_t stream, uint64_t a,
                                 uint64_t b) {
  uint64_t h = flip_mix64(seed ^ 0x9e3779b97f4a7c15ull);
  h = flip_mix64(h ^ stream);
  h = flip_mix64(h + a);
  h = flip_mix64(h + (b ^ 0x632be59bd9b4e019ull));
  return (uint32_t)(h >> 33);
}

#endif /* FLIP_RNG_H */
