/*
 * ref_patch_rand.h — force-included (-include) into the reference's
 * src/corrector.cpp when oracle/Makefile builds oracle/_ref/libflipref.so.
 *
 * The corrector's close-pair kick draws rand() inside an OpenMP loop
 * (src/corrector.cpp:74-76). This header makes those three draws keyed,
 * thread-independent values from include/flip_rng.h, keyed on the indices of
 * the particle pair, so the reference, the CPU oracle and the CUDA kernels
 * draw the same numbers. At those lines the particle pointers `p` and `np` are
 * in scope; the harness allocates all particles in one array so a pointer
 * difference gives the particle index.
 *
 * Test infrastructure only (reference harness); not part of the product.
 */
#ifndef REF_PATCH_RAND_H
#define REF_PATCH_RAND_H
#include <stdlib.h>
#ifdef __cplusplus
#include <cstdlib>
extern "C" {
#endif
int flipref_kick_rand(const void *p, const void *np);
#ifdef __cplusplus
}
#endif
#define rand() flipref_kick_rand((const void *)p, (const void *)np)
#endif
