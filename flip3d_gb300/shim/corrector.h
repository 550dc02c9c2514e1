/* corrector.h (GPU shim) — src/corrector.h:8-11 on libflipgpu, plus the
 * seed/step of the keyed random draws that replace rand(). */
#include <stdint.h>
#include <vector>

#include "common.h"
#include "sorter.h"

namespace corrector {
void resample(sorter *sort, FLOAT p[3], FLOAT u[3], FLOAT re);
void correct(sorter *sort, std::vector<particle *> &particle, FLOAT dt, FLOAT re);
void setRandomKey(uint64_t seed, int64_t step);
}
