/* implicit.h (GPU shim) — src/implicit.h:10 on libflipgpu. */
#ifndef FLIP3D_SHIM_IMPLICIT_H
#define FLIP3D_SHIM_IMPLICIT_H
#include "common.h"
#include "sorter.h"

namespace implicit {
double implicit_func(sorter *sort, FLOAT p[3], FLOAT density);
}
#endif
