/* mesher.h (GPU shim) — src/mesher.h:8-11 on libflipgpu. The mesh is built on
 * the GPU from the sorter's lists (mg must be the sorter's grid size + 1, as
 * src/flip3D.cpp:1002 passes) and copied into the caller's vectors. */
#ifndef FLIP3D_SHIM_MESHER_H
#define FLIP3D_SHIM_MESHER_H
#include <vector>

#include "common.h"
#include "sorter.h"

namespace mesher {
void generateMesh(char ***A, sorter *sort, std::vector<particle *> &particles, FLOAT density,
                  int mg, std::vector<double> &vertices, std::vector<double> &normals,
                  std::vector<int> &faces);
}
#endif
