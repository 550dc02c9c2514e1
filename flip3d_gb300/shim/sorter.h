/*
 * sorter.h (GPU shim) — class sorter with the member functions a flip3d
 * driver calls (src/sorter.h:11-29), backed by libflipgpu: sort() bins on the
 * GPU and keeps the resulting cell lists, which the neighbour queries read.
 * The include guard is the reference header's, so force-including this file
 * (-include) ahead of a driver replaces the reference's declaration.
 */
#ifndef _SORTER_H
#define _SORTER_H

#include <vector>

#include "common.h"

struct FlipShimCells;

class sorter {
public:
  sorter(int gn);
  ~sorter();

  void sort(std::vector<particle *> &particles);
  std::vector<particle *> getNeigboringParticles_wall(int i, int j, int k, int w, int h, int d);
  std::vector<particle *> getNeigboringParticles_cell(int i, int j, int k, int w, int h, int d);
  FLOAT levelset(int i, int j, int k, FLOAT ***halfwall, FLOAT density);

  int getCellSize() { return gn; }
  int getNumParticleAt(int i, int j, int k);
  void markWater(char ***A, FLOAT ***halfwall, FLOAT density);
  void deleteAllParticles();

  /* shim access for the other entry points (not part of the driver's API) */
  FlipShimCells *shim() { return cells_; }

protected:
  FlipShimCells *cells_;
  int gn;
};

#endif
