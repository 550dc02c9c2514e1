/* solver.h (GPU shim) — src/solver.h:9-12 on libflipgpu, plus the relative
 * tolerance setting the benchmarks use (the reference stops at r.r <=
 * 1e-2*n^3; setRelativeTolerance(0) keeps that). */
#include "common.h"

namespace solver {
void setSubcell(char value);
void solve(char ***A, FLOAT ***L, FLOAT ***x, FLOAT ***b, int n);
void setRelativeTolerance(double rel_tol);
}
