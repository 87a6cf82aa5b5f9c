// Instantiations of the per-cell weak-form kernel for TET4 (nodes 4, quad points 1).
#include "fem_assemble.cuh"

namespace fem {
int assemble_tet4(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s) {
  return dispatch_material<4, 1>(P, vec, mat, precision, kmode, s);
}
}  // namespace fem
