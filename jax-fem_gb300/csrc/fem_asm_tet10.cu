// Instantiations of the per-cell weak-form kernel for TET10 (nodes 10, quad points 4).
#include "fem_assemble.cuh"

namespace fem {
int assemble_tet10(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s) {
  return dispatch_material<10, 4>(P, vec, mat, precision, kmode, s);
}
}  // namespace fem
