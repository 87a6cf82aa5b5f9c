// Instantiations of the per-cell weak-form kernel for HEX8 (nodes 8, quad points 8).
#include "fem_assemble.cuh"

namespace fem {
int assemble_hex8(const AsmParams& P, int vec, int mat, int precision, int kmode, cudaStream_t s) {
  return dispatch_material<8, 8>(P, vec, mat, precision, kmode, s);
}
}  // namespace fem
