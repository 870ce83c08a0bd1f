// Explicit instantiations of the pass-2 kernels for the row-only length
// 4096 (compiled in parallel with the other lengths).
#include "pass_kernels.cuh"

namespace cuvgls {
CUVGLS_INSTANTIATE_ROW_LEN(4096)
}  // namespace cuvgls
