// Explicit instantiations of the pass kernels for a subset of the transform
// lengths (split across files so they compile in parallel).
#include "pass_kernels.cuh"

namespace cuvgls {
CUVGLS_INSTANTIATE_LEN(16)
CUVGLS_INSTANTIATE_LEN(32)
CUVGLS_INSTANTIATE_LEN(64)
CUVGLS_INSTANTIATE_LEN(80)
CUVGLS_INSTANTIATE_LEN(2048)
}  // namespace cuvgls
