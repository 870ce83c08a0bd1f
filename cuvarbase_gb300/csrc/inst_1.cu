// Explicit instantiations of the pass kernels for a subset of the transform
// lengths (split across files so they compile in parallel).
#include "pass_kernels.cuh"

namespace cuvgls {
CUVGLS_INSTANTIATE_LEN(128)
CUVGLS_INSTANTIATE_LEN(160)
CUVGLS_INSTANTIATE_LEN(256)
CUVGLS_INSTANTIATE_LEN(1600)
}  // namespace cuvgls
