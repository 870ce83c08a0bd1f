// Explicit instantiations of the pass kernels for a subset of the transform
// lengths (split across files so they compile in parallel).
#include "pass_kernels.cuh"

namespace cuvgls {
CUVGLS_INSTANTIATE_LEN(640)
CUVGLS_INSTANTIATE_LEN(800)
CUVGLS_INSTANTIATE_LEN(1024)
}  // namespace cuvgls
