// Explicit instantiations of the pass kernels for a subset of the transform
// lengths (split across files so they compile in parallel).
#include "pass_kernels.cuh"

namespace cuvgls {
CUVGLS_INSTANTIATE_LEN(320)
CUVGLS_INSTANTIATE_LEN(400)
CUVGLS_INSTANTIATE_LEN(512)
CUVGLS_INSTANTIATE_LEN(1280)
}  // namespace cuvgls
