// Projection kernel instantiations for log2(fhtDim) in {9}.
#include "project_impl.cuh"

namespace ceos {
template cudaError_t launch_project_L<9>(const ProjArgs&, int, int, cudaStream_t);
}  // namespace ceos
