// Projection kernel instantiations for log2(fhtDim) in {7, 8}.
#include "project_impl.cuh"

namespace ceos {
template cudaError_t launch_project_L<7>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<8>(const ProjArgs&, int, int, cudaStream_t);
}  // namespace ceos
