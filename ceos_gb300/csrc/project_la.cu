// Projection kernel instantiations for log2(fhtDim) in {1, 2, 3, 4, 5, 6}.
#include "project_impl.cuh"

namespace ceos {
template cudaError_t launch_project_L<1>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<2>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<3>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<4>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<5>(const ProjArgs&, int, int, cudaStream_t);
template cudaError_t launch_project_L<6>(const ProjArgs&, int, int, cudaStream_t);
}  // namespace ceos
