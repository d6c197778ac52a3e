// Projection kernels: the reference's per-row projection block
// (src/CEOs.cpp:58-88, :343-372, :746-775; src/streamCEOs.cpp:55-86,
// :229-259) and its query twin (src/CEOs.cpp:143-161, :495-513, :895-913).
//
// One kernel body, three consumers of the projected values:
//   ROWS : row-major [rows][R*D]            (query projections)
//   COLS : column-major [slot][ld]          (dense CEOs-Est index; sample and
//                                            fallback dumps of chosen columns)
//   EMIT : no projection matrix at all. Each value is compared against the
//          per-column selection thresholds of the bucket build and, when it
//          can still be among the column's top-m (close end) or bottom-m
//          (far end), its packed (value, id) key is appended to that column
//          end's candidate list. This fuses the projection with the first
//          pass of the two-ended top-m selection (src/CEOs.cpp:377-432), so
//          the n x (R*D) projection matrix never travels to HBM.
#include "kernels.h"

namespace ceos {

template <int L>
cudaError_t launch_project_L(const ProjArgs& a, int mode, int num_sms, cudaStream_t st);

cudaError_t launch_project(const ProjArgs& a, int mode, int L, int num_sms, cudaStream_t st) {
  if (a.n_rows <= 0) return cudaSuccess;
  if (a.tensor && project_tc_supported(L)) return launch_project_tc(a, mode, L, num_sms, st);
  switch (L) {
    case 1: return launch_project_L<1>(a, mode, num_sms, st);
    case 2: return launch_project_L<2>(a, mode, num_sms, st);
    case 3: return launch_project_L<3>(a, mode, num_sms, st);
    case 4: return launch_project_L<4>(a, mode, num_sms, st);
    case 5: return launch_project_L<5>(a, mode, num_sms, st);
    case 6: return launch_project_L<6>(a, mode, num_sms, st);
    case 7: return launch_project_L<7>(a, mode, num_sms, st);
    case 8: return launch_project_L<8>(a, mode, num_sms, st);
    case 9: return launch_project_L<9>(a, mode, num_sms, st);
    case 10: return launch_project_L<10>(a, mode, num_sms, st);
    case 11: return launch_project_L<11>(a, mode, num_sms, st);
    case 12: return launch_project_L<12>(a, mode, num_sms, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ceos
