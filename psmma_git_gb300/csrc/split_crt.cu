// Split path (exact modular slices on BF16 tensor cores).  Under construction: reports
// PSMMA_EUNSUPPORTED until the tcgen05 kernels land.
#include "psmma_internal.h"

namespace psmma {

size_t split_workspace_bytes(int, int, int, int) { return 0; }

int launch_split(int, int, int, double, const double*, long, const double*, long, double, double*,
                 long, int, void*, size_t, cudaStream_t) {
  return PSMMA_EUNSUPPORTED;
}

}  // namespace psmma
