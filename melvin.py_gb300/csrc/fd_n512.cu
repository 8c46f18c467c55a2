// Fourier-x / finite-difference-z kernels for length 512 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_512() {
  static const FdLaunchers L = make_fd_launchers<512>();
  return &L;
}
}  // namespace mgb
