// Fourier-x / finite-difference-z kernels for length 2048 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_2048() {
  static const FdLaunchers L = make_fd_launchers<2048>();
  return &L;
}
}  // namespace mgb
