// Fourier-x / finite-difference-z kernels for length 64 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_64() {
  static const FdLaunchers L = make_fd_launchers<64>();
  return &L;
}
}  // namespace mgb
