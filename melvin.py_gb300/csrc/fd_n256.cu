// Fourier-x / finite-difference-z kernels for length 256 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_256() {
  static const FdLaunchers L = make_fd_launchers<256>();
  return &L;
}
}  // namespace mgb
