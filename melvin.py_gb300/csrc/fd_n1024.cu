// Fourier-x / finite-difference-z kernels for length 1024 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_1024() {
  static const FdLaunchers L = make_fd_launchers<1024>();
  return &L;
}
}  // namespace mgb
