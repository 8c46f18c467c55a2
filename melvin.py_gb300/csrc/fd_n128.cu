// Fourier-x / finite-difference-z kernels for length 128 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_128() {
  static const FdLaunchers L = make_fd_launchers<128>();
  return &L;
}
}  // namespace mgb
