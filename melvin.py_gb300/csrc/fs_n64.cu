// Transform kernels instantiated for length 64.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_64() {
  static const FsLaunchers L = make_fs_launchers<64>();
  return &L;
}
const FdLaunchers* fd_launchers_64() {
  static const FdLaunchers L = make_fd_launchers<64>();
  return &L;
}
}  // namespace mgb
