// Transform kernels instantiated for length 256.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_256() {
  static const FsLaunchers L = make_fs_launchers<256>();
  return &L;
}
const FdLaunchers* fd_launchers_256() {
  static const FdLaunchers L = make_fd_launchers<256>();
  return &L;
}
}  // namespace mgb
