// Transform kernels instantiated for length 4096.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_4096() {
  static const FsLaunchers L = make_fs_launchers<4096>();
  return &L;
}
const FdLaunchers* fd_launchers_4096() {
  static const FdLaunchers L = make_fd_launchers<4096>();
  return &L;
}
}  // namespace mgb
