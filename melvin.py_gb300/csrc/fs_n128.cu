// Transform kernels instantiated for length 128.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_128() {
  static const FsLaunchers L = make_fs_launchers<128>();
  return &L;
}
const FdLaunchers* fd_launchers_128() {
  static const FdLaunchers L = make_fd_launchers<128>();
  return &L;
}
}  // namespace mgb
