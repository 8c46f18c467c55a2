// Transform kernels instantiated for length 32.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_32() {
  static const FsLaunchers L = make_fs_launchers<32>();
  return &L;
}
const FdLaunchers* fd_launchers_32() {
  static const FdLaunchers L = make_fd_launchers<32>();
  return &L;
}
}  // namespace mgb
