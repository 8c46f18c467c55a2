// Shared pieces of the cosine / sine basis transforms
// (melvin/SpectralTransformer.py:90-199): the argument block, the placement
// of kept rows in a transform and the mirror extension of a line.  Used by
// mirror.cu (power-of-two transform lengths) and bluestein.cu (any length).
#pragma once

#include "spectral2d_impl.cuh"

namespace mgb {

// Columns per CTA of an x pass over a length-L (or length-M convolution)
// buffer: 4096 complex values.
template <int L>
struct MTile {
  static constexpr int C0 = 4096 / L;
  static constexpr int C = C0 < 1 ? 1 : (C0 > 64 ? 64 : C0);
};

struct MirrorArgs {
  GridC g;
  int nxp, nzp;          // physical extents
  int lx, lz;            // transform lengths
  int bx, bz;            // basis of each axis (0 exp, 1 cosine, 2 sine)
  zd scale;              // to_physical: product of the per-axis factors; to_spectral: 1/(x_factor z_factor)
  const zd* spec_in;
  zd* spec_out;
  const double* phys_in;
  double* phys_out;
  zd* inter;             // [nxp][nm]
  const void* twx;
  const void* twz;
};

__device__ __forceinline__ zd cmuld(zd a, zd b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// Position of kept spectral row r in a length-L x transform (rows 0..nn, then
// the last nn bins), as _scale_2d places them (melvin/SpectralTransformer.py:21-24).
__device__ __forceinline__ int mbin(int r, int nn, int L) { return r <= nn ? r : L - (2 * nn + 1 - r); }

// Mirror extension of a line of n points to L = 2(n-1) (sign s: +1 cosine,
// -1 sine): j < n-1 -> v[j], j >= n-1 -> s * v[L-j]; an exp axis (L = n) is
// the line itself.
__device__ __forceinline__ int mirror_src(int j, int n, int L, int basis, double& sign) {
  sign = 1.0;
  if (basis == 0 || j < n - 1) return j;
  sign = basis == 2 ? -1.0 : 1.0;
  return L - j;
}

// Tables of a length-L DFT computed as a Bluestein convolution of
// power-of-two length M >= 2L - 1 (bluestein.cu): the chirp
// c_j = exp(-pi i (j^2 mod 2L) / L), j < L, and the transforms of the
// convolution kernels divided by M, for the forward (exp(-...)) and the
// unnormalised inverse (exp(+...)) DFT.
struct BlueTables {
  int L = 0, M = 0;
  const zd* chirp = nullptr;   // [L]
  const zd* bhat_f = nullptr;  // [M]
  const zd* bhat_i = nullptr;  // [M]
  const void* tw = nullptr;    // twiddles of length M
};

// The Bluestein kernels: which = 0 x inverse, 1 z inverse, 2 z forward,
// 3 x forward, as launch_mirror; b describes the axis the pass transforms.
cudaError_t launch_bluestein(int which, const MirrorArgs& a, const BlueTables& b, cudaStream_t s);
// The tables of length L (cached in the plan).
int bluestein_tables(const mgb_plan* p, int L, BlueTables& b);

}  // namespace mgb
