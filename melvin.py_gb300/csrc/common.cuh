// Shared device/host definitions for the Melvin GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "melvin_gb300.h"

namespace mgb {

// Interleaved complex value with the scalar type of the arithmetic.
template <typename T>
struct __align__(2 * sizeof(T)) cx {
  T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename T>
__device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T>
__device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename T>
__device__ __forceinline__ cx<T> operator*(cx<T> a, T s) { return mk(a.x * s, a.y * s); }
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
  return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> conj(cx<T> a) { return mk(a.x, -a.y); }
// multiply by -i (DIR < 0) or +i (DIR > 0)
template <int DIR, typename T>
__device__ __forceinline__ cx<T> mul_i(cx<T> a) {
  return DIR > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x);
}

template <typename To, typename From>
__device__ __forceinline__ cx<To> cvt(cx<From> a) {
  return mk((To)a.x, (To)a.y);
}

typedef cx<double> zd;

// Which device field a fused kernel reads when it forms a spectral input.
enum SrcKind : int {
  SRC_COPY = 0,   // the state itself
  SRC_UX = 1,     // ux = -d/dz psi, psi = solve(-w)
  SRC_UZ = 2,     // uz = +d/dx psi
};

// Grid constants shared by all kernels of a plan.
struct GridC {
  int nx, nz;       // physical points
  int nn, nm;       // kept modes (nm = nz for FDM-z)
  int rows;         // spectral rows: 2nn+1 (fully spectral) or nn (FDM-z)
  int cols;         // spectral columns: nm (fully spectral) or nz (FDM-z)
  int fdm;          // 1 when z is a Dirichlet finite-difference axis
  int sdo;          // 2 or 4
  double dx, dz;
  double dfx, dfz;  // 2*pi/lx, 2*pi/lz (imaginary part of the derivative factor)
  double d2x, d2z;  // -(2*pi)^2/lx^2, -(2*pi)^2/lz^2
};

// Spectral row r of the (2nn+1)-row block -> signed mode number n.
__host__ __device__ __forceinline__ int row_mode(int r, int nn) { return r <= nn ? r : r - (2 * nn + 1); }
// Spectral row r -> index in a full length-N transform.
__host__ __device__ __forceinline__ int row_bin(int r, int nn, int N) { return r <= nn ? r : N - (2 * nn + 1 - r); }

}  // namespace mgb
