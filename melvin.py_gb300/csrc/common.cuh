// Shared device/host definitions for the Melvin GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "df64.cuh"
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
__device__ __forceinline__ cx<T> operator-(cx<T> a) { return mk(-a.x, -a.y); }
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
struct Cvt {
  static __device__ __forceinline__ To run(From v) { return (To)v; }
};

// Precision conversions on the integer pipes.  GB300 executes F2F
// conversions on its narrow FP64 pipe, where they cost as much as the FP32
// transform they feed, so the conversions at the FP64-state / reduced
// precision boundary are done on the bit patterns instead.

// double -> float, round to nearest (ties away from zero); magnitudes below
// the smallest normal float flush to signed zero, above FLT_MAX become inf.
// Works on the two 32-bit halves so that no step can be lowered to an FP64
// instruction.
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned int hi = (unsigned int)__double2hiint(d), lo = (unsigned int)__double2loint(d);
  const unsigned int sign = hi & 0x80000000u;
  const unsigned int lo2 = lo + (1u << 28);
  const unsigned int hm = (hi & 0x7fffffffu) + (lo2 < lo ? 1u : 0u);
  const int e = (int)(hm >> 20) - 896;
  const unsigned int m = ((hm & 0xfffffu) << 3) | (lo2 >> 29);
  const unsigned int bits = e <= 0 ? 0u : (e >= 255 ? 0x7f800000u : (((unsigned int)e << 23) | m));
  return __uint_as_float(bits | sign);
}

// float -> double, exact (float subnormals flush to zero).
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int sign = b & 0x80000000u;
  const unsigned int e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  unsigned int hi, lo;
  if (e == 0) {
    hi = 0u;
    lo = 0u;
  } else if (e == 255) {
    hi = 0x7ff00000u | (m >> 3);
    lo = m << 29;
  } else {
    hi = ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double((int)(hi | sign), (int)lo);
}

// double -> double-float: hi = the significand truncated to 24 bits, lo = the
// remaining 29 bits rounded to a float (48 significant bits in all).
__device__ __forceinline__ df64 d2df_bits(double d) {
  const unsigned int h = (unsigned int)__double2hiint(d), l = (unsigned int)__double2loint(d);
  const unsigned int sign = h & 0x80000000u;
  const int e = (int)((h >> 20) & 0x7ffu);
  const int ef = e - 896;
  if (ef <= 0) return df64(__uint_as_float(sign), 0.0f);
  if (ef >= 255) return df64(__uint_as_float(sign | 0x7f800000u), 0.0f);
  const unsigned int m = ((h & 0xfffffu) << 3) | (l >> 29);
  const float hi = __uint_as_float(sign | ((unsigned int)ef << 23) | m);
  const unsigned int rem = l & 0x1fffffffu;  // value rem * 2^(e-1075)
  const int es = e - 1075 + 127;              // biased exponent of 2^(e-1075)
  float lo = 0.0f;
  if (es > 0) lo = __uint2float_rn(rem) * __uint_as_float((unsigned int)es << 23);
  return df64(hi, sign ? -lo : lo);
}

template <>
struct Cvt<float, double> {
  static __device__ __forceinline__ float run(double v) { return d2f_bits(v); }
};
template <>
struct Cvt<double, float> {
  static __device__ __forceinline__ double run(float v) { return f2d_bits(v); }
};
template <>
struct Cvt<df64, double> {
  static __device__ __forceinline__ df64 run(double v) { return d2df_bits(v); }
};
template <>
struct Cvt<double, df64> {
  static __device__ __forceinline__ double run(df64 v) { return f2d_bits(v.hi) + f2d_bits(v.lo); }
};

template <typename To, typename From>
__device__ __forceinline__ cx<To> cvt(cx<From> a) {
  return mk(Cvt<To, From>::run(a.x), Cvt<To, From>::run(a.y));
}

// A double kernel argument (a grid constant, a stencil or scale factor) in
// the kernel's arithmetic type T.  FP32 goes through the integer-pipe
// conversion: every thread converts its constants, and the hardware
// conversion would take FP64-pipe slots from the FP64 update that shares
// the kernel (split 2048^2 forward x pass 43.4 -> 39.0 us with the psi fix).
// Double-float keeps its constructor (measured 1.5 us faster there).
template <typename T>
__device__ __forceinline__ T to_t(double v) {
  if constexpr (std::is_same<T, float>::value) {
    return Cvt<T, double>::run(v);
  } else {
    return T(v);
  }
}

// Shared-memory FFT buffers of complex T hold column c of row x at
// x*CS + c + (x/8)*PAD.  The padding breaks the bank conflicts of the
// strided Stockham accesses (the first pass stores rows 8 apart; a block
// transform maps consecutive threads to consecutive columns, then rows).
// Shared memory serves 8-byte accesses in half-warp phases and 16-byte ones
// in quarter-warp phases, and the padding that makes consecutive 8-row
// blocks tile the 32 banks is
//   16-byte elements: PAD = CS mod 8 (conflict free for every CS);
//   8-byte elements:  PAD = CS mod 16 for even CS (conflict free), 1 for
//                     CS = 1 and 0 for other odd CS (about 1.3 wavefronts per
//                     request either way, so the smaller buffer is kept),
// found by replaying every pass's addresses against the bank model.  The
// buffer grows by at most one eighth.
// A kernel whose other phases access the buffer row by row (a thread per
// row, as in the z pass) names an explicit stride and pad instead: the
// layout argument L is then CS + kPadCode * (PAD + 1); a plain column count
// L < kPadCode takes the rule above.
template <typename T, int CS>
struct SmemPad {
  static constexpr int value =
      sizeof(cx<T>) >= 16 ? CS % 8 : (CS % 2 == 0 ? CS % 16 : (CS == 1 ? 1 : 0));
};
constexpr int kPadCode = 1 << 12;
template <int CS, int PAD>
struct ExplicitLayout {
  static constexpr int value = CS + kPadCode * (PAD + 1);
};
template <typename T, int L>
struct SmemLayout {
  static constexpr int CS = L % kPadCode;
  static constexpr int PAD = L / kPadCode ? L / kPadCode - 1 : SmemPad<T, CS>::value;
};
template <typename T, int L>
__host__ __device__ __forceinline__ int sx(int x, int c) {
  return x * SmemLayout<T, L>::CS + c + (x >> 3) * SmemLayout<T, L>::PAD;
}
// Elements of a padded buffer of N rows.
template <typename T, int L>
__host__ __device__ constexpr int sbuf_elems(int N) {
  return N * SmemLayout<T, L>::CS + (N / 8) * SmemLayout<T, L>::PAD + 1;
}

typedef cx<double> zd;

// Device-side run control of a step launched by the run driver
// (mgb_run_step): every kernel of the step returns at once when the run
// stopped before iteration `loop` (CFL breach or final time reached), and
// the explicit / PECE update of the Dirichlet path reads dt from the run
// state.  A default Gate (null pointers) is always open.
struct Gate {
  const long long* stop_at = nullptr;  // run state: first iteration not to run
  long long loop = 0;                  // iteration index of this step
  const double* dt = nullptr;          // run state: current dt
};
__device__ __forceinline__ bool gate_closed(const Gate& g) { return g.stop_at != nullptr && g.loop >= *g.stop_at; }

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
  // Basis of each axis for the spectral derivative verbs: 0 complex
  // exponential (factor i*dfx*n), 1 cosine / 2 sine (real factor dfx*n, with
  // dfx = -pi/lx or pi/lx and d2x = -pi^2/lx^2, melvin/BasisFunctions.py:26-59).
  int bx = 0, bz = 0;
};

// Spectral row r of the (2nn+1)-row block -> signed mode number n.
__host__ __device__ __forceinline__ int row_mode(int r, int nn) { return r <= nn ? r : r - (2 * nn + 1); }
// Spectral row r -> index in a full length-N transform.
__host__ __device__ __forceinline__ int row_bin(int r, int nn, int N) { return r <= nn ? r : N - (2 * nn + 1 - r); }

}  // namespace mgb
