// Block-level Stockham FFT held in shared memory.
//
// A CTA transforms C interleaved columns of length N (a power of two) that
// sit in shared memory at buf[sx<T, CS>(x, c)] (x = position along the
// transform, c = column, CS >= C the interleave stride, a few pad elements
// every 8 rows).  Each pass is a radix-8, -4 or
// -2 butterfly computed in registers: a thread reads all R inputs of its
// butterflies, the CTA synchronises, and the thread writes the R outputs to
// the Stockham (self-sorting) positions, so the result ends in natural order
// without a bit-reversal pass.  Consecutive threads take consecutive columns
// of the same butterfly, so the reads of every pass are contiguous in shared
// memory.
//
// Twiddles come from a device table tw[t] = exp(-2*pi*i*t/N), t in [0, N),
// computed on the host in long double; the inverse direction uses their
// conjugates.  DIR = -1 is the forward transform exp(-...), DIR = +1 the
// unnormalised inverse exp(+...).
#pragma once

#include "common.cuh"

namespace mgb {

template <int R, int DIR, typename T>
__device__ __forceinline__ void dft4(cx<T>& a0, cx<T>& a1, cx<T>& a2, cx<T>& a3) {
  cx<T> t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_i<DIR>(a1 - a3);
  a0 = t0 + t2;
  a2 = t0 - t2;
  a1 = t1 + t3;
  a3 = t1 - t3;
}

template <int R, int DIR, typename T>
struct Dft;

template <int DIR, typename T>
struct Dft<2, DIR, T> {
  static __device__ __forceinline__ void run(cx<T>* a) {
    cx<T> t = a[0] - a[1];
    a[0] = a[0] + a[1];
    a[1] = t;
  }
};

template <int DIR, typename T>
struct Dft<4, DIR, T> {
  static __device__ __forceinline__ void run(cx<T>* a) { dft4<4, DIR>(a[0], a[1], a[2], a[3]); }
};

template <int DIR, typename T>
struct Dft<8, DIR, T> {
  // Radix-8 as two radix-4 halves (even / odd inputs) joined by the
  // eighth-roots of unity w^k, w = exp(DIR * 2*pi*i/8).
  static __device__ __forceinline__ void run(cx<T>* a) {
    const T s = (T)0.70710678118654752440084436210484903928;
    cx<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
    cx<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
    dft4<4, DIR>(e0, e1, e2, e3);
    dft4<4, DIR>(o0, o1, o2, o3);
    // o1 *= s (1 + DIR i); o2 *= DIR i; o3 *= s (-1 + DIR i)
    o1 = mk((o1.x - (T)DIR * o1.y) * s, (o1.y + (T)DIR * o1.x) * s);
    o2 = mul_i<DIR>(o2);
    o3 = mk((-o3.x - (T)DIR * o3.y) * s, (-o3.y + (T)DIR * o3.x) * s);
    a[0] = e0 + o0;
    a[4] = e0 - o0;
    a[1] = e1 + o1;
    a[5] = e1 - o1;
    a[2] = e2 + o2;
    a[6] = e2 - o2;
    a[3] = e3 + o3;
    a[7] = e3 - o3;
  }
};

// v * (cr + i ci) for a constant twiddle.
template <typename T>
__device__ __forceinline__ cx<T> ctw(cx<T> v, T cr, T ci) {
  return mk(v.x * cr - v.y * ci, v.x * ci + v.y * cr);
}

template <int DIR, typename T>
struct Dft<16, DIR, T> {
  // Radix-16 as 4 x 4: with n = n1 + 4 n2 and k = 4 k1 + k2,
  //   X[4 k1 + k2] = sum_n1 W4^(n1 k1) W16^(n1 k2) sum_n2 a[n1 + 4 n2] W4^(n2 k2),
  // W16 = exp(DIR * 2*pi*i/16): four DFT4 over n2, the twiddles W16^(n1 k2),
  // four DFT4 over n1.
  static __device__ __forceinline__ void run(cx<T>* a) {
    const T c1 = (T)0.92387953251128675612818318939678828682;  // cos(pi/8)
    const T s1 = (T)0.38268343236508977172845998403039886676;  // sin(pi/8)
    const T r = (T)0.70710678118654752440084436210484903928;   // cos(pi/4)
    const T d = (T)DIR;
    cx<T> y[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
      y[n1][0] = a[n1];
      y[n1][1] = a[n1 + 4];
      y[n1][2] = a[n1 + 8];
      y[n1][3] = a[n1 + 12];
      dft4<4, DIR>(y[n1][0], y[n1][1], y[n1][2], y[n1][3]);
    }
    // W16^e, e = n1 * k2: 1, 2, 3 | 2, 4, 6 | 3, 6, 9
    y[1][1] = ctw(y[1][1], c1, d * s1);
    y[1][2] = ctw(y[1][2], r, d * r);
    y[1][3] = ctw(y[1][3], s1, d * c1);
    y[2][1] = ctw(y[2][1], r, d * r);
    y[2][2] = mul_i<DIR>(y[2][2]);
    y[2][3] = ctw(y[2][3], -r, d * r);
    y[3][1] = ctw(y[3][1], s1, d * c1);
    y[3][2] = ctw(y[3][2], -r, d * r);
    y[3][3] = ctw(y[3][3], -c1, -(d * s1));
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      cx<T> z0 = y[0][k2], z1 = y[1][k2], z2 = y[2][k2], z3 = y[3][k2];
      dft4<4, DIR>(z0, z1, z2, z3);
      a[k2] = z0;
      a[4 + k2] = z1;
      a[8 + k2] = z2;
      a[12 + k2] = z3;
    }
  }
};

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Radix of the pass that starts with sub-transform length NS, at most RM
// (16 or 8).  The tail avoids a radix-2 pass: with RM = 8 a remaining length
// of 16 is split 4 x 4 rather than 8 x 2, with RM = 16 a remaining 32 is
// split 8 x 4 rather than 16 x 2.
template <int N, int NS, int RM>
struct PassRadix {
  static constexpr int rem = N / NS;
  static constexpr int value = (RM >= 16 && rem >= 16 && rem != 32)
                                   ? 16
                                   : ((rem >= 8 && rem != 16) ? 8 : (rem >= 4 ? 4 : 2));
};

// A pass's outputs as stored for the next pass: double-float values are
// renormalised (df_renorm), so the unnormalised low words that additions
// and products leave behind grow over one pass only.
template <typename T>
__device__ __forceinline__ cx<T> pass_out(cx<T> v) {
  return v;
}
template <>
__device__ __forceinline__ cx<df64> pass_out(cx<df64> v) {
  return mk(df_renorm(v.x), df_renorm(v.y));
}

template <typename T, int N, int C, int CS, int NT, int DIR, int R, int NS>
__device__ __forceinline__ void stockham_pass(cx<T>* buf, const cx<T>* __restrict__ tw) {
  constexpr int NB = C * (N / R);
  constexpr int BPT = (NB + NT - 1) / NT;
  constexpr int TWS = N / (R * NS);
  cx<T> v[BPT][R];
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = threadIdx.x + t * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, i = b / C;
#pragma unroll
      for (int r = 0; r < R; ++r) v[t][r] = buf[sx<T, CS>(i + r * (N / R), c)];
      if (NS > 1) {
        const int k = i & (NS - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const cx<T> w = tw[r * k * TWS];
          v[t][r] = DIR < 0 ? cmul(v[t][r], w) : cmulc(v[t][r], w);
        }
      }
      Dft<R, DIR, T>::run(v[t]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = threadIdx.x + t * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, i = b / C;
      const int k = i & (NS - 1);
      const int base = (i - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[sx<T, CS>(base + r * NS, c)] = pass_out(v[t][r]);
    }
  }
  __syncthreads();
}

template <typename T, int N, int C, int CS, int NT, int DIR, int RM, int NS, bool DONE = (NS >= N)>
struct FftPasses {
  static __device__ __forceinline__ void run(cx<T>* buf, const cx<T>* __restrict__ tw) {
    constexpr int R = PassRadix<N, NS, RM>::value;
    stockham_pass<T, N, C, CS, NT, DIR, R, NS>(buf, tw);
    FftPasses<T, N, C, CS, NT, DIR, RM, NS * R>::run(buf, tw);
  }
};

template <typename T, int N, int C, int CS, int NT, int DIR, int RM, int NS>
struct FftPasses<T, N, C, CS, NT, DIR, RM, NS, true> {
  static __device__ __forceinline__ void run(cx<T>*, const cx<T>* __restrict__) {}
};

// Transform columns [0, C) of buf (stride CS) in place with passes of radix
// at most RM; the caller must have synchronised after filling buf.  Ends
// with a __syncthreads().
template <typename T, int N, int C, int CS, int NT, int DIR, int RM = 8>
__device__ __forceinline__ void block_fft(cx<T>* buf, const cx<T>* __restrict__ tw) {
  static_assert((N & (N - 1)) == 0 && N >= 4, "power-of-two length");
  static_assert(RM == 16 || RM == 8, "maximum radix 16 or 8");
  FftPasses<T, N, C, CS, NT, DIR, RM, 1>::run(buf, tw);
}

}  // namespace mgb
