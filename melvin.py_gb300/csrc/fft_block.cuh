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

// ---------------------------------------------------------------------------
// Butterflies with the twiddle products folded into FMAs (FP32 and FP64).
// A DIT butterfly pair a + w v, a - w v computes the first as two chained
// FMAs per component, t = fma(w.x, v.x, fma(-w.y, v.y, a.x)), and the second
// as 2a - t (one FMA per component): 6 instructions where a separate
// complex product and two additions take 8.  The sqrt(1/2) products of the
// radix-8 odd terms fold into the final additions the same way.  Twiddled
// radix-8: 72 FP instructions instead of 84; radix 4: 24 instead of 28.
// Double-float keeps the plain form (its products are not fused).
// ---------------------------------------------------------------------------

__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmx(double a, double b, double c) { return fma(a, b, c); }

// v * w (DIR < 0) or v * conj(w) (DIR > 0)
template <int DIR, typename T>
__device__ __forceinline__ cx<T> tw_mul(cx<T> v, cx<T> w) {
  return DIR < 0 ? mk(fmx(v.x, w.x, -(v.y * w.y)), fmx(v.x, w.y, v.y * w.x))
                 : mk(fmx(v.x, w.x, v.y * w.y), fmx(v.y, w.x, -(v.x * w.y)));
}
// a + v * w (DIR < 0) or a + v * conj(w) (DIR > 0)
template <int DIR, typename T>
__device__ __forceinline__ cx<T> tw_fma(cx<T> a, cx<T> v, cx<T> w) {
  return DIR < 0 ? mk(fmx(w.x, v.x, fmx(-w.y, v.y, a.x)), fmx(w.x, v.y, fmx(w.y, v.x, a.y)))
                 : mk(fmx(w.x, v.x, fmx(w.y, v.y, a.x)), fmx(w.x, v.y, fmx(-w.y, v.x, a.y)));
}
// 2a - t
template <typename T>
__device__ __forceinline__ cx<T> twice_minus(cx<T> a, cx<T> t) {
  return mk(fmx((T)2, a.x, -t.x), fmx((T)2, a.y, -t.y));
}

// Twiddled butterflies: a[r] *= w[r-1] (conjugated for DIR > 0) for r >= 1,
// then the radix-R DFT, fused.  TW = false: no twiddles (w unused).
template <int R, int DIR, typename T, bool TW>
struct FDft;

template <int DIR, typename T, bool TW>
struct FDft<4, DIR, T, TW> {
  static __device__ __forceinline__ void run(cx<T>* a, const cx<T>* w) {
    if constexpr (!TW) {
      dft4<4, DIR>(a[0], a[1], a[2], a[3]);
    } else {
      const cx<T> t0 = tw_fma<DIR>(a[0], a[2], w[1]);        // a0 + W2 a2
      const cx<T> t1 = twice_minus(a[0], t0);                 // a0 - W2 a2
      const cx<T> p = tw_mul<DIR>(a[1], w[0]);                // W1 a1
      const cx<T> t2 = tw_fma<DIR>(p, a[3], w[2]);            // W1 a1 + W3 a3
      const cx<T> t3 = mul_i<DIR>(twice_minus(p, t2));        // (W1 a1 - W3 a3) * (+-i)
      a[0] = t0 + t2;
      a[2] = t0 - t2;
      a[1] = t1 + t3;
      a[3] = t1 - t3;
    }
  }
};

template <int DIR, typename T, bool TW>
struct FDft<8, DIR, T, TW> {
  static __device__ __forceinline__ void run(cx<T>* a, const cx<T>* w) {
    const T s = (T)0.70710678118654752440084436210484903928;
    cx<T> t0, t1, t2, t3, u0, u1, u2, u3;
    if constexpr (TW) {
      // even inputs 0, 2, 4, 6 (twiddles w[1], w[3], w[5])
      t0 = tw_fma<DIR>(a[0], a[4], w[3]);
      t1 = twice_minus(a[0], t0);
      const cx<T> p = tw_mul<DIR>(a[2], w[1]);
      t2 = tw_fma<DIR>(p, a[6], w[5]);
      t3 = mul_i<DIR>(twice_minus(p, t2));
      // odd inputs 1, 3, 5, 7 (twiddles w[0], w[2], w[4], w[6])
      const cx<T> p1 = tw_mul<DIR>(a[1], w[0]);
      u0 = tw_fma<DIR>(p1, a[5], w[4]);
      u1 = twice_minus(p1, u0);
      const cx<T> p3 = tw_mul<DIR>(a[3], w[2]);
      u2 = tw_fma<DIR>(p3, a[7], w[6]);
      u3 = mul_i<DIR>(twice_minus(p3, u2));
    } else {
      t0 = a[0] + a[4];
      t1 = a[0] - a[4];
      t2 = a[2] + a[6];
      t3 = mul_i<DIR>(a[2] - a[6]);
      u0 = a[1] + a[5];
      u1 = a[1] - a[5];
      u2 = a[3] + a[7];
      u3 = mul_i<DIR>(a[3] - a[7]);
    }
    const cx<T> e0 = t0 + t2, e2 = t0 - t2, e1 = t1 + t3, e3 = t1 - t3;
    const cx<T> o0 = u0 + u2, o2 = mul_i<DIR>(u0 - u2), o1 = u1 + u3, o3 = u1 - u3;
    // a[1] = e1 + s (1 + DIR i) o1, a[3] = e3 + s (-1 + DIR i) o3 (and minus for +4)
    const T d1x = o1.x - (T)DIR * o1.y, d1y = o1.y + (T)DIR * o1.x;
    const T d3x = -o3.x - (T)DIR * o3.y, d3y = -o3.y + (T)DIR * o3.x;
    a[0] = e0 + o0;
    a[4] = e0 - o0;
    a[2] = e2 + o2;
    a[6] = e2 - o2;
    a[1] = mk(fmx(s, d1x, e1.x), fmx(s, d1y, e1.y));
    a[5] = mk(fmx(-s, d1x, e1.x), fmx(-s, d1y, e1.y));
    a[3] = mk(fmx(s, d3x, e3.x), fmx(s, d3y, e3.y));
    a[7] = mk(fmx(-s, d3x, e3.x), fmx(-s, d3y, e3.y));
  }
};

// Whether a radix and type take the fused butterflies.
template <int R, typename T>
struct Fused {
  static constexpr bool value = (R == 8 || R == 4) && (std::is_same<T, float>::value || std::is_same<T, double>::value);
};

// Radix-8 DFT (no twiddles) of inputs whose a[3] and a[4] are zero: the
// first pass of an inverse transform of 2/3-rule data, where the inputs
// 3N/8 .. 5N/8 - 1 lie in the band of removed modes.  44 FP instructions
// instead of 52 (fused types) and two fewer loads; the outputs equal the
// full butterfly's (an addition of an exact zero returns the other operand,
// up to the sign of a zero result).
template <int DIR, typename T>
__device__ __forceinline__ void dft8_zero34(cx<T>* a) {
  const T s = (T)0.70710678118654752440084436210484903928;
  const cx<T> t2 = a[2] + a[6], t3 = mul_i<DIR>(a[2] - a[6]);
  const cx<T> u0 = a[1] + a[5], u1 = a[1] - a[5], m7 = mul_i<DIR>(a[7]);
  const cx<T> e0 = a[0] + t2, e2 = a[0] - t2, e1 = a[0] + t3, e3 = a[0] - t3;
  const cx<T> o0 = u0 + a[7], o2 = mul_i<DIR>(u0 - a[7]), o1 = u1 - m7, o3 = u1 + m7;
  a[0] = e0 + o0;
  a[4] = e0 - o0;
  a[2] = e2 + o2;
  a[6] = e2 - o2;
  if constexpr (Fused<8, T>::value) {
    const T d1x = o1.x - (T)DIR * o1.y, d1y = o1.y + (T)DIR * o1.x;
    const T d3x = -o3.x - (T)DIR * o3.y, d3y = -o3.y + (T)DIR * o3.x;
    a[1] = mk(fmx(s, d1x, e1.x), fmx(s, d1y, e1.y));
    a[5] = mk(fmx(-s, d1x, e1.x), fmx(-s, d1y, e1.y));
    a[3] = mk(fmx(s, d3x, e3.x), fmx(s, d3y, e3.y));
    a[7] = mk(fmx(-s, d3x, e3.x), fmx(-s, d3y, e3.y));
  } else {
    const cx<T> p1 = mk((o1.x - (T)DIR * o1.y) * s, (o1.y + (T)DIR * o1.x) * s);
    const cx<T> p3 = mk((-o3.x - (T)DIR * o3.y) * s, (-o3.y + (T)DIR * o3.x) * s);
    a[1] = e1 + p1;
    a[5] = e1 - p1;
    a[3] = e3 + p3;
    a[7] = e3 - p3;
  }
}

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Double-float passes are long (about 700 FP32 instructions per twiddled
// radix-8 butterfly).  Its transforms with maximum radix 8 put the radix-4
// passes first (2048 = 4 x 8 x 8 x 8) and run the radix-8 passes that follow
// as one copy of the code, looped over a runtime sub-transform length, so
// that the kernels' code fits the instruction caches.
template <typename T>
struct LoopedPasses {
  static constexpr bool value = std::is_same<T, df64>::value;
};

// Radix of the pass that starts with sub-transform length NS, at most RM
// (16 or 8).  The tail avoids a radix-2 pass: with RM = 8 a remaining length
// of 16 is split 4 x 4 rather than 8 x 2, with RM = 16 a remaining 32 is
// split 8 x 4 rather than 16 x 2.  small_first (double-float, RM = 8): the
// radix-4 passes come first instead.
__host__ __device__ constexpr int pass_radix(int N, int NS, int RM, bool small_first = false) {
  if (small_first && RM == 8) {
    // log2 N mod 3 = 0: all radix 8; 2: one radix-4 pass first; 1: two
    const int L = ilog2c(N), lead = L % 3 == 0 ? 0 : (L % 3 == 2 ? 1 : 2);
    return ilog2c(NS) < 2 * lead ? 4 : 8;
  }
  return (RM >= 16 && N / NS >= 16 && N / NS != 32) ? 16
                                                    : ((N / NS >= 8 && N / NS != 16) ? 8 : (N / NS >= 4 ? 4 : 2));
}
template <typename T, int N, int NS, int RM>
struct PassRadix {
  static constexpr int value = pass_radix(N, NS, RM, LoopedPasses<T>::value);
};

// First sub-transform length at or after NS whose pass is not radix 8.
__host__ __device__ constexpr int radix8_run_end(int N, int NS, int RM, bool small_first) {
  while (NS < N && pass_radix(N, NS, RM, small_first) == 8) NS *= 8;
  return NS;
}

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

// Whether the first pass of a length-N transform of T with maximum radix RM
// skips the inputs 3N/8 .. 5N/8 - 1 when the caller marks them zero (ZB):
// only a radix-8 first pass does, and the caller then need not fill them.
template <typename T, int N, int RM, bool ZB>
struct ZeroBand {
  static constexpr bool value = ZB && PassRadix<T, N, 1, RM>::value == 8;
};

template <typename T, int N, int C, int CS, int NT, int DIR, int R, int NS, bool ZB = false>
__device__ __forceinline__ void stockham_pass(cx<T>* buf, const cx<T>* __restrict__ tw) {
  constexpr bool zb = ZB && NS == 1 && R == 8;
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
      for (int r = 0; r < R; ++r) {
        if (!zb || (r != 3 && r != 4)) v[t][r] = buf[sx<T, CS>(i + r * (N / R), c)];
      }
      if constexpr (zb) {
        dft8_zero34<DIR>(v[t]);
      } else if constexpr (Fused<R, T>::value) {
        cx<T> w[R - 1];
        if constexpr (NS > 1) {
          const int k = i & (NS - 1);
#pragma unroll
          for (int r = 1; r < R; ++r) w[r - 1] = tw[r * k * TWS];
        }
        FDft<R, DIR, T, (NS > 1)>::run(v[t], w);
      } else {
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

// Twiddled radix-8 Stockham pass with a runtime sub-transform length ns
// (1 < ns <= N / 8): the same arithmetic as stockham_pass<..., 8, NS>.
template <typename T, int N, int C, int CS, int NT, int DIR>
__device__ __forceinline__ void stockham_pass8_rt(cx<T>* buf, const cx<T>* __restrict__ tw, int ns) {
  constexpr int R = 8;
  constexpr int NB = C * (N / R);
  constexpr int BPT = (NB + NT - 1) / NT;
  const int tws = N / (R * ns);
  cx<T> v[BPT][R];
#pragma unroll
  for (int t = 0; t < BPT; ++t) {
    const int b = threadIdx.x + t * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % C, i = b / C;
#pragma unroll
      for (int r = 0; r < R; ++r) v[t][r] = buf[sx<T, CS>(i + r * (N / R), c)];
      const int k = i & (ns - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const cx<T> w = tw[r * k * tws];
        v[t][r] = DIR < 0 ? cmul(v[t][r], w) : cmulc(v[t][r], w);
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
      const int k = i & (ns - 1);
      const int base = (i - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[sx<T, CS>(base + r * ns, c)] = pass_out(v[t][r]);
    }
  }
  __syncthreads();
}

template <typename T, int N, int C, int CS, int NT, int DIR, int RM, int NS, bool ZB = false,
          bool DONE = (NS >= N)>
struct FftPasses {
  static __device__ __forceinline__ void run(cx<T>* buf, const cx<T>* __restrict__ tw) {
    constexpr int R = PassRadix<T, N, NS, RM>::value;
    constexpr int END = radix8_run_end(N, NS, RM, LoopedPasses<T>::value);
    if constexpr (LoopedPasses<T>::value && NS > 1 && R == 8 && END > NS * 8) {
#pragma unroll 1
      for (int ns = NS; ns < END; ns *= 8) stockham_pass8_rt<T, N, C, CS, NT, DIR>(buf, tw, ns);
      FftPasses<T, N, C, CS, NT, DIR, RM, END>::run(buf, tw);
    } else {
      stockham_pass<T, N, C, CS, NT, DIR, R, NS, ZB && NS == 1>(buf, tw);
      FftPasses<T, N, C, CS, NT, DIR, RM, NS * R>::run(buf, tw);
    }
  }
};

template <typename T, int N, int C, int CS, int NT, int DIR, int RM, int NS, bool ZB>
struct FftPasses<T, N, C, CS, NT, DIR, RM, NS, ZB, true> {
  static __device__ __forceinline__ void run(cx<T>*, const cx<T>* __restrict__) {}
};

// Transform columns [0, C) of buf (stride CS) in place with passes of radix
// at most RM; the caller must have synchronised after filling buf.  Ends
// with a __syncthreads().  ZB: the inputs 3N/8 .. 5N/8 - 1 are zero, and
// when ZeroBand<N, RM, ZB> holds they are not read (nor need be written).
template <typename T, int N, int C, int CS, int NT, int DIR, int RM = 8, bool ZB = false>
__device__ __forceinline__ void block_fft(cx<T>* buf, const cx<T>* __restrict__ tw) {
  static_assert((N & (N - 1)) == 0 && N >= 4, "power-of-two length");
  static_assert(RM == 16 || RM == 8, "maximum radix 16 or 8");
  FftPasses<T, N, C, CS, NT, DIR, RM, 1, ZeroBand<T, N, RM, ZB>::value>::run(buf, tw);
}

}  // namespace mgb
