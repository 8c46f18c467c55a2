// Fully spectral (doubly periodic) transform kernels.
//
// Layouts (all row-major):
//   spectral state  zd  [rows = 2nn+1][cols = nm]        (reference layout)
//   intermediate    cx<T>[nx][ld = nm]   z-mode columns after an x pass
//   physical        double[nx][nz]
//
// Inverse (to_physical, melvin/SpectralTransformer.py:90-150): an x pass
// (inverse c2c of length nx over the nm kept columns, zero rows in the 2/3
// gap are never stored) then a z pass (c2r of length nz per row, two real
// rows packed into one complex transform).  Forward
// (melvin/SpectralTransformer.py:152-199): a z pass (r2c per row, two rows
// per complex transform, only the nm kept modes leave the CTA) then an x
// pass (c2c over nm columns, only the 2nn+1 kept rows leave the CTA).
// Both directions are unnormalised: the reference multiplies by nx*nz before
// irfft2, which divides by the same factor, and divides the rfft2 result by
// nx*nz (applied at the end of the forward x pass).
//
// The fused timestep (k_xinv -> k_zz_step -> k_xf_step) evaluates the loop
// body of examples/taylor_green_vortex.py:87-93 and its multi-field
// relatives in three HBM round trips.  The finite-difference stencils of
// vec_dot_nabla (melvin/Variable.py:119-128,
// melvin/SpatialDifferentiator.py:76-185) are applied in the pass that holds
// the full periodic line: d/dz of uz*q inside k_zz_step, as the stencil's
// Fourier symbol on the kept modes after the forward z transform (the same
// circulant operator), and d/dx of (ux*q)^ along each column inside
// k_xf_step (the z transform is linear and commutes with the x stencil).
#pragma once

#include "fft_block.cuh"
#include "internal.h"

namespace mgb {

// Resident CTAs per SM the compiler must allow for (register budget).  The
// FP32 and double-float kernels are latency bound (global loads, chains of
// dependent FP32 ops), so they ask for several 256-thread CTAs per SM: four
// (64 registers) for FP32 transforms of up to 512 points, three (80
// registers) for longer ones, whose larger butterfly sets spill at 64
// (measured: the 256-point KH ensemble step is 6% faster with four, the
// 2048-point turbulence step 4% slower); two for double-float.  The FP64
// kernels are bound by the FP64 pipe and keep the default.
template <typename T, int N>
struct MinCTAs {
  static constexpr int value = 1;
};
template <int N>
struct MinCTAs<float, N> {
  static constexpr int value = N <= 512 ? 4 : 3;
};
template <int N>
struct MinCTAs<df64, N> {
  static constexpr int value = 2;
};

// Resident CTAs per SM a kernel asks the register allocator for: MinCTAs,
// but no more than its shared memory lets reside (228 KB per SM, 1 KB of it
// reserved per CTA), so a large tile is not squeezed into registers for
// CTAs that could never be resident together.
template <typename T, int N, size_t SMEM>
struct Occ {
  static constexpr int by_smem = (int)(233472 / (SMEM + 1024));
  static constexpr int value =
      by_smem < 1 ? 1 : (by_smem < MinCTAs<T, N>::value ? by_smem : MinCTAs<T, N>::value);
};

// Columns per CTA of an x pass: 4096 complex values in shared memory
// (64 KB at 16 bytes, 32 KB at 8 bytes, so more FP32 CTAs are resident).
template <typename T, int N>
struct XTile {
  static constexpr int E = 4096;
  static constexpr int C0 = E / N;
  static constexpr int C = C0 < 1 ? 1 : (C0 > 64 ? 64 : C0);
};

// Tile variants of the fused-step kernels, chosen per plan (and per number
// of advected fields) by an autotuner that times them on the caller's own
// workload.  Variant 0 is the default.
//   x passes (k_xinv, k_xf_step): columns per CTA C and maximum FFT radix
//     v = 0: C = XTile::C (halved for the FP64 forward pass, XfVar), radix 8;
//     v = 1: C/2; v = 2: 2C; v = 3: C, radix 16
//   z pass (k_zz_step): row pairs per CTA P and maximum FFT radix
//     v = 0: P = 1, radix 8; v = 1: P = 2; v = 2: P = 4; v = 3: P = 1, radix 16
//   z pass v = 4 (FP32, N = 128..4096): the register-resident kernel
//     k_zz_reg (zreg.cuh), N/8 threads per row pair; x passes have no v = 4
// Variants with the same shape share one kernel; those whose shared memory
// does not fit are absent.  Columns and row pairs change only which CTA does
// the work, so they give bit-identical results; the radix and the kind of
// transform change rounding.
constexpr int kTileVariants = 5;

template <typename T, int N, int V>
struct XVar {
  static constexpr int C0 = XTile<T, N>::C;
  static constexpr int Cr = V == 1 ? C0 / 2 : (V == 2 ? 2 * C0 : C0);
  static constexpr int C = Cr < 1 ? 1 : (Cr > 64 ? 64 : Cr);
  static constexpr int RM = V == 3 ? 16 : 8;
};

// The forward x pass takes the same variants around a base tile that FP64
// and double-float halve: at 2048 points the halved tile gives 683 CTAs
// instead of 341 (a full wave plus a 37-CTA tail at two resident CTAs per
// SM): FP64 0.172 -> 0.150 ms per launch.
template <typename T, int N, int V>
struct XfVar {
  static constexpr int B = XTile<T, N>::C;
  static constexpr int C0 = std::is_same<T, float>::value ? B : (B > 1 ? B / 2 : 1);
  static constexpr int Cr = V == 1 ? C0 / 2 : (V == 2 ? 2 * C0 : C0);
  static constexpr int C = Cr < 1 ? 1 : (Cr > 64 ? 64 : Cr);
  static constexpr int RM = V == 3 ? 16 : 8;
};

template <int V>
struct ZVar {
  static constexpr int P = V == 1 ? 2 : (V == 2 ? 4 : 1);
  static constexpr int RM = V == 3 ? 16 : 8;
};

// Largest dynamic shared memory a CTA may request (227 KB minus the static
// reduction scratch).
constexpr size_t kMaxDynSmem = 232448 - 1024;

// Batched launches: member z of a launch (the last grid dimension) works on
// slot = members ? members[z] : z; the arrays of a slot sit at
// base + slot * stride.  A single simulation is a batch of one with zero
// strides.
struct BatchC {
  const int* members;    // device slot list, or null for slots 0..count-1
  size_t q_stride;       // zd elements between slots of a state array
  size_t h_stride;       // zd elements between slots of a history array
  size_t inter_stride;   // bytes between members' intermediate blocks
  const double* tcoef;   // optional per-slot term coefficients [slot][3][4]
  Gate gate;             // run control of a driven step
};

__device__ __forceinline__ int batch_slot(const BatchC& b, int z) { return b.members ? b.members[z] : z; }

template <typename T>
__device__ __forceinline__ T nan_max(T m, T v) {
  return (v != v || v > m) ? v : m;
}

// Laplacian symbol d2x*n^2 + d2z*m^2 evaluated without contraction, as
// calc_lap does (melvin/SpatialDifferentiator.py:70-74).
__device__ __forceinline__ double lap_symbol(const GridC& g, int n, int m) {
  return __dadd_rn(__dmul_rn(g.d2x, (double)(n * n)), __dmul_rn(g.d2z, (double)(m * m)));
}

// ---------------------------------------------------------------------------
// x pass, inverse
// ---------------------------------------------------------------------------

struct XinvJob {
  const zd* src;  // spectral state
  int kind;       // SrcKind
  void* out;      // intermediate [nx][ld]
  zd* spec_out;   // optional (FP64 kernels): the derived spectral field (ux_s / uz_s)
  zd* psi_out;    // optional (FP64 kernels): psi = solve(-src)
};

// Per-mode factors of the streamfunction inversion, precomputed per plan
// (lap(0,0) := 1, melvin/LaplacianSolver.py:58-68):
//   tux = (2 pi/lz) m / lap,  tuz = (2 pi/lx) n / lap,  rlap = 1 / lap,
// so that ux = -(2 pi i/lz) m psi = i tux w and uz = (2 pi i/lx) n psi =
// -i tuz w with psi = -w / lap (melvin/utility.py:62-79).
struct XinvArgs {
  GridC g;
  XinvJob job[5];
  int ld;
  const void* tux;     // T[rows*cols]
  const void* tuz;     // T[rows*cols]
  const double* rlap;  // double[rows*cols]
  const void* tw;
  BatchC b;            // member = blockIdx.z
};

// Loads per thread issued together before they are used (latency hiding in
// the gather loops of the x passes).
constexpr int kXLoads = 4;

template <typename T, int N, int C, int RM>
__global__ void __launch_bounds__(NT, (Occ<T, N, sbuf_elems<T, C>(N) * sizeof(cx<T>)>::value)) k_xinv(const XinvArgs a) {
  if (gate_closed(a.b.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const XinvJob jb = a.job[blockIdx.y];
  const int m0 = blockIdx.x * C;
  const T* tab = (const T*)(jb.kind == SRC_UX ? a.tux : a.tuz);
  const zd* src = jb.src + (size_t)batch_slot(a.b, blockIdx.z) * a.b.q_stride;
  // zero the 2/3-rule gap rows nn+1 .. N-nn-1 (the kept rows are written
  // below), except 3N/8 .. 5N/8 - 1, which a pruned first pass does not read
  // (nn < 3N/8 holds for every fully spectral plan)
  constexpr bool zb = ZeroBand<T, N, RM, true>::value;
  constexpr int skip = zb ? N / 4 : 0;
  for (int e = threadIdx.x; e < (N - g.rows - skip) * C; e += NT) {
    const int x0 = g.nn + 1 + e / C, c = e % C;
    const int x = (zb && x0 >= 3 * N / 8) ? x0 + N / 4 : x0;
    buf[sx<T, C>(x, c)] = mk<T>(0, 0);
  }
  const int total = g.rows * C;
  for (int e0 = threadIdx.x; e0 < total; e0 += NT * kXLoads) {
    zd w[kXLoads];
    T t[kXLoads];
#pragma unroll
    for (int u = 0; u < kXLoads; ++u) {
      const int e = e0 + u * NT;
      const int r = e / C, m = m0 + (e - r * C);
      const bool ok = e < total && m < g.cols;
      const size_t idx = (size_t)r * g.cols + m;
      w[u] = ok ? src[idx] : mk(0.0, 0.0);
      t[u] = (ok && jb.kind != SRC_COPY) ? tab[idx] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < kXLoads; ++u) {
      const int e = e0 + u * NT;
      if (e >= total) break;
      const int r = e / C, c = e - r * C, m = m0 + c;
      const size_t idx = (size_t)r * g.cols + m;
      const cx<T> wt = cvt<T>(w[u]);
      cx<T> v = wt;
      if (jb.kind == SRC_UX) {
        v = mk(-(t[u] * wt.y), t[u] * wt.x);
      } else if (jb.kind == SRC_UZ) {
        v = mk(t[u] * wt.y, -(t[u] * wt.x));
      }
      if (m < g.cols) {
        if (jb.spec_out) jb.spec_out[idx] = cvt<double>(v);
        if (jb.psi_out) {
          const double rl = a.rlap[idx];
          jb.psi_out[idx] = mk(-(w[u].x * rl), -(w[u].y * rl));
        }
      }
      buf[sx<T, C>(row_bin(r, g.nn, N), c)] = v;  // zero for columns past the last mode
    }
  }
  __syncthreads();
  block_fft<T, N, C, C, NT, +1, RM, true>(buf, (const cx<T>*)a.tw);
  cx<T>* out = (cx<T>*)((char*)jb.out + (size_t)blockIdx.z * a.b.inter_stride);
  for (int e = threadIdx.x; e < N * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    if (m < g.cols) out[(size_t)x * a.ld + m] = buf[sx<T, C>(x, c)];
  }
}

// ---------------------------------------------------------------------------
// z pass helpers: two real rows A, B of half spectra packed as one complex
// transform W = A_h + i B_h (A_h = Hermitian extension; the imaginary part of
// the m = 0 term is dropped, as irfft does).
// ---------------------------------------------------------------------------

template <typename T, int N, int CS>
__device__ __forceinline__ void put_pair(cx<T>* buf, int col, int m, cx<T> A, cx<T> B) {
  if (m == 0) {
    buf[col] = mk(A.x, B.x);
  } else {
    buf[sx<T, CS>(m, col)] = mk(A.x - B.y, A.y + B.x);
    buf[sx<T, CS>(N - m, col)] = mk(A.x + B.y, B.x - A.y);
  }
}

// Split the forward transform Z of a + i b into the half spectra of a and b
// (HALF = false: twice them, the factor 1/2 left to the caller).
template <typename T, int N, int CS, bool HALF = true>
__device__ __forceinline__ void get_pair(const cx<T>* buf, int col, int m, cx<T>& A, cx<T>& B) {
  const cx<T> zm = buf[sx<T, CS>(m, col)];
  const cx<T> zn = buf[sx<T, CS>((N - m) & (N - 1), col)];
  if constexpr (HALF) {
    const T h = (T)0.5;
    A = mk((zm.x + zn.x) * h, (zm.y - zn.y) * h);
    B = mk((zm.y + zn.y) * h, (zn.x - zm.x) * h);
  } else {
    A = mk(zm.x + zn.x, zm.y - zn.y);
    B = mk(zm.y + zn.y, zn.x - zm.x);
  }
}

// Periodic central first difference of the imaginary parts of column `col`
// at position i (melvin/SpatialDifferentiator.py:91-104, 157-185), scaled by
// inv = 1/(2h) (order 2) or 1/(3h) (order 4).
template <typename T, int N, int CS>
__device__ __forceinline__ T fd_imag(const cx<T>* buf, int col, int i, int sdo, T inv) {
  const T p1 = buf[sx<T, CS>((i + 1) & (N - 1), col)].y;
  const T m1 = buf[sx<T, CS>((i - 1) & (N - 1), col)].y;
  if (sdo == 2) return (p1 - m1) * inv;
  const T p2 = buf[sx<T, CS>((i + 2) & (N - 1), col)].y;
  const T m2 = buf[sx<T, CS>((i - 2) & (N - 1), col)].y;
  return (((T)-0.25 * p2 + (T)2 * p1) - (T)2 * m1 + (T)0.25 * m2) * inv;
}

// Replace the imaginary parts of columns [0, NCOL) by their periodic
// z-derivative (in place, staged through registers).  A column's writes
// only conflict with that column's reads, so groups of G columns share one
// barrier (G x elements per thread <= 16 staged values).
template <typename T, int N, int CS, int NCOL>
__device__ __forceinline__ void fd_imag_columns(cx<T>* buf, int sdo, T inv) {
  constexpr int EPT = (N + NT - 1) / NT;
  constexpr int G0 = 16 / EPT < 1 ? 1 : 16 / EPT;
  constexpr int G = G0 < NCOL ? G0 : NCOL;
#pragma unroll 1
  for (int c0 = 0; c0 < NCOL; c0 += G) {
    T v[G][EPT];
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        const int z = threadIdx.x + i * NT;
        if (c0 + g < NCOL && z < N) v[g][i] = fd_imag<T, N, CS>(buf, c0 + g, z, sdo, inv);
      }
    __syncthreads();
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        const int z = threadIdx.x + i * NT;
        if (c0 + g < NCOL && z < N) buf[sx<T, CS>(z, c0 + g)].y = v[g][i];
      }
  }
  __syncthreads();
}

// Deterministic CTA reduction of (sum, max, max, sum) -> partial[blockIdx.x*kDiagW].
__device__ __forceinline__ void block_diag(double s, double mx, double mz, double fl, double* partial) {
  __shared__ double red[4][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mx = nan_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mz = nan_max(mz, __shfl_xor_sync(0xffffffffu, mz, o));
    fl += __shfl_xor_sync(0xffffffffu, fl, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s;
    red[1][w] = mx;
    red[2][w] = mz;
    red[3][w] = fl;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0, MX = -INFINITY, MZ = -INFINITY, FL = 0;
    for (int i = 0; i < NT / 32; ++i) {
      S += red[0][i];
      MX = nan_max(MX, red[1][i]);
      MZ = nan_max(MZ, red[2][i]);
      FL += red[3][i];
    }
    partial[kDiagW * blockIdx.x + 0] = S;
    partial[kDiagW * blockIdx.x + 1] = MX;
    partial[kDiagW * blockIdx.x + 2] = MZ;
    partial[kDiagW * blockIdx.x + 3] = FL;
  }
}

// ---------------------------------------------------------------------------
// Fused z pass of the timestep: for P row pairs (rows x0 = 2*(P*blockIdx.x+p)
// and x0+1, p < P),
//   inverse c2r of ux, uz and the F advected fields,
//   a_f = ux * q_f, b_f = uz * q_f, forward r2c of a_f + i b_f, keep the nm
//   leading modes, C_f = d/dz B_f (the periodic stencil applied as its
//   Fourier symbol: the same circulant operator, only rounding differs).
// The outputs are scaled for the forward x pass: 2 A_f and -C_f / (nx nz)
// (cscale = -1 / (2 nx nz) multiplies the symbol); the x pass's stencil
// factor carries the matching -1 / (2 nx nz), so N = -J / (nx nz) costs no
// product per mode.  All three factors are powers of two: the results are
// those of the unscaled form.
// Pair p's inputs sit in columns p*NIN + i and its outputs in p*NOUT + j of
// the CTA's buffer; a thread reads every input of a position z before it
// writes that position's outputs.  Outputs may alias the inputs: a CTA reads
// only its own rows, before it writes them.
// ---------------------------------------------------------------------------

struct ZzArgs {
  GridC g;
  int ld;
  const void* in[5];  // ux, uz, q_0 .. q_{F-1}
  void* aout[3];
  void* cout[3];
  double* ux_phys;    // optional physical velocity
  double* uz_phys;
  double* partial;    // optional [member][gridDim.x][kDiagW]
  int flux_f;         // field whose sum of uz * q the partials carry (-1: none)
  double fdz;         // 1/(2dz) or 1/(3dz)
  double cscale;      // -1 / (2 nx nz): scale of the C outputs' symbol
  const void* tw;
  BatchC b;           // member = blockIdx.y
};

template <int F, int P>
struct ZzShape {
  static constexpr int NIN = 2 + F, NOUT = 2 * F;
  static constexpr int CS = P * (NIN > NOUT ? NIN : NOUT);
};

// Shared-memory layout of the z pass: stride and pad per 8 rows for each
// element size, field count and row-pair count, chosen with a model of the
// kernel's shared-memory requests (every FFT pass, the row-per-thread
// packing, product, stencil and unpacking phases; 8-byte requests served in
// half-warp phases, 16-byte ones in quarter-warp phases) to minimise the
// total wavefronts over lengths 256..2048.  Modelled gains over the plain
// stride with one pad element: 1.0-1.25x with one row pair, up to 3.4x with
// two or four (an odd stride removes the 8- and 16-way conflicts of the
// row-per-thread phases).
template <typename T, int F, int P>
struct ZzLayout {
  static constexpr int C0 = ZzShape<F, P>::CS;
  static constexpr bool wide = sizeof(cx<T>) >= 16;
  // (F, P) -> stride, pad for 8-byte and 16-byte elements
  static constexpr int k = (F - 1) * 3 + (P == 1 ? 0 : (P == 2 ? 1 : 2));
  static constexpr int cs8[9] = {3, 6, 12, 4, 9, 17, 6, 12, 25};
  static constexpr int pad8[9] = {0, 3, 1, 3, 0, 0, 5, 1, 0};
  static constexpr int cs16[9] = {3, 6, 13, 5, 9, 17, 6, 13, 25};
  static constexpr int pad16[9] = {3, 6, 4, 4, 0, 0, 5, 2, 0};
  static constexpr int value = ExplicitLayout<wide ? cs16[k] : cs8[k], wide ? pad16[k] : pad8[k]>::value;
  static_assert(SmemLayout<T, value>::CS >= C0, "z-pass stride below the column count");
};

// One advected field, one row pair, FP32: the outputs (2 columns) get a
// layout of their own in the same buffer instead of the inputs' stride 3.
// The products phase writes them compacted over the inputs, one block of NT
// rows at a time, behind a barrier (a block's outputs end below the next
// block's inputs), so the forward FFT and its first-pass scatter run on a
// stride-2 layout.  Modelled shared-memory wavefronts per CTA at N = 2048:
// 10670 -> 7422 with radix 16, 10414 -> 8194 with radix 8.
template <typename T, int F, int P, int RM>
struct ZzIo {
  static constexpr bool compact = F == 1 && P == 1 && std::is_same<T, float>::value;
  static constexpr int in = compact ? ExplicitLayout<3, RM == 16 ? 2 : 0>::value : ZzLayout<T, F, P>::value;
  static constexpr int out = compact ? ExplicitLayout<2, 1>::value : in;
};

// The compacted outputs of every block of NT rows end below the inputs of
// the next block.
template <typename T, int N, int LI, int LO, int NIN, int NOUT>
__host__ __device__ constexpr bool zz_compact_safe() {
  using I = SmemLayout<T, LI>;
  using O = SmemLayout<T, LO>;
  for (int z0 = NT; z0 < N; z0 += NT) {
    const int out_end = (z0 - 1) * O::CS + (NOUT - 1) + ((z0 - 1) >> 3) * O::PAD;
    const int in_start = z0 * I::CS + (z0 >> 3) * I::PAD;
    if (out_end >= in_start) return false;
  }
  return true;
}

// Resident CTAs the z pass asks for.  The FP64 pass with one field and one
// row pair takes two where its shared memory allows (128 registers; a few
// hundred bytes spill to L1, which this FP64-bound kernel leaves idle): at
// 2048 points 0.780 -> 0.761 ms.  With more fields the spills grow to
// kilobytes, so those keep Occ.
template <typename T, int N, int F, int P, int RM>
struct ZzOcc {
  using O = Occ<T, N, sbuf_elems<T, ZzIo<T, F, P, RM>::in>(N) * sizeof(cx<T>)>;
  static constexpr bool two = std::is_same<T, double>::value && F == 1 && P == 1 && O::by_smem >= 2;
  static constexpr int value = two ? 2 : O::value;
};

template <typename T, int N, int F, int P, int RM>
__global__ void __launch_bounds__(NT, (ZzOcc<T, N, F, P, RM>::value))
    k_zz_step(const ZzArgs a) {
  if (gate_closed(a.b.gate)) return;
  constexpr int NIN = ZzShape<F, P>::NIN, NOUT = ZzShape<F, P>::NOUT;
  constexpr int CS = ZzIo<T, F, P, RM>::in, CSO = ZzIo<T, F, P, RM>::out;
  constexpr bool compact = ZzIo<T, F, P, RM>::compact;
  static_assert(!compact || (sbuf_elems<T, CSO>(N) <= sbuf_elems<T, CS>(N) &&
                             zz_compact_safe<T, N, CS, CSO, P * NIN, P * NOUT>()),
                "compacted z-pass outputs must stay inside the buffer, below later inputs");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int xb = 2 * P * blockIdx.x;
  const int nm = g.cols, ld = a.ld;
  const size_t moff = (size_t)blockIdx.y * a.b.inter_stride;
  // zero the modes nm .. N-nm of the input columns (the rest is written
  // below), except 3N/8 .. 5N/8 - 1, which a pruned first pass does not read
  // (nm <= 3N/8 holds for every fully spectral plan)
  constexpr bool zb = ZeroBand<T, N, RM, true>::value;
  constexpr int skip = zb ? N / 4 : 0;
  for (int e = threadIdx.x; e < (N - 2 * nm + 1 - skip) * P * NIN; e += NT) {
    const int z0 = nm + e / (P * NIN), c = e % (P * NIN);
    const int z = (zb && z0 >= 3 * N / 8) ? z0 + N / 4 : z0;
    buf[sx<T, CS>(z, c)] = mk<T>(0, 0);
  }
  {
    const cx<T>* ux = (const cx<T>*)((const char*)a.in[0] + moff);
    const cx<T>* uz = (const cx<T>*)((const char*)a.in[1] + moff);
    for (int m = threadIdx.x; m < nm; m += NT) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const size_t r0 = (size_t)(xb + 2 * p) * ld, r1 = r0 + ld;
        put_pair<T, N, CS>(buf, p * NIN + 0, m, ux[r0 + m], uz[r0 + m]);
        put_pair<T, N, CS>(buf, p * NIN + 1, m, ux[r1 + m], uz[r1 + m]);
#pragma unroll
        for (int f = 0; f < F; ++f) {
          const cx<T>* q = (const cx<T>*)((const char*)a.in[2 + f] + moff);
          put_pair<T, N, CS>(buf, p * NIN + 2 + f, m, q[r0 + m], q[r1 + m]);
        }
      }
    }
  }
  __syncthreads();
  block_fft<T, N, P * NIN, CS, NT, +1, RM, true>(buf, (const cx<T>*)a.tw);

  double ke = 0.0, mx = -INFINITY, mz = -INFINITY, fl = 0.0;
  for (int z0 = 0; z0 < N; z0 += NT) {
    const int z = z0 + threadIdx.x;
    cx<T> w[P * NIN];
    if (z < N) {
#pragma unroll
      for (int c = 0; c < P * NIN; ++c) w[c] = buf[sx<T, CS>(z, c)];
    }
    if constexpr (compact) __syncthreads();  // the block's inputs are read before outputs overwrite them
    if (z >= N) continue;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const cx<T>* wp = w + p * NIN;
      const int x0 = xb + 2 * p;
      const T ux0 = wp[0].x, uz0 = wp[0].y, ux1 = wp[1].x, uz1 = wp[1].y;
      if (a.ux_phys) {
        a.ux_phys[(size_t)x0 * N + z] = (double)ux0;
        a.ux_phys[(size_t)(x0 + 1) * N + z] = (double)ux1;
        a.uz_phys[(size_t)x0 * N + z] = (double)uz0;
        a.uz_phys[(size_t)(x0 + 1) * N + z] = (double)uz1;
      }
      if (a.partial) {
        const double dx0 = (double)ux0, dz0 = (double)uz0, dx1 = (double)ux1, dz1 = (double)uz1;
        ke += (dz0 * dz0 + dx0 * dx0) + (dz1 * dz1 + dx1 * dx1);
        mx = nan_max(nan_max(mx, dx0), dx1);
        mz = nan_max(nan_max(mz, dz0), dz1);
      }
#pragma unroll
      for (int f = 0; f < F; ++f) {
        const T q0 = wp[2 + f].x, q1 = wp[2 + f].y;
        if (a.partial && f == a.flux_f) fl += (double)uz0 * (double)q0 + (double)uz1 * (double)q1;
        buf[sx<T, CSO>(z, p * NOUT + f)] = mk(ux0 * q0, uz0 * q0);
        buf[sx<T, CSO>(z, p * NOUT + F + f)] = mk(ux1 * q1, uz1 * q1);
      }
    }
  }
  __syncthreads();
  // Up to 512 points (64-register kernels) the diagnostics are folded here,
  // so the accumulators hold no registers through the forward transform
  // (the 256-point KH ensemble kernel: 420 -> 196 bytes of spills); longer
  // transforms fold at the end (measured 7% faster at 2048 points).
  constexpr bool kEarlyDiag = N <= 512;
  if constexpr (kEarlyDiag) {
    if (a.partial) block_diag(ke, mx, mz, fl, a.partial + (size_t)blockIdx.y * gridDim.x * kDiagW);
  }
  block_fft<T, N, P * NOUT, CSO, NT, -1, RM>(buf, (const cx<T>*)a.tw);
  const cx<T>* twt = (const cx<T>*)a.tw;
  const T fdz = to_t<T>(a.fdz), cscale = to_t<T>(a.cscale);
  for (int m = threadIdx.x; m < nm; m += NT) {
    // c = d/dz b by the periodic stencil is the circulant whose symbol at
    // th = 2 pi m / N is i * sig, sig = 2 sin(th) fdz (order 2) or
    // (4 sin(th) - sin(2 th) / 2) fdz (order 4), with tw[t] = exp(-2 pi i t / N)
    const T s1 = -twt[m].y;
    const T sig = (g.sdo == 2 ? (T)2 * s1 * fdz : ((T)4 * s1 - (T)0.5 * (-twt[2 * m].y)) * fdz) * cscale;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const size_t r0 = (size_t)(xb + 2 * p) * ld, r1 = r0 + ld;
#pragma unroll
      for (int f = 0; f < F; ++f) {
        cx<T>* ao = (cx<T>*)((char*)a.aout[f] + moff);
        cx<T>* co = (cx<T>*)((char*)a.cout[f] + moff);
#pragma unroll
        for (int rho = 0; rho < 2; ++rho) {
          cx<T> A, B;
          get_pair<T, N, CSO, false>(buf, p * NOUT + rho * F + f, m, A, B);
          ao[(rho ? r1 : r0) + m] = A;
          co[(rho ? r1 : r0) + m] = mk(-(sig * B.y), sig * B.x);
        }
      }
    }
  }
  if constexpr (!kEarlyDiag) {
    if (a.partial) block_diag(ke, mx, mz, fl, a.partial + (size_t)blockIdx.y * gridDim.x * kDiagW);
  }
}

// ---------------------------------------------------------------------------
// Fused x pass of the timestep: J_f = d/dx(A_f) + C_f along each column,
// forward c2c, keep the 2nn+1 rows, N_f = -J_f/(nx*nz) + linear terms,
// history write and the Adams-Bashforth / semi-implicit update
// (melvin/Integrator.py:5-18, 53-63), boundary rules.
// ---------------------------------------------------------------------------

struct XfField {
  int nterms;
  int tsrc[4];
  int top[4];
  double tcoef[4];
  int bc;
};

struct XfArgs {
  GridC g;
  int ld;
  const void* ain[3];
  const void* cin[3];
  zd* q[3];
  zd* hist[3];
  const zd* coef[3];   // per-mode update coefficients (a, b) from mgb_step_prepare
  const double* rlap;  // 1/lap, for linear terms of psi
  int order, curr, integrator, need_psi;
  double fdx;          // stencil factor 1/(2dx) or 1/(3dx) times -1/(2 nx nz) (the z pass's scaling)
  XfField eq[3];
  const void* tw;
  BatchC b;            // member = blockIdx.y
};

// J at (x, m): periodic x stencil of A plus C (both intermediates).
template <typename T, int N>
__device__ __forceinline__ cx<T> jac_x(const cx<T>* __restrict__ A, const cx<T>* __restrict__ Cc,
                                      int x, int m, int ld, int sdo, T inv) {
  const cx<T> p1 = A[(size_t)((x + 1) & (N - 1)) * ld + m];
  const cx<T> m1 = A[(size_t)((x - 1) & (N - 1)) * ld + m];
  cx<T> d;
  if (sdo == 2) {
    d = (p1 - m1) * inv;
  } else {
    const cx<T> p2 = A[(size_t)((x + 2) & (N - 1)) * ld + m];
    const cx<T> m2 = A[(size_t)((x - 2) & (N - 1)) * ld + m];
    d = (((p2 * (T)-0.25 + p1 * (T)2) - m1 * (T)2) + m2 * (T)0.25) * inv;
  }
  return d + Cc[(size_t)x * ld + m];
}

// Weighted Adams-Bashforth sum 3 f0 - f1 (AB2) or
// 55 f0 - 59 f1 + 37 f2 - 9 f3 (AB4) (melvin/Integrator.py:5-18) of the
// newest value f0 and the previous ones hp[i] = f_{-1-i}; the dt/2 or dt/24
// factor is part of the update coefficients.
__device__ __forceinline__ zd ab_sum(int order, zd f0, const zd* hp) {
  if (order == 2) return mk(3 * f0.x - hp[0].x, 3 * f0.y - hp[0].y);
  return mk(((55 * f0.x - 59 * hp[0].x) + 37 * hp[1].x) - 9 * hp[2].x,
            ((55 * f0.y - 59 * hp[0].y) + 37 * hp[1].y) - 9 * hp[2].y);
}

// Elements per thread whose state, coefficient and history loads the update
// loop of k_xf_step issues together (F fields x up to 5 complex doubles each).
template <int F>
struct XfLoads {
  static constexpr int value = F == 1 ? 2 : 1;
};

template <typename T, int N, int F, int C, int RM>
__global__ void __launch_bounds__(NT, (Occ<T, N, F * sbuf_elems<T, C>(N) * sizeof(cx<T>)>::value))
    k_xf_step(const XfArgs a) {
  if (gate_closed(a.b.gate)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  const int sdo = g.sdo;
  const T fdx = to_t<T>(a.fdx);
  const size_t moff = (size_t)blockIdx.y * a.b.inter_stride;
  const int mslot = batch_slot(a.b, blockIdx.y);
  // J_f = d/dx(A_f) + C_f: periodic x stencil along each column
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const cx<T>* A = (const cx<T>*)((const char*)a.ain[f] + moff);
    const cx<T>* Cc = (const cx<T>*)((const char*)a.cin[f] + moff);
    cx<T>* bf = buf + f * sbuf_elems<T, C>(N);
    for (int e0 = threadIdx.x; e0 < N * C; e0 += NT * kXLoads) {
      cx<T> p1[kXLoads], m1[kXLoads], p2[kXLoads], m2[kXLoads], cc[kXLoads];
#pragma unroll
      for (int u = 0; u < kXLoads; ++u) {
        const int e = e0 + u * NT;
        const int x = e / C, m = m0 + (e - x * C);
        const bool ok = e < N * C && m < g.cols;
        const bool o4 = ok && sdo != 2;
        const cx<T> z0 = mk<T>(0, 0);
        p1[u] = ok ? A[(size_t)((x + 1) & (N - 1)) * a.ld + m] : z0;
        m1[u] = ok ? A[(size_t)((x - 1) & (N - 1)) * a.ld + m] : z0;
        p2[u] = o4 ? A[(size_t)((x + 2) & (N - 1)) * a.ld + m] : z0;
        m2[u] = o4 ? A[(size_t)((x - 2) & (N - 1)) * a.ld + m] : z0;
        cc[u] = ok ? Cc[(size_t)x * a.ld + m] : z0;
      }
#pragma unroll
      for (int u = 0; u < kXLoads; ++u) {
        const int e = e0 + u * NT;
        if (e >= N * C) break;
        const int x = e / C, c = e - x * C;
        cx<T> d;
        if (sdo == 2) {
          d = (p1[u] - m1[u]) * fdx;
        } else {
          d = (((p2[u] * (T)-0.25 + p1[u] * (T)2) - m1[u] * (T)2) + m2[u] * (T)0.25) * fdx;
        }
        bf[sx<T, C>(x, c)] = d + cc[u];  // zero for columns past the last mode
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < F; ++f) block_fft<T, N, C, C, NT, -1, RM>(buf + f * sbuf_elems<T, C>(N), (const cx<T>*)a.tw);

  // the transform already holds -J / (nx*nz): the z pass's output scales and
  // this pass's stencil factor carry the normalisation (powers of two)
  const size_t slot = (size_t)g.rows * g.cols;
  zd* qf[F];
  zd* hf[F];
#pragma unroll
  for (int f = 0; f < F; ++f) {
    qf[f] = a.q[f] + (size_t)mslot * a.b.q_stride;
    hf[f] = a.hist[f] + (size_t)mslot * a.b.h_stride;
  }
  const double* tco = a.b.tcoef ? a.b.tcoef + (size_t)mslot * 12 : nullptr;
  const bool ab4 = a.order != 2;
  // history slots of f_{-1}, f_{-2}, f_{-3} (melvin/TimeDerivative.py:4-65)
  const size_t hs0 = (size_t)(ab4 ? ((a.curr + 3) & 3) : ((a.curr + 1) & 1)) * slot;
  const size_t hs1 = (size_t)((a.curr + 2) & 3) * slot, hs2 = (size_t)((a.curr + 1) & 3) * slot;
  constexpr int U = XfLoads<F>::value;
  const int total = g.rows * C;
  for (int e0 = threadIdx.x; e0 < total; e0 += NT * U) {
    zd qo[U][F], cf[U][F], hp[U][F][3];
    double rl[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * NT;
      const int r = e / C, m = m0 + (e - r * C);
      const bool ok = e < total && m < g.cols;
      const size_t idx = (size_t)r * g.cols + m;
      const zd z0 = mk(0.0, 0.0);
      rl[u] = (ok && a.need_psi) ? a.rlap[idx] : 0.0;
#pragma unroll
      for (int f = 0; f < F; ++f) {
        qo[u][f] = ok ? qf[f][idx] : z0;
        cf[u][f] = ok ? a.coef[f][idx] : z0;
        hp[u][f][0] = ok ? hf[f][hs0 + idx] : z0;
        hp[u][f][1] = (ok && ab4) ? hf[f][hs1 + idx] : z0;
        hp[u][f][2] = (ok && ab4) ? hf[f][hs2 + idx] : z0;
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * NT;
      const int r = e / C, c = e - r * C, m = m0 + c;
      if (e >= total || m >= g.cols) continue;
      const int n = row_mode(r, g.nn), k = row_bin(r, g.nn, N);
      const size_t idx = (size_t)r * g.cols + m;
#pragma unroll
      for (int f = 0; f < F; ++f) {
        const XfField& eq = a.eq[f];
        // dq[:] = -q.vec_dot_nabla(...) + linear terms
        const cx<T> J = buf[f * sbuf_elems<T, C>(N) + sx<T, C>(k, c)];  // already -J / (nx nz)
        zd fv = cvt<double>(J);
        for (int t = 0; t < eq.nterms; ++t) {
          const int sidx = eq.tsrc[t];
          // psi = -q_0 / lap, formed only for a term that reads it (computed
          // ahead of the terms, the compiler made it unconditional: two FP64
          // products per mode of every step)
          zd sv = sidx < 0 ? mk(-(qo[u][0].x * rl[u]), -(qo[u][0].y * rl[u])) : qo[u][0];
#pragma unroll
          for (int q2 = 1; q2 < F; ++q2)
            if (sidx == q2) sv = qo[u][q2];
          // d/dx, d/dz: the factor 2 pi n / lx or 2 pi m / lz rides on the
          // coefficient and i on the value (one product fewer per term)
          double cc = tco ? tco[f * 4 + t] : eq.tcoef[t];
          const int op = eq.top[t];
          if (op != 0) {
            cc *= op == 1 ? g.dfx * (double)n : g.dfz * (double)m;
            sv = mk(-sv.y, sv.x);
          }
          fv = mk(fv.x + cc * sv.x, fv.y + cc * sv.y);
        }
        const zd cff = cf[u][f], q0 = qo[u][f];
        zd qn;
        if (a.integrator == MGB_INT_SEMI_IMPLICIT) {
          // q' = ((1 + (1-a) dt L) q + AB) / (1 - a dt L) = cf.x q + cf.y * sum
          hf[f][(size_t)a.curr * slot + idx] = fv;
          const zd sm = ab_sum(a.order, fv, hp[u][f]);
          qn = mk(cff.x * q0.x + cff.y * sm.x, cff.x * q0.y + cff.y * sm.y);
        } else {
          // explicit: the history keeps N + D, D = kappa * snabla2(q) = cf.x q
          fv = mk(fv.x + cff.x * q0.x, fv.y + cff.x * q0.y);
          hf[f][(size_t)a.curr * slot + idx] = fv;
          const zd sm = ab_sum(a.order, fv, hp[u][f]);
          qn = mk(q0.x + cff.y * sm.x, q0.y + cff.y * sm.y);
        }
        if ((eq.bc & MGB_BC_ZERO_M0) && m == 0) qn = mk(0.0, 0.0);
        qf[f][idx] = qn;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-verb kernels (FP64): z passes to / from physical rows and an x pass to
// a spectral output.
// ---------------------------------------------------------------------------

struct ZinvArgs {
  GridC g;
  int ld;
  const void* in[2];
  double* out[2];
  const void* tw;
};

template <typename T, int N, int NF>
__global__ void __launch_bounds__(NT) k_zinv_phys(const ZinvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  const size_t r0 = (size_t)x0 * a.ld, r1 = r0 + a.ld;
  for (int e = threadIdx.x; e < sbuf_elems<T, NF>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const cx<T>* q = (const cx<T>*)a.in[f];
      put_pair<T, N, NF>(buf, f, m, q[r0 + m], q[r1 + m]);
    }
  }
  __syncthreads();
  block_fft<T, N, NF, NF, NT, +1>(buf, (const cx<T>*)a.tw);
  for (int z = threadIdx.x; z < N; z += NT) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const cx<T> w = buf[sx<T, NF>(z, f)];
      a.out[f][(size_t)x0 * N + z] = (double)w.x;
      a.out[f][(size_t)(x0 + 1) * N + z] = (double)w.y;
    }
  }
}

struct ZfwdArgs {
  GridC g;
  int ld;
  const double* in;
  void* out;
  const void* tw;
};

template <typename T, int N>
__global__ void __launch_bounds__(NT) k_zfwd_phys(const ZfwdArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  for (int z = threadIdx.x; z < N; z += NT)
    buf[sx<T, 1>(z, 0)] = mk((T)a.in[(size_t)x0 * N + z], (T)a.in[(size_t)(x0 + 1) * N + z]);
  __syncthreads();
  block_fft<T, N, 1, 1, NT, -1>(buf, (const cx<T>*)a.tw);
  cx<T>* out = (cx<T>*)a.out;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
    cx<T> A, B;
    get_pair<T, N, 1>(buf, 0, m, A, B);
    out[(size_t)x0 * a.ld + m] = A;
    out[(size_t)(x0 + 1) * a.ld + m] = B;
  }
}

struct ZvdnArgs {
  GridC g;
  int ld;
  const void* qin;
  double* qphys;
  const double* ux;
  const double* uz;
  void* aout;  // may alias qin
  void* cout;
  double fdz;
  const void* tw;
};

// z pass of vec_dot_nabla: q to physical (written out), a = ux*q,
// c = d/dz(uz*q), forward r2c of a + i c.
template <typename T, int N>
__global__ void __launch_bounds__(NT) k_zz_vdn(const ZvdnArgs a) {
  constexpr int CS = 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  const size_t r0 = (size_t)x0 * a.ld, r1 = r0 + a.ld;
  for (int e = threadIdx.x; e < sbuf_elems<T, CS>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  const cx<T>* q = (const cx<T>*)a.qin;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) put_pair<T, N, CS>(buf, 0, m, q[r0 + m], q[r1 + m]);
  __syncthreads();
  block_fft<T, N, 1, CS, NT, +1>(buf, (const cx<T>*)a.tw);
  const size_t p0 = (size_t)x0 * N, p1 = p0 + N;
  for (int z = threadIdx.x; z < N; z += NT) {
    const cx<T> w = buf[sx<T, CS>(z, 0)];
    const double q0 = (double)w.x, q1 = (double)w.y;
    a.qphys[p0 + z] = q0;
    a.qphys[p1 + z] = q1;
    buf[sx<T, CS>(z, 0)] = mk((T)(a.ux[p0 + z] * q0), (T)(a.uz[p0 + z] * q0));
    buf[sx<T, CS>(z, 1)] = mk((T)(a.ux[p1 + z] * q1), (T)(a.uz[p1 + z] * q1));
  }
  __syncthreads();
  fd_imag_columns<T, N, CS, 2>(buf, a.g.sdo, (T)a.fdz);
  block_fft<T, N, 2, CS, NT, -1>(buf, (const cx<T>*)a.tw);
  cx<T>* ao = (cx<T>*)a.aout;
  cx<T>* co = (cx<T>*)a.cout;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
    cx<T> A, Cc;
    get_pair<T, N, CS>(buf, 0, m, A, Cc);
    ao[r0 + m] = A;
    co[r0 + m] = Cc;
    get_pair<T, N, CS>(buf, 1, m, A, Cc);
    ao[r1 + m] = A;
    co[r1 + m] = Cc;
  }
}

struct XfOutArgs {
  GridC g;
  int ld;
  const void* ain;
  const void* cin;  // null: J = A; otherwise J = d/dx A + C
  zd* out;
  double scale;
  double fdx;
  const void* tw;
};

template <typename T, int N>
__global__ void __launch_bounds__(NT) k_xf_out(const XfOutArgs a) {
  constexpr int C = XTile<T, N>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  const cx<T>* A = (const cx<T>*)a.ain;
  const cx<T>* Cc = (const cx<T>*)a.cin;
  for (int e = threadIdx.x; e < N * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    cx<T> v = mk<T>(0, 0);
    if (m < g.cols) v = Cc ? jac_x<T, N>(A, Cc, x, m, a.ld, g.sdo, (T)a.fdx) : A[(size_t)x * a.ld + m];
    buf[sx<T, C>(x, c)] = v;
  }
  __syncthreads();
  block_fft<T, N, C, C, NT, -1>(buf, (const cx<T>*)a.tw);
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    const cx<T> v = buf[sx<T, C>(row_bin(r, g.nn, N), c)];
    a.out[(size_t)r * g.cols + m] = mk((double)v.x * a.scale, (double)v.y * a.scale);
  }
}

// ---------------------------------------------------------------------------
// Launchers (one instantiation set per transform length N).
// ---------------------------------------------------------------------------

// Opt in to more than the default 48 KB of shared memory per CTA, once per
// kernel and device (the first launch sets the attribute, so later launches,
// including those inside a stream capture, make no attribute call).  Kernels
// here use at most 1 KB of static shared memory, so any dynamic request above
// 47 KB opts in; the attribute is set to the largest size any launch needs.
bool smem_optin_done(const void* kernel, int device, size_t smem);
void smem_optin_record(const void* kernel, int device, size_t smem);

template <typename K>
inline cudaError_t prep_smem(K kernel, size_t smem) {
  if (smem <= 47 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (smem_optin_done((const void*)kernel, dev, smem)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) smem_optin_record((const void*)kernel, dev, smem);
  return e;
}

template <typename T, int N, int V>
cudaError_t launch_xinv(const XinvArgs& a, int njobs, int nb, cudaStream_t s) {
  constexpr int C = XVar<T, N, V>::C, RM = XVar<T, N, V>::RM;
  const size_t smem = (size_t)sbuf_elems<T, C>(N) * sizeof(cx<T>);
  cudaError_t e = prep_smem(k_xinv<T, N, C, RM>, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((a.g.cols + C - 1) / C, njobs, nb);
  k_xinv<T, N, C, RM><<<grid, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int N, int F, int V>
cudaError_t launch_zz_step(const ZzArgs& a, int nb, cudaStream_t s) {
  constexpr int P = ZVar<V>::P, RM = ZVar<V>::RM;
  const size_t smem = (size_t)sbuf_elems<T, ZzIo<T, F, P, RM>::in>(N) * sizeof(cx<T>);
  cudaError_t e = prep_smem(k_zz_step<T, N, F, P, RM>, smem);
  if (e != cudaSuccess) return e;
  k_zz_step<T, N, F, P, RM><<<dim3(a.g.nx / (2 * P), nb), NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int N, int F, int V>
cudaError_t launch_xf_step(const XfArgs& a, int nb, cudaStream_t s) {
  constexpr int C = XfVar<T, N, V>::C, RM = XfVar<T, N, V>::RM;
  const size_t smem = (size_t)F * sbuf_elems<T, C>(N) * sizeof(cx<T>);
  cudaError_t e = prep_smem(k_xf_step<T, N, F, C, RM>, smem);
  if (e != cudaSuccess) return e;
  k_xf_step<T, N, F, C, RM><<<dim3((a.g.cols + C - 1) / C, nb), NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N, int NF>
cudaError_t launch_zinv_phys(const ZinvArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<double, NF>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zinv_phys<double, N, NF>, smem);
  if (e != cudaSuccess) return e;
  k_zinv_phys<double, N, NF><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_zfwd_phys(const ZfwdArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<double, 1>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zfwd_phys<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_zfwd_phys<double, N><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_zz_vdn(const ZvdnArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<double, 2>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zz_vdn<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_zz_vdn<double, N><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_xf_out(const XfOutArgs& a, cudaStream_t s) {
  constexpr int C = XTile<double, N>::C;
  const size_t smem = (size_t)sbuf_elems<double, C>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_xf_out<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_xf_out<double, N><<<(a.g.cols + C - 1) / C, NT, smem, s>>>(a);
  return cudaGetLastError();
}

// Shape of one tile variant of a fused-step kernel: columns (x passes) or
// row pairs (z pass) per CTA, maximum FFT radix and dynamic shared memory;
// smem == 0 marks a variant whose shared memory does not fit.
struct TileShape {
  int shape, radix;
  size_t smem;
  int kind = 0;  // 0: shared-memory passes; 1: register-resident (k_zz_reg)
};

#include "zreg.cuh"

// Table of launchers for one length N, filled by the per-N translation units.
struct FsLaunchers {
  // [precision][variant](args, jobs, members)
  cudaError_t (*xinv[3][kTileVariants])(const XinvArgs&, int, int, cudaStream_t);
  // [precision][F-1][variant](args, members)
  cudaError_t (*zz_step[3][3][kTileVariants])(const ZzArgs&, int, cudaStream_t);
  cudaError_t (*xf_step[3][3][kTileVariants])(const XfArgs&, int, cudaStream_t);
  TileShape xinv_shape[3][kTileVariants];
  TileShape zz_shape[3][3][kTileVariants];
  TileShape xf_shape[3][3][kTileVariants];
  cudaError_t (*zinv_phys[2])(const ZinvArgs&, cudaStream_t);        // [NF-1]
  cudaError_t (*zfwd_phys)(const ZfwdArgs&, cudaStream_t);
  cudaError_t (*zz_vdn)(const ZvdnArgs&, cudaStream_t);
  cudaError_t (*xf_out)(const XfOutArgs&, cudaStream_t);
};

template <typename T, int N, int V>
void fill_xinv(FsLaunchers& L, int prec) {
  constexpr int C = XVar<T, N, V>::C;
  constexpr size_t smem = (size_t)sbuf_elems<T, C>(N) * sizeof(cx<T>);
  L.xinv_shape[prec][V] = TileShape{C, XVar<T, N, V>::RM, smem <= kMaxDynSmem ? smem : 0};
  if constexpr (smem <= kMaxDynSmem) {
    L.xinv[prec][V] = launch_xinv<T, N, V>;
  } else {
    L.xinv[prec][V] = nullptr;
  }
}

template <typename T, int N, int F, int V>
void fill_zz(FsLaunchers& L, int prec) {
  constexpr int P = ZVar<V>::P;
  constexpr size_t smem = (size_t)sbuf_elems<T, ZzIo<T, F, P, ZVar<V>::RM>::in>(N) * sizeof(cx<T>);
  L.zz_shape[prec][F - 1][V] = TileShape{P, ZVar<V>::RM, smem <= kMaxDynSmem ? smem : 0};
  if constexpr (smem <= kMaxDynSmem) {
    L.zz_step[prec][F - 1][V] = launch_zz_step<T, N, F, V>;
  } else {
    L.zz_step[prec][F - 1][V] = nullptr;
  }
}

template <typename T, int N, int F, int V>
void fill_xf(FsLaunchers& L, int prec) {
  constexpr int C = XfVar<T, N, V>::C;
  constexpr size_t smem = (size_t)F * sbuf_elems<T, C>(N) * sizeof(cx<T>);
  L.xf_shape[prec][F - 1][V] = TileShape{C, XfVar<T, N, V>::RM, smem <= kMaxDynSmem ? smem : 0};
  if constexpr (smem <= kMaxDynSmem) {
    L.xf_step[prec][F - 1][V] = launch_xf_step<T, N, F, V>;
  } else {
    L.xf_step[prec][F - 1][V] = nullptr;
  }
}

template <typename T, int N, int V>
void fill_step_variant(FsLaunchers& L, int prec) {
  fill_xinv<T, N, V>(L, prec);
  fill_zz<T, N, 1, V>(L, prec);
  fill_zz<T, N, 2, V>(L, prec);
  fill_zz<T, N, 3, V>(L, prec);
  fill_xf<T, N, 1, V>(L, prec);
  fill_xf<T, N, 2, V>(L, prec);
  fill_xf<T, N, 3, V>(L, prec);
}

template <typename T, int N, int V>
void clear_step_variant(FsLaunchers& L, int prec) {
  L.xinv[prec][V] = nullptr;
  L.xinv_shape[prec][V] = TileShape{XVar<T, N, V>::C, XVar<T, N, V>::RM, 0};
  for (int f = 0; f < 3; ++f) {
    L.zz_step[prec][f][V] = nullptr;
    L.xf_step[prec][f][V] = nullptr;
    L.zz_shape[prec][f][V] = TileShape{ZVar<V>::P, ZVar<V>::RM, 0};
    L.xf_shape[prec][f][V] = TileShape{XfVar<T, N, V>::C, XfVar<T, N, V>::RM, 0};
  }
}

template <typename T, int N, int V, bool ON>
void fill_or_clear(FsLaunchers& L, int prec) {
  if constexpr (ON) {
    fill_step_variant<T, N, V>(L, prec);
  } else {
    clear_step_variant<T, N, V>(L, prec);
  }
}

// Variant 4: the register-resident z pass, FP32 only; no x-pass kernels.
template <typename T, int N, int F>
void fill_zz_reg(FsLaunchers& L, int prec) {
  if constexpr (std::is_same<T, float>::value && ZrShape<N>::ok) {
    constexpr size_t smem = ZrSmem<N, F>::bytes;
    L.zz_shape[prec][F - 1][4] = TileShape{ZrShape<N>::PAIRS, 8, smem <= kMaxDynSmem ? smem : 0, 1};
    if constexpr (smem <= kMaxDynSmem) {
      L.zz_step[prec][F - 1][4] = launch_zz_reg<N, F>;
    } else {
      L.zz_step[prec][F - 1][4] = nullptr;
    }
  } else {
    L.zz_step[prec][F - 1][4] = nullptr;
    L.zz_shape[prec][F - 1][4] = TileShape{1, 8, 0, 1};
  }
}

template <typename T, int N>
void fill_variant4(FsLaunchers& L, int prec) {
  L.xinv[prec][4] = nullptr;
  L.xinv_shape[prec][4] = TileShape{XVar<T, N, 0>::C, 8, 0};
  for (int f = 0; f < 3; ++f) {
    L.xf_step[prec][f][4] = nullptr;
    L.xf_shape[prec][f][4] = TileShape{XfVar<T, N, 0>::C, 8, 0};
  }
  fill_zz_reg<T, N, 1>(L, prec);
  fill_zz_reg<T, N, 2>(L, prec);
  fill_zz_reg<T, N, 3>(L, prec);
}

// The fused-step kernels of one precision, the tile variants in MASK (bit v
// = variant v).  The double-float kernels are built in the default tile
// only: they are several times larger to compile than the others.
template <typename T, int N, int MASK = 0xF>
void fill_step_kernels(FsLaunchers& L, int prec) {
  fill_or_clear<T, N, 0, (MASK & 1) != 0>(L, prec);
  fill_or_clear<T, N, 1, (MASK & 2) != 0>(L, prec);
  fill_or_clear<T, N, 2, (MASK & 4) != 0>(L, prec);
  fill_or_clear<T, N, 3, (MASK & 8) != 0>(L, prec);
  fill_variant4<T, N>(L, prec);
}

// The FP64 per-verb kernels.
template <int N>
void fill_verb_kernels(FsLaunchers& L) {
  L.zinv_phys[0] = launch_zinv_phys<N, 1>;
  L.zinv_phys[1] = launch_zinv_phys<N, 2>;
  L.zfwd_phys = launch_zfwd_phys<N>;
  L.zz_vdn = launch_zz_vdn<N>;
  L.xf_out = launch_xf_out<N>;
}

// Defined by fs_n<N>.cu; returns nullptr for lengths that are not built.
const FsLaunchers* fs_launchers(int N);

}  // namespace mgb
