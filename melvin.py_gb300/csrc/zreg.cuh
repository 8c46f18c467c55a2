// Register-resident z pass of the fused timestep, FP32 (split precision).
//
// Same job as k_zz_step (inverse c2r of ux, uz and the advected fields along
// each grid row, products, z derivative, forward r2c keeping the nm leading
// modes), with the shared-memory traffic cut to the data exchanges an FFT
// cannot avoid:
//
//  * A team of TPC = N/8 threads transforms one pair of grid rows; each
//    thread keeps 8 points of every column in registers.  Every Stockham
//    pass reads the points t + s*N/8 (s = 0..7) of thread t, so the passes
//    are radix 8 (a short last pass of radix 2 or 4 runs 4 or 2
//    butterflies per thread on the same points); the shared-memory buffer
//    is only the exchange between passes (write, barrier, read).
//  * The first inverse pass gathers its inputs straight from the x-pass
//    intermediates (packing two real rows into one complex transform as
//    put_pair does), and the last forward pass leaves its outputs in
//    registers: no staging copy at either end.
//  * The inverse leaves point t + s*N/8 in register s of thread t, which is
//    where the forward transform's first pass wants it: the products
//    ux*q, uz*q are formed in registers and fed straight back.
//  * The periodic z stencil of vec_dot_nabla (melvin/SpatialDifferentiator.py:
//    91-104, 157-185) is applied as its exact Fourier symbol,
//    i*2*sin(th)/(2dz) (order 2) or i*(8 sin th - sin 2th)/(6dz) (order 4),
//    th = 2*pi*m/N, on the kept modes after the forward transform: the same
//    circulant operator as the physical stencil, so only rounding differs.
//  * Shared-memory addresses are swizzled (zsw) so that every exchange
//    pattern -- 16 consecutive points, stride 8 (first-pass writes), two
//    runs of 8 points 64 apart (second-pass writes) -- is one wavefront per
//    half warp.
//  * Twiddles of the middle passes (NS = 8, 64) come from per-CTA tables in
//    shared memory laid out [k][r] with an odd row length (conflict free);
//    the last pass (k = butterfly index) loads w^k from the plan's table and
//    forms the powers it needs by products.
//
// Included by spectral2d_impl.cuh inside namespace mgb, after the z-pass
// argument block (ZzArgs) and its helpers.
#pragma once

// Read-only load of a complex FP32 value.
__device__ __forceinline__ cx<float> ldg_cx(const cx<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return mk(v.x, v.y);
}

// Shared-memory slot of point x of a column (see above).  The map is linear
// over GF(2): zsw(a ^ b) = zsw(a) ^ zsw(b), so an address t + s*Q with
// bit-disjoint parts is a per-thread base XOR a compile-time constant.
__host__ __device__ constexpr int zsw(int x) { return x ^ (((x >> 4) & 7) | ((x >> 3) & 8)); }

template <int N>
struct ZrShape {
  static constexpr int Q = N / 8;                      // threads per row pair
  static constexpr int NTZ = Q > NT ? Q : NT;          // threads per CTA
  static constexpr int PAIRS = NTZ / Q;                // row pairs per CTA
  static constexpr int N8 = ilog2c(N) / 3;             // radix-8 passes
  static constexpr int RL = N >> (3 * N8);             // radix of a short last pass (1: none)
  static constexpr int NS_LAST = RL > 1 ? (N / RL) : (N / 8);
  static constexpr int R_LAST = RL > 1 ? RL : 8;
  static constexpr bool ok = N >= 128 && N <= 4096;
};

// Middle-pass twiddle tables: NS = 8 (8 x 7 entries) and NS = 64 (64 x 7).
constexpr int kZrTab = 8 * 7 + 64 * 7;

template <int F>
struct ZrCols {
  static constexpr int NIN = 2 + F, NOUT = 2 * F;
  static constexpr int NC = NIN > NOUT ? NIN : NOUT;
};

template <int N, int F>
struct ZrSmem {
  static constexpr size_t bytes = (size_t)(kZrTab + ZrShape<N>::PAIRS * ZrCols<F>::NC * N) * sizeof(cx<float>);
};

template <int DIR>
__device__ __forceinline__ cx<float> zr_tw(cx<float> v, cx<float> w) {
  return DIR < 0 ? cmul(v, w) : cmulc(v, w);
}

// A middle radix-8 pass of stride NS over columns [0, NCOL): read the
// thread's points, twiddle, DFT8, write the Stockham outputs.
template <int DIR, int N, int NCOL, int NCA, int NS>
__device__ __forceinline__ void zr_mid_pass(cx<float> (&v)[NCA][8], cx<float>* buf, const cx<float>* tab, int t,
                                            int zt) {
  constexpr int Q = N / 8;
#pragma unroll
  for (int c = 0; c < NCOL; ++c)
#pragma unroll
    for (int s = 0; s < 8; ++s) v[c][s] = buf[c * N + (zt ^ zsw(s * Q))];
  const int k = t & (NS - 1);
  const cx<float>* wk = tab + (NS == 8 ? 0 : 56) + k * 7;
  cx<float> w[7];
#pragma unroll
  for (int r = 0; r < 7; ++r) w[r] = wk[r];
  __syncthreads();  // every point of the buffer has been read
#pragma unroll
  for (int c = 0; c < NCOL; ++c) FDft<8, DIR, float, true>::run(v[c], w);
  const int zb = zsw((t - k) * 8 + k);  // bit-disjoint from r * NS
#pragma unroll
  for (int c = 0; c < NCOL; ++c)
#pragma unroll
    for (int r = 0; r < 8; ++r) buf[c * N + (zb ^ zsw(r * NS))] = v[c][r];
  __syncthreads();
}

// The last pass (stride NS = N/R): butterflies i = t + j*N/8, j < 8/R, on
// the thread's own points; outputs land on the same points.
template <int DIR, int N, int NCOL, int NCA>
__device__ __forceinline__ void zr_last_pass(cx<float> (&v)[NCA][8], const cx<float>* buf,
                                             const cx<float>* __restrict__ tw, int t, int zt) {
  constexpr int Q = N / 8, R = ZrShape<N>::R_LAST, G = 8 / R;
#pragma unroll
  for (int c = 0; c < NCOL; ++c)
#pragma unroll
    for (int s = 0; s < 8; ++s) v[c][s] = buf[c * N + (zt ^ zsw(s * Q))];
#pragma unroll
  for (int j = 0; j < G; ++j) {
    // w^(r*i), i = t + j*Q: w^i from the table, higher powers by products
    cx<float> wp[8];
    wp[1] = ldg_cx(tw + t + j * Q);
    if constexpr (R >= 4) {
      wp[2] = cmul(wp[1], wp[1]);
      wp[3] = cmul(wp[2], wp[1]);
    }
    if constexpr (R == 8) {
      wp[4] = cmul(wp[2], wp[2]);
      wp[5] = cmul(wp[4], wp[1]);
      wp[6] = cmul(wp[3], wp[3]);
      wp[7] = cmul(wp[6], wp[1]);
    }
#pragma unroll
    for (int c = 0; c < NCOL; ++c) {
      cx<float> a[R];
#pragma unroll
      for (int r = 0; r < R; ++r) a[r] = v[c][j + r * G];
      if constexpr (Fused<R, float>::value) {
        FDft<R, DIR, float, true>::run(a, wp + 1);
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) a[r] = zr_tw<DIR>(a[r], wp[r]);
        Dft<R, DIR, float>::run(a);
      }
#pragma unroll
      for (int r = 0; r < R; ++r) v[c][j + r * G] = a[r];
    }
  }
}

// Whole transform of columns [0, NCOL): v holds point t + s*N/8 of every
// column in register s on entry (the first pass's inputs) and on exit.
// The buffer must be free to write on entry (SYNC_FIRST adds the barrier);
// on exit every thread may still be reading it.  ZB: registers 3 and 4 (the
// points 3N/8 .. 5N/8 - 1) are zero and not read.
template <int DIR, int N, int NCOL, int NCA, bool SYNC_FIRST, bool ZB = false>
__device__ __forceinline__ void zr_fft(cx<float> (&v)[NCA][8], cx<float>* buf, const cx<float>* tab,
                                       const cx<float>* __restrict__ tw, int t) {
  const int zt = zsw(t), z8 = zsw(8 * t);  // bases of the reads and of the first-pass writes
  if constexpr (SYNC_FIRST) __syncthreads();
#pragma unroll
  for (int c = 0; c < NCOL; ++c) {
    if constexpr (ZB) {
      dft8_zero34<DIR>(v[c]);
    } else {
      FDft<8, DIR, float, false>::run(v[c], nullptr);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) buf[c * N + (z8 ^ r)] = v[c][r];
  }
  __syncthreads();
  zr_mid_pass<DIR, N, NCOL, NCA, 8>(v, buf, tab, t, zt);
  if constexpr (N >= 1024) zr_mid_pass<DIR, N, NCOL, NCA, 64>(v, buf, tab, t, zt);
  zr_last_pass<DIR, N, NCOL, NCA>(v, buf, tw, t, zt);
}

// Deterministic reduction of the per-thread diagnostics over a CTA of NTH
// threads into partial[kDiagW * blockIdx.x ..] (as block_diag).
template <int NTH>
__device__ __forceinline__ void zr_block_diag(double s, double mx, double mz, double fl, double* partial) {
  __shared__ double red[4][NTH / 32];
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
    for (int i = 0; i < NTH / 32; ++i) {
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

template <int N, int F>
struct ZrOcc {
  static constexpr int by_smem = (int)(233472 / (ZrSmem<N, F>::bytes + 1024));
  static constexpr int want = ZrShape<N>::NTZ > NT ? 1 : (F == 1 ? 3 : 2);
  static constexpr int value = by_smem < 1 ? 1 : (by_smem < want ? by_smem : want);
};

// Row pairs rp = PAIRS*blockIdx.x + team, rows x0 = 2*rp and x0+1; a team
// past the last row pair still takes part in every barrier.
template <int N, int F>
__global__ void __launch_bounds__(ZrShape<N>::NTZ, (ZrOcc<N, F>::value)) k_zz_reg(const ZzArgs a) {
  if (gate_closed(a.b.gate)) return;
  using S = ZrShape<N>;
  constexpr int Q = S::Q, NIN = ZrCols<F>::NIN, NOUT = ZrCols<F>::NOUT, NC = ZrCols<F>::NC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<float>* tab = reinterpret_cast<cx<float>*>(smem_raw);
  const int team = threadIdx.x / Q, t = threadIdx.x - team * Q;
  cx<float>* buf = tab + kZrTab + team * NC * N;
  const cx<float>* __restrict__ tw = (const cx<float>*)a.tw;
  const GridC& g = a.g;
  const int nm = g.cols, ld = a.ld;
  const int rp = S::PAIRS * blockIdx.x + team;
  const bool live = 2 * rp < g.nx;
  const int x0 = 2 * rp;
  const size_t moff = (size_t)blockIdx.y * a.b.inter_stride;

  // twiddle tables of the middle passes: [k][r-1] = w^(r k N/(8 NS))
  for (int e = threadIdx.x; e < kZrTab; e += S::NTZ) {
    if (e < 56) {
      const int k = e / 7, r = e - 7 * k + 1;
      tab[e] = tw[r * k * (N / 64)];
    } else if (N >= 1024) {
      const int e2 = e - 56, k = e2 / 7, r = e2 - 7 * k + 1;
      tab[e] = tw[r * k * (N / 512)];
    }
  }

  // gather: column 0 packs (ux, uz) of row x0, column 1 those of row x0+1,
  // column 2+f the field f of rows x0 and x0+1 (Hermitian halves of two real
  // rows in one complex transform)
  cx<float> v[NC][8];
  {
    const cx<float>* src[NIN][2];
    size_t row[NIN][2];
    const cx<float>* ux = (const cx<float>*)((const char*)a.in[0] + moff);
    const cx<float>* uz = (const cx<float>*)((const char*)a.in[1] + moff);
    const size_t r0 = (size_t)x0 * ld, r1 = r0 + ld;
    src[0][0] = ux; src[0][1] = uz; row[0][0] = r0; row[0][1] = r0;
    src[1][0] = ux; src[1][1] = uz; row[1][0] = r1; row[1][1] = r1;
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const cx<float>* q = (const cx<float>*)((const char*)a.in[2 + f] + moff);
      src[2 + f][0] = q; src[2 + f][1] = q; row[2 + f][0] = r0; row[2 + f][1] = r1;
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      if (s == 3 || s == 4) continue;  // removed modes (nm <= 3N/8): the pruned first pass skips them
      const int x = t + s * Q;
      const bool lo = x < nm, hi = x > N - nm;
      const int m = lo ? x : N - x;
#pragma unroll
      for (int c = 0; c < NIN; ++c) {
        cx<float> A = mk(0.f, 0.f), B = mk(0.f, 0.f);
        if (live && (lo || hi)) {
          A = ldg_cx(src[c][0] + row[c][0] + m);
          B = ldg_cx(src[c][1] + row[c][1] + m);
        }
        v[c][s] = x == 0 ? mk(A.x, B.x) : (hi ? mk(A.x + B.y, B.x - A.y) : mk(A.x - B.y, A.y + B.x));
      }
    }
  }
  zr_fft<+1, N, NIN, NC, false, true>(v, buf, tab, tw, t);

  // products in registers: column f <- (ux0 q_f0, uz0 q_f0), column F+f <-
  // (ux1 q_f1, uz1 q_f1); diagnostics of the start-of-step velocity
  double ke = 0.0, mx = -INFINITY, mz = -INFINITY, fl = 0.0;
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int z = t + s * Q;
    const float ux0 = v[0][s].x, uz0 = v[0][s].y, ux1 = v[1][s].x, uz1 = v[1][s].y;
    float q0[F], q1[F];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      q0[f] = v[2 + f][s].x;
      q1[f] = v[2 + f][s].y;
    }
    if (live) {
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
#pragma unroll
        for (int f = 0; f < F; ++f)
          if (f == a.flux_f) fl += (double)uz0 * (double)q0[f] + (double)uz1 * (double)q1[f];
      }
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      v[f][s] = mk(ux0 * q0[f], uz0 * q0[f]);
      v[F + f][s] = mk(ux1 * q1[f], uz1 * q1[f]);
    }
  }
  zr_fft<-1, N, NOUT, NC, true>(v, buf, tab, tw, t);

  // unpack: Z(m) is in register, Z(N-m) comes from the thread that holds it
  __syncthreads();
  const int zt = zsw(t);
#pragma unroll
  for (int s = 5; s < 8; ++s) {
    const int x = t + s * Q;
    if (x > N - nm) {
#pragma unroll
      for (int o = 0; o < NOUT; ++o) buf[o * N + (zt ^ zsw(s * Q))] = v[o][s];
    }
  }
  __syncthreads();
  if (live) {
    const float inv = to_t<float>(a.fdz), cscale = to_t<float>(a.cscale);
    const size_t r0 = (size_t)x0 * ld, r1 = r0 + ld;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int m = t + s * Q;
      if (m < nm) {
        // FD symbol: sigma = 2 sin(th) inv (order 2), (4 sin th - sin(2th)/2) inv (order 4)
        const float s1 = -ldg_cx(tw + m).y;
        const float sig =
            (g.sdo == 2 ? 2.f * s1 * inv : (4.f * s1 - 0.5f * -ldg_cx(tw + ((2 * m) & (N - 1))).y) * inv) * cscale;
#pragma unroll
        for (int o = 0; o < NOUT; ++o) {
          const cx<float> zm = v[o][s];
          const cx<float> zn = m == 0 ? zm : buf[o * N + zsw(N - m)];
          // 2 A and 2 B: the factor 1/2 is in the scales (see ZzArgs)
          const cx<float> A = mk(zm.x + zn.x, zm.y - zn.y);
          const cx<float> B = mk(zm.y + zn.y, zn.x - zm.x);
          const int f = o < F ? o : o - F;
          const size_t rr = o < F ? r0 : r1;
          cx<float>* ao = (cx<float>*)((char*)a.aout[f] + moff);
          cx<float>* co = (cx<float>*)((char*)a.cout[f] + moff);
          ao[rr + m] = A;
          co[rr + m] = mk(-sig * B.y, sig * B.x);
        }
      }
    }
  }
  if (a.partial) zr_block_diag<S::NTZ>(ke, mx, mz, fl, a.partial + (size_t)blockIdx.y * gridDim.x * kDiagW);
}

template <int N, int F>
cudaError_t launch_zz_reg(const ZzArgs& a, int nb, cudaStream_t s) {
  using S = ZrShape<N>;
  const size_t smem = ZrSmem<N, F>::bytes;
  cudaError_t e = prep_smem(k_zz_reg<N, F>, smem);
  if (e != cudaSuccess) return e;
  const int pairs = a.g.nx / 2;
  k_zz_reg<N, F><<<dim3((pairs + S::PAIRS - 1) / S::PAIRS, nb), S::NTZ, smem, s>>>(a);
  return cudaGetLastError();
}
