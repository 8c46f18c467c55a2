// Cosine / sine basis transforms (and complex-exponential transforms of a
// plan whose axes are not powers of two) for any transform length L in
// [16, 4096], by Bluestein's algorithm.
//
// The reference transforms an axis with numpy.fft (pocketfft), which takes
// any length (melvin/SpectralTransformer.py:58,85,132,191); a cosine or sine
// axis of n points is a mirrored periodic signal of L = 2(n-1) points, so the
// reference's own basis tests at n = 256 (test/SpectralTransformer_test.py:
// 64-310) need L = 510 = 2*3*5*17.  With jk = (j^2 + k^2 - (k-j)^2)/2 a
// length-L DFT becomes a circular convolution:
//   X_k = c_k * sum_j (x_j c_j) conj(c_(k-j)),   c_j = exp(-pi i j^2 / L)
// (forward; the unnormalised inverse conjugates every chirp), evaluated with
// power-of-two FFTs of length M >= 2L - 1 and the transform of the kernel
// conj(c) precomputed per length:
//   X = c . IFFT_M(FFT_M(x . c, zero padded) . FFT_M(b) / M).
// Each kernel below does exactly what its power-of-two twin in mirror.cu
// does (extension, crop, basis factors, zeroth-mode rule), with the block
// FFT of length M in place of the length-L one.  FP64 (per-verb transforms).
//
// Tables (host, long double, cached per plan and length): the chirp with
// j^2 reduced mod 2L so the angle stays in [0, 2 pi), and FFT_M of the
// kernel by a radix-2 transform with directly evaluated twiddles.
#include <cmath>
#include <complex>
#include <vector>

#include "mirror.cuh"

namespace mgb {

namespace {

// conv: buf holds x . chirp (zero beyond L) in columns [0, C); on exit it
// holds the convolution, still to be multiplied by the chirp.
template <int M, int C>
__device__ __forceinline__ void blue_conv(zd* buf, const zd* __restrict__ bhat, const zd* __restrict__ tw) {
  block_fft<double, M, C, C, NT, -1>(buf, tw);
  for (int e = threadIdx.x; e < M * C; e += NT) {
    const int x = e / C, c = e - x * C;
    buf[sx<double, C>(x, c)] = cmuld(buf[sx<double, C>(x, c)], bhat[x]);
  }
  __syncthreads();
  block_fft<double, M, C, C, NT, +1>(buf, tw);
}

__device__ __forceinline__ zd conjd(zd a) { return mk(a.x, -a.y); }

template <int M, int C>
__device__ __forceinline__ void zero_buf(zd* buf) {
  for (int e = threadIdx.x; e < sbuf_elems<double, C>(M); e += NT) buf[e] = mk(0.0, 0.0);
  __syncthreads();
}

// to_physical, x pass (inverse, length Lx): spectral column m -> first nxp
// rows of the intermediate (k_mx_inv).
template <int M>
__global__ void __launch_bounds__(NT) k_bx_inv(const MirrorArgs a, const BlueTables b) {
  constexpr int C = MTile<M>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C, L = b.L;
  zero_buf<M, C>(buf);
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m < g.cols) {
      zd v = cmuld(a.spec_in[(size_t)r * g.cols + m], a.scale);
      if (a.bx == 1 && r == 0) v = mk(2 * v.x, 2 * v.y);
      if (a.bz == 1 && m == 0) v = mk(2 * v.x, 2 * v.y);
      const int j = mbin(r, g.nn, L);
      buf[sx<double, C>(j, c)] = cmuld(v, conjd(b.chirp[j]));
    }
  }
  __syncthreads();
  blue_conv<M, C>(buf, b.bhat_i, (const zd*)b.tw);
  for (int e = threadIdx.x; e < a.nxp * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    if (m < g.cols) a.inter[(size_t)x * g.cols + m] = cmuld(buf[sx<double, C>(x, c)], conjd(b.chirp[x]));
  }
}

// to_physical, z pass (inverse c2r, length Lz): two intermediate rows ->
// first nzp points (k_mz_inv).
template <int M>
__global__ void __launch_bounds__(NT) k_bz_inv(const MirrorArgs a, const BlueTables b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int x0 = 2 * blockIdx.x, L = b.L;
  const bool two = x0 + 1 < a.nxp;
  zero_buf<M, 1>(buf);
  for (int m = threadIdx.x; m < g.cols; m += NT) {
    const zd A = a.inter[(size_t)x0 * g.cols + m];
    const zd B = two ? a.inter[(size_t)(x0 + 1) * g.cols + m] : mk(0.0, 0.0);
    // put_pair: W = A_h + i B_h at m and L - m (the imaginary part of m = 0 dropped)
    if (m == 0) {
      buf[0] = mk(A.x, B.x);
    } else {
      buf[sx<double, 1>(m, 0)] = cmuld(mk(A.x - B.y, A.y + B.x), conjd(b.chirp[m]));
      buf[sx<double, 1>(L - m, 0)] = cmuld(mk(A.x + B.y, B.x - A.y), conjd(b.chirp[L - m]));
    }
  }
  __syncthreads();
  blue_conv<M, 1>(buf, b.bhat_i, (const zd*)b.tw);
  for (int z = threadIdx.x; z < a.nzp; z += NT) {
    const zd w = cmuld(buf[sx<double, 1>(z, 0)], conjd(b.chirp[z]));
    a.phys_out[(size_t)x0 * a.nzp + z] = w.x;
    if (two) a.phys_out[(size_t)(x0 + 1) * a.nzp + z] = w.y;
  }
}

// to_spectral, z pass (forward r2c, length Lz): two physical rows ->
// extension -> the nm kept modes of each row (k_mz_fwd).
template <int M>
__global__ void __launch_bounds__(NT) k_bz_fwd(const MirrorArgs a, const BlueTables b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int x0 = 2 * blockIdx.x, L = b.L;
  const bool two = x0 + 1 < a.nxp;
  zero_buf<M, 1>(buf);
  for (int j = threadIdx.x; j < L; j += NT) {
    double s;
    const int z = mirror_src(j, a.nzp, L, a.bz, s);
    const double u = a.phys_in[(size_t)x0 * a.nzp + z];
    const double v = two ? a.phys_in[(size_t)(x0 + 1) * a.nzp + z] : 0.0;
    buf[sx<double, 1>(j, 0)] = cmuld(mk(s * u, s * v), b.chirp[j]);
  }
  __syncthreads();
  blue_conv<M, 1>(buf, b.bhat_f, (const zd*)b.tw);
  for (int m = threadIdx.x; m < g.cols; m += NT) {
    // get_pair on Z_k = conv_k c_k
    const int n = m == 0 ? 0 : L - m;
    const zd zm = cmuld(buf[sx<double, 1>(m, 0)], b.chirp[m]);
    const zd zn = cmuld(buf[sx<double, 1>(n, 0)], b.chirp[n]);
    const zd A = mk((zm.x + zn.x) * 0.5, (zm.y - zn.y) * 0.5);
    const zd B = mk((zm.y + zn.y) * 0.5, (zn.x - zm.x) * 0.5);
    a.inter[(size_t)x0 * g.cols + m] = A;
    if (two) a.inter[(size_t)(x0 + 1) * g.cols + m] = B;
  }
}

// to_spectral, x pass (forward, length Lx): intermediate column m ->
// extension -> the 2nn+1 kept rows, scaled (k_mx_fwd).
template <int M>
__global__ void __launch_bounds__(NT) k_bx_fwd(const MirrorArgs a, const BlueTables b) {
  constexpr int C = MTile<M>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C, L = b.L;
  for (int e = threadIdx.x; e < M * C; e += NT) {
    const int j = e / C, c = e - j * C, m = m0 + c;
    zd v = mk(0.0, 0.0);
    if (m < g.cols && j < L) {
      double s;
      const int x = mirror_src(j, a.nxp, L, a.bx, s);
      const zd w = a.inter[(size_t)x * g.cols + m];
      v = cmuld(mk(s * w.x, s * w.y), b.chirp[j]);
    }
    buf[sx<double, C>(j, c)] = v;
  }
  __syncthreads();
  blue_conv<M, C>(buf, b.bhat_f, (const zd*)b.tw);
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    const int k = mbin(r, g.nn, L);
    zd v = cmuld(cmuld(buf[sx<double, C>(k, c)], b.chirp[k]), a.scale);
    if (a.bx == 1 && r == 0) v = mk(0.5 * v.x, 0.5 * v.y);
    if (a.bz == 1 && m == 0) v = mk(0.5 * v.x, 0.5 * v.y);
    a.spec_out[(size_t)r * g.cols + m] = v;
  }
}

template <int M>
cudaError_t launch_b(int which, const MirrorArgs& a, const BlueTables& b, cudaStream_t s) {
  constexpr int C = MTile<M>::C;
  const size_t sx_smem = (size_t)sbuf_elems<double, C>(M) * sizeof(zd);
  const size_t sz_smem = (size_t)sbuf_elems<double, 1>(M) * sizeof(zd);
  cudaError_t e = cudaSuccess;
  switch (which) {
    case 0:
      e = prep_smem(k_bx_inv<M>, sx_smem);
      if (e == cudaSuccess) k_bx_inv<M><<<(a.g.cols + C - 1) / C, NT, sx_smem, s>>>(a, b);
      break;
    case 1:
      e = prep_smem(k_bz_inv<M>, sz_smem);
      if (e == cudaSuccess) k_bz_inv<M><<<(a.nxp + 1) / 2, NT, sz_smem, s>>>(a, b);
      break;
    case 2:
      e = prep_smem(k_bz_fwd<M>, sz_smem);
      if (e == cudaSuccess) k_bz_fwd<M><<<(a.nxp + 1) / 2, NT, sz_smem, s>>>(a, b);
      break;
    default:
      e = prep_smem(k_bx_fwd<M>, sx_smem);
      if (e == cudaSuccess) k_bx_fwd<M><<<(a.g.cols + C - 1) / C, NT, sx_smem, s>>>(a, b);
      break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

typedef std::complex<long double> cld;

// In-place radix-2 FFT of length n (a power of two), exp(-2 pi i jk / n),
// twiddles evaluated directly in long double.
void host_fft(std::vector<cld>& v) {
  const size_t n = v.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(v[i], v[j]);
  }
  const long double tp = 6.283185307179586476925286766559005768L;
  for (size_t len = 2; len <= n; len <<= 1) {
    for (size_t i = 0; i < n; i += len) {
      for (size_t k = 0; k < len / 2; ++k) {
        const long double ang = -tp * (long double)k / (long double)len;
        const cld w(cosl(ang), sinl(ang));
        const cld u = v[i + k], t = w * v[i + k + len / 2];
        v[i + k] = u + t;
        v[i + k + len / 2] = u - t;
      }
    }
  }
}

int upload(const std::vector<zd>& h, void** out) {
  MGB_CUDA(cudaMalloc(out, h.size() * sizeof(zd)));
  MGB_CUDA(cudaMemcpy(*out, h.data(), h.size() * sizeof(zd), cudaMemcpyHostToDevice));
  return MGB_OK;
}

}  // namespace

int bluestein_tables(const mgb_plan* p, int L, BlueTables& b) {
  int M = 32;
  while (M < 2 * L - 1) M *= 2;
  b.L = L;
  b.M = M;
  b.tw = mirror_twiddles(p, M);
  if (!b.tw) return fail(MGB_ERR_CUDA, "twiddle table of length %d", M);
  std::lock_guard<std::mutex> lock(p->mu);
  auto it = p->blue.find(L);
  if (it == p->blue.end()) {
    const long double pi = 3.141592653589793238462643383279502884L;
    std::vector<cld> chirp(L), kf(M, cld(0, 0)), ki(M, cld(0, 0));
    for (int j = 0; j < L; ++j) {
      const long long q = ((long long)j * j) % (2LL * L);
      const long double ang = -pi * (long double)q / (long double)L;
      chirp[j] = cld(cosl(ang), sinl(ang));
    }
    for (int j = 0; j < L; ++j) {
      kf[j] = std::conj(chirp[j]);
      ki[j] = chirp[j];
      if (j > 0) {
        kf[M - j] = std::conj(chirp[j]);
        ki[M - j] = chirp[j];
      }
    }
    host_fft(kf);
    host_fft(ki);
    std::vector<zd> hc(L), hf(M), hi(M);
    for (int j = 0; j < L; ++j) hc[j] = mk((double)chirp[j].real(), (double)chirp[j].imag());
    for (int j = 0; j < M; ++j) {
      hf[j] = mk((double)(kf[j].real() / M), (double)(kf[j].imag() / M));
      hi[j] = mk((double)(ki[j].real() / M), (double)(ki[j].imag() / M));
    }
    std::array<void*, 3> d = {nullptr, nullptr, nullptr};
    int st = upload(hc, &d[0]);
    if (!st) st = upload(hf, &d[1]);
    if (!st) st = upload(hi, &d[2]);
    if (st) {
      for (void* q : d) cudaFree(q);
      return st;
    }
    it = p->blue.emplace(L, d).first;
  }
  b.chirp = (const zd*)it->second[0];
  b.bhat_f = (const zd*)it->second[1];
  b.bhat_i = (const zd*)it->second[2];
  return MGB_OK;
}

cudaError_t launch_bluestein(int which, const MirrorArgs& a, const BlueTables& b, cudaStream_t s) {
  switch (b.M) {
    case 32: return launch_b<32>(which, a, b, s);
    case 64: return launch_b<64>(which, a, b, s);
    case 128: return launch_b<128>(which, a, b, s);
    case 256: return launch_b<256>(which, a, b, s);
    case 512: return launch_b<512>(which, a, b, s);
    case 1024: return launch_b<1024>(which, a, b, s);
    case 2048: return launch_b<2048>(which, a, b, s);
    case 4096: return launch_b<4096>(which, a, b, s);
    case 8192: return launch_b<8192>(which, a, b, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mgb
