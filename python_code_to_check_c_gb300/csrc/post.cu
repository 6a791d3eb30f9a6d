// Integral build from density-fitting factors and the dipole spectrum.
//
// tei_antisym_kernel: <pq||rs> = (pr|qs) - (ps|qr) in place over the
//   Coulomb-ordered product X[p,q,r,s] = (pr|qs) (the GEMM sum_Q B_Q,pr B_Q,qs
//   is written in that order by the strided GEMM).
// spectrum_kernel: the shifted discrete Fourier transforms of Re mu(t) and
//   Im mu(t), as the reference's post-processing computes them
//   (Plots.py:20-25: np.fft.fft of the real and imaginary parts, fftshift).
#include <cuda_runtime.h>

#include "engine.h"
#include "post.h"

namespace tdcc {

// one thread per (p, q, r, s); the thread with r < s handles the pair
// (r, s), (s, r) of its (p, q) slice (that slice, n^2 doubles, stays in L2
// while its threads run, so the transposed accesses are L2 hits)
__global__ void tei_antisym_kernel(double* __restrict__ X, int n) {
  const long long nn = (long long)n * n;
  const long long total = nn * nn;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long rs = i % nn;
    const int r = (int)(rs / n), s = (int)(rs % n);
    if (r > s) continue;
    double* base = X + (i - rs);
    if (r == s) {
      base[rs] = 0.0;
    } else {
      const long long sr = (long long)s * n + r;
      const double a = base[rs], b = base[sr];
      base[rs] = a - b;
      base[sr] = b - a;
    }
  }
}

cudaError_t launch_tei_antisym(double* X, int n, cudaStream_t st) {
  const long long total = (long long)n * n * n * n;
  long long blocks = (total + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  if (blocks < 1) blocks = 1;
  tei_antisym_kernel<<<(unsigned)blocks, 256, 0, st>>>(X, n);
  count_launch();
  return cudaGetLastError();
}

// tw[r] = exp(-2 pi i r / N)
__global__ void twiddle_kernel(double2* __restrict__ tw, long long N) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)r / (double)N, &s, &c);
    tw[r] = make_double2(c, -s);
  }
}

// One block per output position j of the shifted spectra: frequency index
// k = (j + N - N/2) mod N; Yr[j] = sum_n Re mu[n] tw[k n mod N], Yi likewise
// with Im mu.
__global__ void __launch_bounds__(256) spectrum_kernel(const double2* __restrict__ mu, long long N, long long stride,
                                                       const double2* __restrict__ tw, double2* __restrict__ Yr,
                                                       double2* __restrict__ Yi) {
  const long long j = blockIdx.x;
  const long long k = (j + N - N / 2) % N;
  const long long step = (k * (long long)blockDim.x) % N;
  long long r = (k * (long long)threadIdx.x) % N;
  double rr = 0.0, ri = 0.0, ir = 0.0, ii = 0.0;
  for (long long nn = threadIdx.x; nn < N; nn += blockDim.x) {
    const double2 m = mu[nn * stride];
    const double2 w = tw[r];
    rr = fma(m.x, w.x, rr);
    ri = fma(m.x, w.y, ri);
    ir = fma(m.y, w.x, ir);
    ii = fma(m.y, w.y, ii);
    r += step;
    if (r >= N) r -= N;
  }
  for (int d = 16; d > 0; d >>= 1) {
    rr += __shfl_down_sync(0xffffffffu, rr, d);
    ri += __shfl_down_sync(0xffffffffu, ri, d);
    ir += __shfl_down_sync(0xffffffffu, ir, d);
    ii += __shfl_down_sync(0xffffffffu, ii, d);
  }
  __shared__ double red[4][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][w] = rr;
    red[1][w] = ri;
    red[2][w] = ir;
    red[3][w] = ii;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      a += red[0][q];
      b += red[1][q];
      c += red[2][q];
      d += red[3][q];
    }
    Yr[j] = make_double2(a, b);
    Yi[j] = make_double2(c, d);
  }
}

cudaError_t launch_spectrum(const double2* mu, long long N, long long stride, double2* tw, double2* Yr, double2* Yi,
                            cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  long long tb = (N + 255) / 256;
  if (tb > 152LL * 8) tb = 152LL * 8;
  twiddle_kernel<<<(unsigned)tb, 256, 0, st>>>(tw, N);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (N > 0x7fffffffLL) return cudaErrorInvalidValue;
  spectrum_kernel<<<(unsigned)N, 256, 0, st>>>(mu, N, stride, tw, Yr, Yi);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdcc
