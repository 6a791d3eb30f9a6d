// Ground-state CC amplitudes on the GPU: Jacobi sweeps with eigh(F)
// denominators, DIIS extrapolation and the energies that monitor it.
//
// Follows the reference's solvers: DIIS_solver / DIIS_solver_Lam
// (CCSD_Helper.py:347-416, 702-776), DIIS_solver_CC2 / DIIS_solver_Lam_CC2
// (CC2_Helper.py:179-248, 324-400), corrected_T1/T2/lam1/lam2
// (CCSD_Helper.py:320-344, 650-677), CCSD_Corr_E / CCSD_pseudo_E
// (CCSD_Helper.py:312-318, 650-656).  The residuals are the engine's
// programs; the vectors stay on the device; the (maxsize+1)^2 DIIS system is
// solved on the host by Gaussian elimination with partial pivoting.
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tdcc.h"
#include "engine.h"
#include "ground.h"

namespace tdcc {

// x += r / (e_occ - e_vir)   for t1/l1 (rank 2) or t2/l2 (rank 4)
__global__ void jacobi_kernel(double2* x, const double2* r, const double* eps, int o, int v, int rank,
                              long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double d;
    if (rank == 2) {
      const int a = (int)(i % v), ii = (int)(i / v);
      d = eps[ii] - eps[o + a];
    } else {
      long long l = i;
      const int b = (int)(l % v);
      l /= v;
      const int a = (int)(l % v);
      l /= v;
      const int j = (int)(l % o);
      const int ii = (int)(l / o);
      d = eps[ii] + eps[j] - eps[o + a] - eps[o + b];
    }
    const double inv = 1.0 / d;
    const double2 rr = r[i];
    double2 xx = x[i];
    xx.x += rr.x * inv;
    xx.y += rr.y * inv;
    x[i] = xx;
  }
}

// out = sum_k c_k src_k (up to 16 sources)
struct LinComb {
  const double2* src[16];
  double c[16];
  int n;
};
__global__ void lincomb_kernel(double2* out, const LinComb lc, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int k = 0; k < lc.n; ++k) {
      const double2 v = lc.src[k][i];
      s.x += lc.c[k] * v.x;
      s.y += lc.c[k] * v.y;
    }
    out[i] = s;
  }
}

// out = a - b
__global__ void sub_kernel(double2* out, const double2* a, const double2* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 x = a[i], y = b[i];
    out[i] = make_double2(x.x - y.x, x.y - y.y);
  }
}

// res[k] = sum_i a_k[i] * b_k[i] (complex product, no conjugation, like
// contract('ia,ia->')); one block per pair, deterministic two-level sum
__global__ void dot_kernel(const DotPairs p, double2* res) {
  const int k = blockIdx.x;
  if (k >= p.count) return;
  const double2* a = p.a[k];
  const double2* b = p.b[k];
  double sr = 0.0, si = 0.0;
  for (long long i = threadIdx.x; i < p.n[k]; i += blockDim.x) {
    const double2 x = a[i], y = b[i];
    sr = fma(x.x, y.x, sr);
    sr = fma(-x.y, y.y, sr);
    si = fma(x.x, y.y, si);
    si = fma(x.y, y.x, si);
  }
  for (int d = 16; d > 0; d >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, d);
    si += __shfl_down_sync(0xffffffffu, si, d);
  }
  __shared__ double wr[32], wi[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    wr[w] = sr;
    wi[w] = si;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    sr = lane < nw ? wr[lane] : 0.0;
    si = lane < nw ? wi[lane] : 0.0;
    for (int d = 16; d > 0; d >>= 1) {
      sr += __shfl_down_sync(0xffffffffu, sr, d);
      si += __shfl_down_sync(0xffffffffu, si, d);
    }
    if (lane == 0) res[k] = make_double2(sr, si);
  }
}

// CCSD_Corr_E (mode 0):  f_ia t1_ia + 1/4 <ij||ab> t2_ijab + 1/2 <ij||ab> t1_ia t1_jb
// CCSD_pseudo_E (mode 1): f_ia l1_ia  and  1/4 <ij||ab> l2_ijab  (two outputs)
__global__ void energy_kernel(const double* tei, const double* fock, const double2* x1, const double2* x2,
                              int o, int v, int mode, double2* res) {
  const int n = o + v;
  double e1r = 0, e1i = 0, e2r = 0, e2i = 0;
  const long long nov = (long long)o * v, n2 = nov * nov;
  for (long long idx = threadIdx.x; idx < n2 + nov; idx += blockDim.x) {
    if (idx < nov) {
      const int i = (int)(idx / v), a = (int)(idx % v);
      const double f = fock[(long long)i * n + o + a];
      e1r += f * x1[idx].x;
      e1i += f * x1[idx].y;
    } else {
      long long l = idx - nov;
      const int b = (int)(l % v);
      l /= v;
      const int a = (int)(l % v);
      l /= v;
      const int j = (int)(l % o);
      const int i = (int)(l / o);
      const double g = tei[(((long long)i * n + j) * n + o + a) * n + o + b];
      const double2 t = x2[l * v * v + (long long)a * v + b];
      double xr = 0.25 * t.x, xi = 0.25 * t.y;
      if (mode == 0) {
        const double2 p = x1[(long long)i * v + a], q = x1[(long long)j * v + b];
        xr += 0.5 * (p.x * q.x - p.y * q.y);
        xi += 0.5 * (p.x * q.y + p.y * q.x);
      }
      e2r += g * xr;
      e2i += g * xi;
    }
  }
  __shared__ double s[4][1024];
  s[0][threadIdx.x] = e1r;
  s[1][threadIdx.x] = e1i;
  s[2][threadIdx.x] = e2r;
  s[3][threadIdx.x] = e2i;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 4; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    res[0] = make_double2(s[0][0], s[1][0]);
    res[1] = make_double2(s[2][0], s[3][0]);
  }
}

__global__ void to_complex_kernel(double2* out, const double* in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = make_double2(in[i], 0.0);
}

// res[0].x = max_i |x_i| over two arrays (residual check)
__global__ void maxabs_kernel(const double2* a, long long na, const double2* b, long long nb, double2* res) {
  double m = 0.0;
  for (long long i = threadIdx.x; i < na + nb; i += blockDim.x) {
    const double2 x = i < na ? a[i] : b[i - na];
    m = fmax(m, sqrt(x.x * x.x + x.y * x.y));
  }
  for (int d = 16; d > 0; d >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, d));
  __shared__ double w[32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = fmax(r, w[k]);
    res[0] = make_double2(r, 0.0);
  }
}

static unsigned grid_n(long long n) {
  long long b = (n + 255) / 256;
  return (unsigned)(b > 152 * 8 ? 152 * 8 : (b < 1 ? 1 : b));
}

cudaError_t g_jacobi(double2* x, const double2* r, const double* eps, int o, int v, int rank, long long n,
                     cudaStream_t st) {
  jacobi_kernel<<<grid_n(n), 256, 0, st>>>(x, r, eps, o, v, rank, n);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_lincomb(double2* out, const std::vector<const double2*>& src, const std::vector<double>& c,
                      long long n, cudaStream_t st) {
  LinComb lc{};
  if (src.size() > 16) return cudaErrorInvalidValue;
  lc.n = (int)src.size();
  for (int k = 0; k < lc.n; ++k) {
    lc.src[k] = src[k];
    lc.c[k] = c[k];
  }
  lincomb_kernel<<<grid_n(n), 256, 0, st>>>(out, lc, n);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_sub(double2* out, const double2* a, const double2* b, long long n, cudaStream_t st) {
  sub_kernel<<<grid_n(n), 256, 0, st>>>(out, a, b, n);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_dots(const DotPairs& p, double2* res, cudaStream_t st) {
  dot_kernel<<<p.count, 1024, 0, st>>>(p, res);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_energy(const double* tei, const double* fock, const double2* x1, const double2* x2, int o, int v,
                     int mode, double2* res, cudaStream_t st) {
  energy_kernel<<<1, 1024, 0, st>>>(tei, fock, x1, x2, o, v, mode, res);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_to_complex(double2* out, const double* in, long long n, cudaStream_t st) {
  to_complex_kernel<<<grid_n(n), 256, 0, st>>>(out, in, n);
  count_launch();
  return cudaGetLastError();
}
cudaError_t g_maxabs(const double2* a, long long na, const double2* b, long long nb, double2* res,
                     cudaStream_t st) {
  maxabs_kernel<<<1, 1024, 0, st>>>(a, na, b, nb, res);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdcc
