// Kernels of the ground-state solver (ground.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "engine.h"

namespace tdcc {

// pairs (a_k, b_k) of device vectors for dot products sum_i a_k[i] b_k[i]
struct DotPairs {
  const double2* a[64];
  const double2* b[64];
  long long n[64];
  int count;
};

cudaError_t g_jacobi(double2* x, const double2* r, const double* eps, int o, int v, int rank, long long n,
                     cudaStream_t st);
cudaError_t g_lincomb(double2* out, const std::vector<const double2*>& src, const std::vector<double>& c,
                      long long n, cudaStream_t st);
cudaError_t g_sub(double2* out, const double2* a, const double2* b, long long n, cudaStream_t st);
cudaError_t g_dots(const DotPairs& p, double2* res, cudaStream_t st);
cudaError_t g_energy(const double* tei, const double* fock, const double2* x1, const double2* x2, int o, int v,
                     int mode, double2* res, cudaStream_t st);
cudaError_t g_to_complex(double2* out, const double* in, long long n, cudaStream_t st);
cudaError_t g_maxabs(const double2* a, long long na, const double2* b, long long nb, double2* res,
                     cudaStream_t st);

}  // namespace tdcc
