#pragma once
// Integral build from density-fitting factors and the dipole spectrum (post.cu).
#include <cuda_runtime.h>

namespace tdcc {

// X[p,q,r,s] (= (pr|qs)) <- X[p,q,r,s] - X[p,q,s,r], in place, n^4 doubles
cudaError_t launch_tei_antisym(double* X, int n, cudaStream_t st);

// shifted DFTs of Re mu and Im mu (mu[n * stride], n < N); tw: N scratch
// entries (the twiddles exp(-2 pi i r / N))
cudaError_t launch_spectrum(const double2* mu, long long N, long long stride, double2* tw, double2* Yr, double2* Yi,
                            cudaStream_t st);

}  // namespace tdcc
