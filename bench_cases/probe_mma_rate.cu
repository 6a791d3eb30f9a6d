// Measurement driver: cycles per tcgen05.mma (kind::f16, BF16 in, FP32
// accumulate, M = 128, K = 16) for N = 64 and 128, operands resident in
// shared memory, issued from one thread as the slice-product kernels issue
// them: 4 slices of A and of B, products (s, t) with s + t <= 5 into four
// level accumulators, 4 K steps each, 200 repetitions (mode 0), or every
// product on the same stage (mode 1); operand values constant (data 0) or
// random integers in [-64, 64] (data 1); one CTA or one per SM.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o gpurun_out/probe_mma_rate bench_cases/probe_mma_rate.cu
//   gpurun_out/probe_mma_rate
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
               "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(a), "r"(parity) : "memory");
  return ok != 0;
}

template <int N>
__global__ void __launch_bounds__(128, 1) probe(int R, int mode, int data, long long* out, int* err) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  constexpr int AB = 16384, BB = N * 128;
  uint8_t* A = sm;                 // 4 x 16 KB
  uint8_t* B = sm + 4 * AB;        // 4 x N*128
  __shared__ uint64_t bar;
  __shared__ uint32_t tm;
  const int warp = threadIdx.x >> 5;
  const int nelem = (4 * AB + 4 * BB) / 2;
  unsigned seed = 12345u + threadIdx.x * 7919u + blockIdx.x;
  for (int i = threadIdx.x; i < nelem; i += blockDim.x) {
    seed = seed * 1664525u + 1013904223u;
    int v = data ? (int)((seed >> 9) % 129) - 64 : 1 + (i & 3);
    float f = (float)v;
    uint32_t bits = __float_as_uint(f);
    reinterpret_cast<uint16_t*>(sm)[i] = (uint16_t)(bits >> 16);  // exact: |v| <= 64
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tm)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tm;
  if (threadIdx.x == 0) {
    constexpr uint32_t id = idesc_bf16(128, N);
    long long t0 = clock64();
    int nm = 0;
    for (int r = 0; r < R; ++r) {
      for (int L = 2; L <= 5; ++L) {
        const uint32_t d = tmem + (uint32_t)(((L - 2) * N) % 512);
        for (int s = 1; s < L; ++s) {
          const int t = L - s;
          if (s > 4 || t > 4) continue;
          const int sa = mode ? 0 : s - 1, sb = mode ? 0 : t - 1;
          const uint64_t da = sdesc(smem_u32(A + sa * AB)), db = sdesc(smem_u32(B + sb * BB));
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            umma(d, da + 2 * k, db + 2 * k, id, (r > 0 || k > 0 || s > 1) ? 1u : 0u);
            ++nm;
          }
        }
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
    bool ok = false;
    for (int i = 0; i < (1 << 26) && !ok; ++i) ok = mbar_try(smem_u32(&bar), 0);
    long long t1 = clock64();
    if (!ok) atomicExch(err, 1);
    out[blockIdx.x] = (t1 - t0) * 1000 / nm;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

template <int N>
void run(int grid, int R, int mode, int data) {
  long long* d; int* e;
  cudaMalloc(&d, 256 * sizeof(long long));
  cudaMalloc(&e, sizeof(int));
  cudaMemset(e, 0, sizeof(int));
  const int smem = 200 * 1024;
  cudaFuncSetAttribute(probe<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  probe<N><<<grid, 128, smem>>>(R, mode, data, d, e);
  probe<N><<<grid, 128, smem>>>(R, mode, data, d, e);
  cudaError_t st = cudaDeviceSynchronize();
  long long h[256]; int he = 0;
  cudaMemcpy(h, d, grid * sizeof(long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(&he, e, sizeof(int), cudaMemcpyDeviceToHost);
  double mx = 0, mn = 1e30;
  for (int i = 0; i < grid; ++i) { mx = h[i] > mx ? h[i] : mx; mn = h[i] < mn ? h[i] : mn; }
  printf("N=%3d grid=%3d mode=%d(%s) data=%d(%s): cycles/mma min %.1f max %.1f (%s, err %d)\n", N, grid, mode,
         mode ? "one stage" : "slice pattern", data, data ? "random" : "const", mn / 1000.0, mx / 1000.0,
         cudaGetErrorString(st), he);
  cudaFree(d); cudaFree(e);
}

int main() {
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  for (int g : {1, nsm})
    for (int mode : {1, 0})
      for (int data : {0, 1}) {
        run<64>(g, 200, mode, data);
        run<128>(g, 200, mode, data);
      }
  return 0;
}
