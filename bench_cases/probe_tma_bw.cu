// Measurement driver: TMA load throughput (cp.async.bulk.tensor 2D,
// SWIZZLE_128B, 64 x 128 BF16 boxes = 16 KB, the slice-product kernels'
// boxes) against the number of CTAs (one per SM), the ring depth and the
// buffer size (48 MB: L2-resident; 2 GB: from DRAM).  One thread per CTA
// issues the loads; each stage is issued again as soon as it lands.  Every
// wait is bounded.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o gpurun_out/probe_tma_bw bench_cases/probe_tma_bw.cu -lcuda
//   gpurun_out/probe_tma_bw
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(a), "r"(parity) : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long gtime() { unsigned long long t; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)); return t; }

__global__ void __launch_bounds__(32, 1) tma_bw(const __grid_constant__ CUtensorMap tm, int R, int iters, int ntiles_x,
                                                  int ntiles_y, unsigned long long* out, int* err) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t bar[16];
  if (threadIdx.x != 0) return;
  for (int i = 0; i < R; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[i])));
  asm volatile("fence.mbarrier_init.release.cluster;");
  unsigned seed = blockIdx.x * 7919u + 13u;
  auto issue = [&](int st) {
    seed = seed * 1664525u + 1013904223u;
    const int tx = (seed >> 8) % ntiles_x, ty = (seed >> 20) % ntiles_y;
    const uint32_t b = smem_u32(&bar[st]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(16384) : "memory");
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(smem_u32(sm + st * 16384)), "l"((uint64_t)&tm), "r"(tx * 64), "r"(ty * 128), "r"(b) : "memory");
  };
  const unsigned long long t0 = gtime();
  for (int i = 0; i < R; ++i) issue(i);
  int it = 0;
  for (; it < iters; ++it) {
    const int st = it % R;
    const uint32_t ph = (uint32_t)((it / R) & 1);
    bool ok = false;
    for (int k = 0; k < (1 << 24) && !ok; ++k) ok = mbar_try(smem_u32(&bar[st]), ph);
    if (!ok) { atomicExch(err, 1); break; }
    if (it + R < iters) issue(st);
  }
  const unsigned long long t1 = gtime();
  out[blockIdx.x] = t1 - t0;
}

int main() {
  void* fn = nullptr; cudaDriverEntryPointQueryResult q;
  cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  auto enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  int nsm = 0; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  const size_t K = 8192;  // columns (BF16), 16 KB rows
  for (size_t mb : {48, 2048}) {
    const size_t rows = mb * 1024 * 1024 / (K * 2);
    void* buf; cudaMalloc(&buf, rows * K * 2); cudaMemset(buf, 1, rows * K * 2);
    CUtensorMap m;
    cuuint64_t dims[2] = {K, rows}; cuuint64_t strides[1] = {K * 2};
    cuuint32_t box[2] = {64, 128}; cuuint32_t es[2] = {1, 1};
    CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, buf, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { printf("encode failed %d\n", (int)r); return 1; }
    unsigned long long* d; int* e; cudaMalloc(&d, 256 * 8); cudaMalloc(&e, 4); cudaMemset(e, 0, 4);
    cudaFuncSetAttribute(tma_bw, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    for (int G : {1, 8, 38, 76, 152}) {
      if (G > nsm) continue;
      for (int R : {2, 4, 8, 12}) {
        const int iters = 2000;
        tma_bw<<<G, 32, 220 * 1024>>>(m, R, iters, (int)(K / 64), (int)(rows / 128), d, e);
        tma_bw<<<G, 32, 220 * 1024>>>(m, R, iters, (int)(K / 64), (int)(rows / 128), d, e);
        cudaError_t st = cudaDeviceSynchronize();
        unsigned long long h[256]; int he; cudaMemcpy(h, d, G * 8, cudaMemcpyDeviceToHost); cudaMemcpy(&he, e, 4, cudaMemcpyDeviceToHost);
        double mx = 0; for (int i = 0; i < G; ++i) mx = h[i] > mx ? h[i] : mx;
        const double bytes = (double)G * iters * 16384;
        printf("buf %5zu MB  CTAs %3d  stages %2d : %8.1f GB/s aggregate, %6.1f GB/s per CTA  (%s err %d)\n", mb, G, R,
               bytes / mx, bytes / mx / G, cudaGetErrorString(st), he);
      }
    }
    cudaFree(buf); cudaFree(d); cudaFree(e);
  }
  return 0;
}
