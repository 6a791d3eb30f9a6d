// Tensor-core backend of the mixed-precision mode: FP64 contractions
// computed as exact integer products of BF16 slices on tcgen05.
//
// Operand packing (pack_kernel): each row of A (an M x K view) and each
// column of B (a K x N view) is scaled by 2^-e with e the binary exponent of
// its largest magnitude, then cut into S slices of 7 bits,
//     x * 2^-e = sum_s q_s 2^(-7s),  q_s integers, |q_1| <= 128, |q_s| <= 64
// (balanced digits: each lower digit in [-64, 63], carries into the next),
// each exactly representable in BF16.  Complex operands contribute two packed
// rows (real, imaginary) per logical row.  Packed layout: [S][rows][K] BF16,
// K contiguous (K-major for UMMA), rows and K zero-padded to the tile sizes.
//
// Products (ozaki_kernel): for every pair (s, t) with s + t <= S + 1 the
// slice product A_s B_t^T is accumulated by tcgen05.mma (kind::f16, BF16
// inputs, FP32 accumulate in TMEM) into the accumulator of its level
// L = s + t.  With |q_1| <= 128 and |q_s| <= 64 the products of one level
// at one K index add up to at most 2^14 + 2^13 + 2^13 = 2^15 in magnitude
// (level 7 of S = 6; 2^14 + 2^13 + 2^12 for level 6), so the FP32 level sums
// over a 512-wide K chunk stay within 2^24 and are exact integers; after
// every chunk the epilogue warps drain the TMEM
// accumulators into FP64 registers with their 2^(-7L) weights.  The final
// value is scaled back by 2^(e_row + e_col); real/imaginary rows of complex
// operands are combined with a lane-pair shuffle and written through the
// same strided output decoder as the FP64 kernel.
//
// Pipeline (two variants, TcCfg in gemm_tc.h): warp 0 issues TMA loads
// (SWIZZLE_128B) into a shared-memory ring, one (A_s, B_s) slice pair per
// stage; warp 1 owns TMEM and issues the MMAs from one thread; the other
// warps drain TMEM, EPI / 4 per TMEM lane quarter, each taking a slice of
// the tile's columns.  The wide variant (64 columns, 8 stages, 16 drain
// warps) runs one CTA per SM; the narrow one (32 columns, 5 stages, 8 drain
// warps) two, so that one CTA's drain overlaps the other's MMAs -- for
// contractions with short K, whose time is per-CTA latency.
// Every wait has an iteration limit: on expiry the kernel records an error
// code, stops issuing work, waits (bounded) for its own operations and frees
// TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>

#include "engine.h"
#include "gemm_tc.h"
#include "slice_math.cuh"

namespace tdcc {

// ---------------------------------------------------------------------------
// packing
// ---------------------------------------------------------------------------
// Digits of two neighbouring elements of a packed row (same exponent e), one
// BF16 pair per slice: out is the packed buffer as BF16 pairs, plane2 the
// pairs per slice, idx2 the pair's index within a slice.
__device__ __forceinline__ void store_digit_pair(uint32_t* out, size_t plane2, size_t idx2, double x0, double x1,
                                                 int e, int nbits, int S) {
  int q0[TC_MAX_SLICES], q1[TC_MAX_SLICES];
  balanced_digits(fixed_point(x0, e, nbits), S, q0);
  balanced_digits(fixed_point(x1, e, nbits), S, q1);
  const bool n0 = __double_as_longlong(x0) < 0, n1 = __double_as_longlong(x1) < 0;  // sign bits
#pragma unroll
  for (int s = 0; s < TC_MAX_SLICES; ++s)
    if (s < S) out[s * plane2 + idx2] = digit_pair_bf16x2(n0 ? -q0[s] : q0[s], n1 ? -q1[s] : q1[s]);
}

// One block per logical row (per batch; the real and imaginary rows of a
// complex row together): pass 1 takes the binary exponent e of the row's
// max |x| (max = f 2^e, f in [0.5, 1); integer ops on the bit patterns, the
// order of |x| for finite doubles), pass 2 cuts |x| 2^-e truncated to 7S
// bits into S balanced digits (|q_1| <= 128, |q_s| <= 64, exact in BF16) and
// gives them the sign of x:
//   x 2^-e ~= sum_s q_s 2^(-7s).
// The real and imaginary rows share e, so that the slice-product epilogue
// combines re*re - im*im and re*im + im*re exactly in integers.  K padding
// is written as zero; padding rows (up to the tile multiple of each batch)
// are not written at all: they only feed accumulator rows (A) or columns (B)
// that the product kernel never stores, and their exponent entries only
// scale those values, so whatever the buffer holds there is harmless.
// With tab set, the K offsets (the same for every row) are decoded once per
// block into shared memory as 32-bit integers (K of them) and both passes
// read them there.
__global__ void __launch_bounds__(1024) pack_kernel(const PackArgs p, int tab) {
  extern __shared__ int kofs[];
  const int per = p.cplx ? 2 : 1;
  const int z = blockIdx.x / p.rows, m = blockIdx.x - z * p.rows;  // one block per live row
  long long ro = 0;
  decomp_tc(p.gr, m, ro);
  ro += z * p.bs;
  if (tab) {
    for (int k = threadIdx.x; k < p.K; k += blockDim.x) {
      long long ko;
      decomp_tc(p.gk, k, ko);
      kofs[k] = (int)ko;
    }
    __syncthreads();
  }
  auto koff = [&](int k) -> long long {
    if (tab) return kofs[k];
    long long ko;
    decomp_tc(p.gk, k, ko);
    return ko;
  };
  const unsigned long long* bits = static_cast<const unsigned long long*>(p.src);
  const double* src = static_cast<const double*>(p.src);
  constexpr unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long mx = 0;
  // four independent loads in flight per thread (complex elements as one 16-byte load)
  constexpr int U = 4;
  for (int k0 = threadIdx.x; k0 < p.K; k0 += U * blockDim.x) {
    unsigned long long v[U][2];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const int k = k0 + j * blockDim.x;
      v[j][0] = v[j][1] = 0ull;
      if (k < p.K) {
        const long long e = ro + koff(k);
        if (p.cplx) {
          const ulonglong2 w = *reinterpret_cast<const ulonglong2*>(bits + 2 * e);
          v[j][0] = w.x;
          v[j][1] = w.y;
        } else {
          v[j][0] = bits[e];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < U; ++j) mx = max(mx, max(v[j][0] & kAbs, v[j][1] & kAbs));
  }
  for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  __shared__ unsigned long long wmax[32];
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = max(mx, wmax[w]);
  const int E = (int)(mx >> 52);
  const int eb = mx != 0 ? (E > 0 ? E - 1022 : -1022) + kExpBias : 0;
  const size_t prow = (size_t)z * p.rows_pad + (size_t)m * per;  // first packed row
  if (threadIdx.x == 0) {
    p.exps[prow] = eb;
    if (p.cplx) p.exps[prow + 1] = eb;
  }
  const int e = row_exp(eb);
  const int nbits = 7 * p.S;
  uint32_t* out = static_cast<uint32_t*>(p.out);  // BF16 pairs (K_pad is even)
  const size_t plane2 = (size_t)p.nb * p.rows_pad * (p.K_pad / 2);
  // pass 2 over pairs of neighbouring K indices (one 4-byte store per slice
  // and part), two pairs per thread: four loads in flight
  constexpr int U2 = 2;
  for (int k0 = 2 * threadIdx.x; k0 < p.K_pad; k0 += 2 * U2 * blockDim.x) {
    double x[U2][2][2];  // [pair][element][part]
#pragma unroll
    for (int j = 0; j < U2; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = k0 + 2 * j * blockDim.x + h;
        x[j][h][0] = x[j][h][1] = 0.0;
        if (k < p.K) {
          const long long el = ro + koff(k);
          if (p.cplx) {
            const double2 w = *reinterpret_cast<const double2*>(src + 2 * el);
            x[j][h][0] = w.x;
            x[j][h][1] = w.y;
          } else {
            x[j][h][0] = src[el];
          }
        }
      }
#pragma unroll
    for (int j = 0; j < U2; ++j) {
      const int k = k0 + 2 * j * blockDim.x;
      if (k >= p.K_pad) break;
      for (int part = 0; part < per; ++part)
        store_digit_pair(out, plane2, ((prow + part) * p.K_pad + k) / 2, x[j][0][part], x[j][1][part], e, nbits,
                         p.S);
    }
  }
}

// Rows of up to 64 W KP elements: W warps per logical row, 8 / W rows per
// 256-thread block.  Each lane keeps KP pairs of neighbours in registers
// (pair index 32 w + lane + 32 W j for warp w of the row), so the row is read
// once: the exponent comes from shuffles (and shared memory across the W
// warps), the digits from the registers (same exponent, digits and layout as
// pack_kernel).
template <int KP, int W>
__global__ void __launch_bounds__(256) pack_rows_regs_kernel(const PackArgs p) {
  static_assert(W == 1 || W == 2 || W == 4 || W == 8, "warps per row divide the block");
  constexpr int RPB = 8 / W;
  const int per = p.cplx ? 2 : 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = warp % W;  // warp within the row
  const long long lr = (long long)blockIdx.x * RPB + warp / W;  // logical row over all batches
  const bool live = lr < (long long)p.nb * p.rows;              // uniform over the row's warps
  const int z = live ? (int)(lr / p.rows) : 0, m = live ? (int)(lr - (long long)z * p.rows) : 0;
  long long ro = 0;
  decomp_tc(p.gr, m, ro);
  ro += z * p.bs;
  const double* src = static_cast<const double*>(p.src);
  constexpr unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull;
  double x[KP][2][2];  // [pair][element][part]
  unsigned long long mx = 0;
#pragma unroll
  for (int j = 0; j < KP; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 2 * (32 * wr + lane + 32 * W * j) + h;
      x[j][h][0] = x[j][h][1] = 0.0;
      if (live && k < p.K) {
        long long ko;
        decomp_tc(p.gk, k, ko);
        const long long el = ro + ko;
        if (p.cplx) {
          const double2 v = *reinterpret_cast<const double2*>(src + 2 * el);
          x[j][h][0] = v.x;
          x[j][h][1] = v.y;
        } else {
          x[j][h][0] = src[el];
        }
      }
      mx = max(mx, max((unsigned long long)__double_as_longlong(x[j][h][0]) & kAbs,
                       (unsigned long long)__double_as_longlong(x[j][h][1]) & kAbs));
    }
  for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  if (W > 1) {
    __shared__ unsigned long long wmax[8];
    if (lane == 0) wmax[warp] = mx;
    __syncthreads();  // every thread of the block arrives (no return above)
    const int w0 = warp - wr;
#pragma unroll
    for (int w = 0; w < W; ++w) mx = max(mx, wmax[w0 + w]);
  }
  if (!live) return;
  const int E = (int)(mx >> 52);
  const int eb = mx != 0 ? (E > 0 ? E - 1022 : -1022) + kExpBias : 0;
  const size_t prow = (size_t)z * p.rows_pad + (size_t)m * per;
  if (wr == 0 && lane == 0) {
    p.exps[prow] = eb;
    if (p.cplx) p.exps[prow + 1] = eb;
  }
  const int e = row_exp(eb);
  const int nbits = 7 * p.S;
  uint32_t* out = static_cast<uint32_t*>(p.out);  // BF16 pairs (K_pad is even)
  const size_t plane2 = (size_t)p.nb * p.rows_pad * (p.K_pad / 2);
#pragma unroll
  for (int j = 0; j < KP; ++j) {
    const int k = 2 * (32 * wr + lane + 32 * W * j);
    if (k >= p.K_pad) break;
    for (int part = 0; part < per; ++part)
      store_digit_pair(out, plane2, ((prow + part) * p.K_pad + k) / 2, x[j][0][part], x[j][1][part], e, nbits, p.S);
  }
}

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t c) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(c));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false after `limit` polls (each poll may suspend briefly)
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try(a, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma3d(uint32_t dst, const CUtensorMap* tm, int x, int y, int z, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(z), "r"(mbar)
      : "memory");
}
// UMMA shared-memory descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tmem_ld16u(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
}
// issue only: the caller waits (tcgen05.wait::ld) before reading r
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_st16u(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// ---------------------------------------------------------------------------
// slice-product kernel
// ---------------------------------------------------------------------------
constexpr int kWaitLimit = 1 << 22;

template <class C>
struct TcShared {
  uint64_t full[C::STAGES];
  uint64_t empty[C::STAGES];
  uint64_t accfull, accempty, done;
  uint32_t tmem;
  volatile int abort;  // set by any role on an expired wait; polled by all
  long long col_off[C::BN];  // output offset of each logical column of the tile (-1: outside)
  int col_exp[C::BN];        // exponent of each packed column of B
};

template <class SH>
__device__ __forceinline__ void fail(SH* sh, int* err, int code) {
  sh->abort = 1;
  atomicCAS(err, 0, code);
}

template <bool AC, bool BC, class C>
__global__ void __launch_bounds__(C::THREADS, C::MINB)
    ozaki_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TcArgs g) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t* stA = sm;                                   // STAGES x 16 KB
  uint8_t* stB = sm + C::STAGES * TC_A_BYTES;          // STAGES x BN x 128 B
  TcShared<C>* sh = (TcShared<C>*)(stB + C::STAGES * C::B_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = g.S;
  const int ncols = g.tmem_cols;

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::STAGES; ++i) {
      mbar_init(smem_u32(&sh->full[i]), 1);
      mbar_init(smem_u32(&sh->empty[i]), 1);
    }
    mbar_init(smem_u32(&sh->accfull), 1);
    mbar_init(smem_u32(&sh->accempty), 32 * C::EPI);
    mbar_init(smem_u32(&sh->done), 1);
    sh->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = sh->tmem;

  const int mt = g.m_fast ? blockIdx.x : blockIdx.y, nt = g.m_fast ? blockIdx.y : blockIdx.x;
  const int zb = blockIdx.z / g.nsplit;                 // batch
  const int kb0 = (blockIdx.z - zb * g.nsplit) * g.kb_per_split;
  const int rowA0 = (g.bat_a ? zb * g.rowsA_pad : 0);  // packed-row origin of this batch
  const int rowB0 = (g.bat_b ? zb * g.rowsB_pad : 0);
  const int kb1 = min(g.kblocks, kb0 + g.kb_per_split);
  const int nkb = kb1 - kb0;
  const int nchunks = (nkb + TC_CHUNK_KB - 1) / TC_CHUNK_KB;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0;
      for (int kb = kb0; kb < kb1 && !sh->abort; ++kb)
        for (int s = 0; s < S && !sh->abort; ++s, ++it) {
          const int st = it % C::STAGES;
          const uint32_t ph = (uint32_t)((it / C::STAGES) & 1);
          if (!mbar_wait(smem_u32(&sh->empty[st]), ph ^ 1u, kWaitLimit)) {
            fail(sh, g.err, 1);
            break;
          }
          const uint32_t fb = smem_u32(&sh->full[st]);
          mbar_expect_tx(fb, TC_A_BYTES + C::B_BYTES);
          tma3d(smem_u32(stA + st * TC_A_BYTES), &tmA, kb * TC_BK, rowA0 + mt * TC_BM, s, fb);
          tma3d(smem_u32(stB + st * C::B_BYTES), &tmB, kb * TC_BK, rowB0 + nt * C::BN, s, fb);
        }
      // drain: every issued load must land before the CTA exits
      const int issued = it;
      for (int j = (issued > C::STAGES ? issued - C::STAGES : 0); j < issued; ++j)
        mbar_wait(smem_u32(&sh->full[j % C::STAGES]), (uint32_t)((j / C::STAGES) & 1), kWaitLimit);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t id = idesc_bf16(TC_BM, C::BN);
      int it = 0;
      for (int c = 0; c < nchunks && !sh->abort; ++c) {
        if (c > 0 && !mbar_wait(smem_u32(&sh->accempty), (uint32_t)((c - 1) & 1), kWaitLimit)) {
          fail(sh, g.err, 2);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int kbs = kb0 + c * TC_CHUNK_KB, kbe = min(kb1, kbs + TC_CHUNK_KB);
        bool first = true;
        for (int kb = kbs; kb < kbe && !sh->abort; ++kb, it += S) {
          bool ok = true;
          for (int s = 0; s < S; ++s) {
            const int j = it + s;
            if (!mbar_wait(smem_u32(&sh->full[j % C::STAGES]), (uint32_t)((j / C::STAGES) & 1), kWaitLimit)) {
              ok = false;
              break;
            }
          }
          if (!ok) {
            fail(sh, g.err, 3);
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          for (int L = 2; L <= S + 1; ++L) {
            const uint32_t dacc = tmem + (uint32_t)((L - 2) * C::BN);
            int np = 0;
            for (int s = 1; s < L; ++s) {
              const int t = L - s;
              if (s > S || t > S) continue;
              const int sa = (it + s - 1) % C::STAGES, sb = (it + t - 1) % C::STAGES;
              const uint64_t da = sdesc(smem_u32(stA + sa * TC_A_BYTES));
              const uint64_t db = sdesc(smem_u32(stB + sb * C::B_BYTES));
#pragma unroll
              for (int k = 0; k < TC_BK / 16; ++k) {
                const uint32_t accf = (first && np == 0 && k == 0) ? 0u : 1u;
                umma(dacc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), id, accf);
              }
              ++np;
            }
          }
          first = false;
          for (int s = 0; s < S; ++s) umma_commit(smem_u32(&sh->empty[(it + s) % C::STAGES]));
        }
        umma_commit(smem_u32(&sh->accfull));
      }
      // all issued MMAs complete before TMEM is released
      umma_commit(smem_u32(&sh->done));
      mbar_wait(smem_u32(&sh->done), 0, kWaitLimit);
    }
  } else {
    // ---------------- epilogue (warps 2 .. 2 + C::EPI - 1) ----------------
    // C::EPI / 4 warps per TMEM lane quarter, each owning a slice of the
    // tile's columns: the drain is latency-bound per warp, so the work is
    // spread over warps.
    constexpr int kWq = C::EPI / 4;   // warps per lane quarter
    constexpr int kCw = C::BN / kWq;        // packed columns per warp (multiple of 16)
    const int q = warp & 3;             // TMEM lane quarter this warp may access
    const int hcol = (warp - 2) >> 2;   // column slice of this warp
    const int row = q * 32 + lane;      // tile row == TMEM lane
    // Exact sums in integer units of 2^-u, u = 7 (min(S,5) + 1).  The level
    // sums are integers (products of integer slices, FP32-exact per chunk),
    // so sum_L v_L 2^(u - 7L) is exact for S <= 5 (the seventh-slice level of
    // S = 6 is truncated by 7 bits, below its own resolution) and stays
    // below 2^52 per chunk: int64 holds up to 2^11 chunks.  No FP64
    // arithmetic until the final conversion -- the FP64 pipe is narrow.
    const int u = 7 * ((S < 5 ? S : 5) + 1);
    {
      // per-tile column data, shared by all rows: output offsets and B exponents
      const int t = threadIdx.x - 64;  // 0 .. 32 * C::EPI - 1
      constexpr int ncl = BC ? C::BN / 2 : C::BN;
      if (t < ncl) {
        const int n = nt * ncl + t;
        long long o = -1;
        if (n < g.N) decomp_tc(g.gnC, n, o);
        sh->col_off[t] = o;
      }
      if (t < C::BN) sh->col_exp[t] = row_exp(g.expB[rowB0 + nt * C::BN + t]);
      asm volatile("bar.sync 1, %0;" ::"n"(32 * C::EPI) : "memory");  // the epilogue warps
    }
    // Row data and the staging tile of this warp (final chunk): the operand
    // ring is idle once the last accumulators are complete.
    const int prow = mt * TC_BM + row;          // packed row of A (within the batch)
    const int m = AC ? (prow >> 1) : prow;
    const bool odd = AC && (lane & 1);
    constexpr int ncol_log = BC ? C::BN / 2 : C::BN;  // logical output columns in this tile
    constexpr int rows_out = AC ? 16 : 32;             // logical output rows of this warp
    constexpr int RS = ncol_log + 1;                    // staging row stride (double2), padded
    double2* stage = reinterpret_cast<double2*>(sm) + (size_t)q * (32 * RS);
    const int lr = AC ? (lane >> 1) : lane;            // this lane's staging row
    const uint32_t tl = (uint32_t)(q * 32) << 16;      // TMEM lane base of this warp
    const uint32_t t64 = (uint32_t)(S * C::BN);        // int64 partial sums: 2 words per column
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      // warp-uniform decisions: tcgen05.ld/st and the shuffles below are collective
      if (__any_sync(0xffffffffu, sh->abort != 0)) {
        ok = false;
        break;
      }
      const bool got = mbar_wait(smem_u32(&sh->accfull), (uint32_t)(c & 1), kWaitLimit);
      if (!__all_sync(0xffffffffu, got)) {
        fail(sh, g.err, 4);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const bool last = c == nchunks - 1;
      int ebase = 0;
      if (last) {
        const int ea = prow < g.rowsA_pad ? row_exp(g.expA[rowA0 + prow]) : 0;
        ebase = ea - u + (g.alpha_pow2 ? g.alpha_e : 0);
      }
      // 16 columns at a time (a runtime loop keeps the code small)
#pragma unroll 1
      for (int j0 = hcol * kCw; j0 < (hcol + 1) * kCw; j0 += 16) {
        // all loads of the group in flight before one wait (TMEM latency)
        constexpr int kMaxLv = 6;  // levels 2..7 (S <= 6)
        long long a16[16];
        if (c > 0) {
          uint32_t lo[16], hi[16];
          tmem_ld16_nowait(tmem + tl + t64 + 2 * j0, lo);
          tmem_ld16_nowait(tmem + tl + t64 + 2 * j0 + 16, hi);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) a16[j] = (long long)(((unsigned long long)hi[j] << 32) | lo[j]);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) a16[j] = 0;
        }
        // levels in batches of three loads before one wait
#pragma unroll
        for (int L0 = 2; L0 <= kMaxLv + 1; L0 += 3) {
          if (L0 > S + 1) break;
          uint32_t lv[3][16];
#pragma unroll
          for (int i = 0; i < 3; ++i)
            if (L0 + i <= S + 1) tmem_ld16_nowait(tmem + tl + (uint32_t)((L0 + i - 2) * C::BN + j0), lv[i]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const int L = L0 + i;
            if (L > S + 1) break;
            const int sh = u - 7 * L;
            // |v| <= 2^24: a 32-bit conversion is exact and stays off the FP64 pipe
            if (sh >= 0) {
#pragma unroll
              for (int j = 0; j < 16; ++j) a16[j] += (long long)__float2int_rn(__uint_as_float(lv[i][j])) << sh;
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j) a16[j] += (long long)__float2int_rn(__uint_as_float(lv[i][j])) >> (-sh);
            }
          }
        }
        if (!last) {
          uint32_t lo[16], hi[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            lo[j] = (uint32_t)(unsigned long long)a16[j];
            hi[j] = (uint32_t)((unsigned long long)a16[j] >> 32);
          }
          tmem_st16u(tmem + tl + t64 + 2 * j0, lo);
          tmem_st16u(tmem + tl + t64 + 2 * j0 + 16, hi);
          continue;
        }
        // final chunk: combine, scale back, stage (lanes own rows here)
        const bool neg = g.alpha_pow2 && g.alpha_neg;
        constexpr int NJ = BC ? 8 : 16;  // logical columns in this group
#pragma unroll
        for (int k = 0; k < NJ; ++k) {
          const int jj = (BC ? j0 / 2 : j0) + k;
          // integer combine: the pair exponents are shared, so these are exact
          long long re, im;
          if constexpr (BC) {
            const long long x0 = a16[2 * k], x1 = a16[2 * k + 1];
            if constexpr (AC) {
              const long long p0 = __shfl_xor_sync(0xffffffffu, x0, 1);
              const long long p1 = __shfl_xor_sync(0xffffffffu, x1, 1);
              // even lane: (rr, ri) own, (ir, ii) partner; odd lane the reverse
              const long long rr = odd ? p0 : x0, ri = odd ? p1 : x1, ir = odd ? x0 : p0, ii = odd ? x1 : p1;
              re = rr - ii;
              im = ri + ir;
            } else {
              re = x0;
              im = x1;
            }
          } else {
            const long long x = a16[k];
            if constexpr (AC) {
              const long long p = __shfl_xor_sync(0xffffffffu, x, 1);
              re = odd ? p : x;
              im = odd ? x : p;
            } else {
              re = x;
              im = 0;
            }
          }
          // with complex A the two lanes of a pair hold the same output: split columns
          if (AC && ((jj & 1) != (lane & 1))) continue;
          const int E = ebase + sh->col_exp[BC ? 2 * jj : jj];
          double vr, vi;
          if (g.alpha_pow2) {
            vr = scaled_i64_to_double(neg ? -re : re, E);
            vi = scaled_i64_to_double(neg ? -im : im, E);
          } else {
            const double dr = scaled_i64_to_double(re, E), di = scaled_i64_to_double(im, E);
            vr = g.ar * dr - g.ai * di;
            vi = g.ar * di + g.ai * dr;
          }
          stage[lr * RS + jj] = make_double2(vr, vi);
        }
      }
      if (!last) asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(smem_u32(&sh->accempty));
    }
    if (ok && !__any_sync(0xffffffffu, sh->abort != 0)) {
      // write the staged tile: rows of contiguous columns per pass
      __syncwarp();
      long long coffm = 0;
      if (m < g.M) decomp_tc(g.gmC, m, coffm);
      double2* Cc = static_cast<double2*>(g.C) + (g.cc ? zb * g.bsC : 0);
      double* Cr = static_cast<double*>(g.C) + (g.cc ? 0 : zb * g.bsC);
      const int m0w = AC ? ((mt * TC_BM + q * 32) >> 1) : (mt * TC_BM + q * 32);
      constexpr int NCW = ncol_log / kWq;  // logical columns of this warp (<= 32)
      // every lane owns a (row, column) pair: NCW columns by 32 / NCW rows per
      // pass.  Accumulated outputs are added in L2 (reductions without a
      // return value), so the pass issues no load: one writer per element
      // and launch (split K aside), so the single addition c + v is the same
      // as a read-modify-write.
      static_assert(32 % NCW == 0, "columns per warp divide the warp");
      constexpr int RPP = 32 / NCW;
      constexpr int NPASS = (rows_out + RPP - 1) / RPP;
      const int lc = lane % NCW, lrw = lane / NCW;
      const int cc = hcol * NCW + lc;  // this lane's column while storing
      const long long cn = sh->col_off[cc];
      const int nrows = min(rows_out, g.M - m0w);
      const bool red = g.acc || g.atomic;
#pragma unroll 4
      for (int p = 0; p < NPASS; ++p) {
        const int r = p * RPP + lrw;
        // row offsets live in the lanes of the rows' TMEM rows
        const long long cm = __shfl_sync(0xffffffffu, coffm, (AC ? 2 * r : r) & 31);
        if (r >= nrows || cn < 0) continue;
        const long long off = cm + cn;
        const double2 v = stage[r * RS + cc];
        if (g.cc) {
          if (red) {
            atomicAdd(&Cc[off].x, v.x);
            atomicAdd(&Cc[off].y, v.y);
          } else {
            Cc[off] = v;
          }
        } else {
          if (red)
            atomicAdd(&Cr[off], v.x);
          else
            Cr[off] = v.x;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------------------
// 128-column tile for S <= 4 slices (TcTile128): one K range per CTA.
//
// A tcgen05.mma of 128 x N x 16 costs the same ~71 cycles for every N <= 128,
// and the TMA unit of an SM delivers about 62 GB/s, so the 64-column tile
// spends half of its MMA time and 1.5x the loaded bytes per output that a
// 128-column tile does.  S level accumulators of 128 columns fill TMEM
// (S <= 4), which leaves no room for int64 partial sums across K chunks:
// each CTA therefore takes at most one exact chunk of K (the planner splits
// longer K across CTAs, whose results meet in the output by L2 reductions)
// and drains TMEM once.  Level sums per K index are at most
// 2^13 + 2^12 + 2^12 + 2^13 = 24576 (S = 4), so 10 K blocks (640) stay
// below 2^24 and exact in FP32 (tc_chunk_kblocks).  The ring holds single
// slices (a 128 x 64 tile of A or of B) with their own barriers: the
// products of a K block run row by row, (1,1) .. (1,S), (2,1) .., and each
// slice is released right after its last product, so the TMA (the bound
// of this tile: about 62 GB/s per SM) keeps loading the next block while
// the current one finishes.  The drain takes 16 columns at a time per warp,
// stages them in the idle operand ring (one area per warp) and writes them
// at once, so the whole tile is never staged.
// ---------------------------------------------------------------------------
template <bool AC, bool BC>
__global__ void __launch_bounds__(TcTile128::THREADS, 1)
    ozaki_tile128_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                         const TcArgs g) {
  using C = TcTile128;
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t* ring = sm;  // STAGES slots of 16 KB: one slice of A or of B each
  TcShared<C>* sh = (TcShared<C>*)(ring + C::STAGES * C::SLOT_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = g.S;
  const int ncols = g.tmem_cols;

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::STAGES; ++i) {
      mbar_init(smem_u32(&sh->full[i]), 1);
      mbar_init(smem_u32(&sh->empty[i]), 1);
    }
    mbar_init(smem_u32(&sh->accfull), 1);
    mbar_init(smem_u32(&sh->accempty), 32 * C::EPI);
    mbar_init(smem_u32(&sh->done), 1);
    sh->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = sh->tmem;

  const int mt = g.m_fast ? blockIdx.x : blockIdx.y, nt = g.m_fast ? blockIdx.y : blockIdx.x;
  const int zb = blockIdx.z / g.nsplit;  // batch
  const int kb0 = (blockIdx.z - zb * g.nsplit) * g.kb_per_split;
  const int rowA0 = (g.bat_a ? zb * g.rowsA_pad : 0);
  const int rowB0 = (g.bat_b ? zb * g.rowsB_pad : 0);
  const int kb1 = min(g.kblocks, kb0 + g.kb_per_split);
  // Per K block the 2S slices enter the ring in the order A1, B1 .. BS,
  // A2 .. AS, and the products run row by row, (1,1) .. (1,S), (2,1) ..
  // (2,S-1), .., (S,1): products start once A1 and B1 have landed, and after
  // row s both A_s and B_(S+1-s) have had their last use and are released.
  // Position of a slice within its block: A1 -> 0, B_t -> t, A_s -> S + s - 1.
  const int per = 2 * S;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int j = 0;
      for (int kb = kb0; kb < kb1 && !sh->abort; ++kb)
        for (int i = 0; i < per && !sh->abort; ++i, ++j) {
          const int st = j % C::STAGES;
          const uint32_t ph = (uint32_t)((j / C::STAGES) & 1);
          if (!mbar_wait(smem_u32(&sh->empty[st]), ph ^ 1u, kWaitLimit)) {
            fail(sh, g.err, 1);
            break;
          }
          const uint32_t fb = smem_u32(&sh->full[st]);
          mbar_expect_tx(fb, C::SLOT_BYTES);
          if (i == 0 || i > S)  // A_1, then A_2 .. A_S
            tma3d(smem_u32(ring + st * C::SLOT_BYTES), &tmA, kb * TC_BK, rowA0 + mt * TC_BM, i == 0 ? 0 : i - S, fb);
          else  // B_1 .. B_S
            tma3d(smem_u32(ring + st * C::SLOT_BYTES), &tmB, kb * TC_BK, rowB0 + nt * C::BN, i - 1, fb);
        }
      const int issued = j;
      for (int q = (issued > C::STAGES ? issued - C::STAGES : 0); q < issued; ++q)
        mbar_wait(smem_u32(&sh->full[q % C::STAGES]), (uint32_t)((q / C::STAGES) & 1), kWaitLimit);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t id = idesc_bf16(TC_BM, C::BN);
      int j0 = 0;
      bool first = true;
      for (int kb = kb0; kb < kb1 && !sh->abort; ++kb, j0 += per) {
        bool ok = true;
        for (int s = 1; s <= S && ok; ++s) {
          const int ja = j0 + (s == 1 ? 0 : S + s - 1);  // A_s
          if (!mbar_wait(smem_u32(&sh->full[ja % C::STAGES]), (uint32_t)((ja / C::STAGES) & 1), kWaitLimit)) {
            ok = false;
            break;
          }
          const uint64_t da = sdesc(smem_u32(ring + (ja % C::STAGES) * C::SLOT_BYTES));
          for (int t = 1; t <= S + 1 - s; ++t) {
            const int jb = j0 + t;  // B_t
            if (s == 1 &&
                !mbar_wait(smem_u32(&sh->full[jb % C::STAGES]), (uint32_t)((jb / C::STAGES) & 1), kWaitLimit)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint64_t db = sdesc(smem_u32(ring + (jb % C::STAGES) * C::SLOT_BYTES));
            const uint32_t dacc = tmem + (uint32_t)((s + t - 2) * C::BN);
#pragma unroll
            for (int k = 0; k < TC_BK / 16; ++k) {
              // the first product of each level (s = 1) in the first K block starts its accumulator
              const uint32_t accf = (first && s == 1 && k == 0) ? 0u : 1u;
              umma(dacc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), id, accf);
            }
          }
          if (!ok) break;
          // A_s and B_(S+1-s) have had their last use: free their slots
          umma_commit(smem_u32(&sh->empty[ja % C::STAGES]));
          umma_commit(smem_u32(&sh->empty[(j0 + S + 1 - s) % C::STAGES]));
        }
        if (!ok) {
          fail(sh, g.err, 3);
          break;
        }
        first = false;
      }
      umma_commit(smem_u32(&sh->accfull));
      umma_commit(smem_u32(&sh->done));
      mbar_wait(smem_u32(&sh->done), 0, kWaitLimit);
    }
  } else {
    // ---------------- epilogue (warps 2 .. 17) ----------------
    constexpr int kWq = C::EPI / 4;   // 4 warps per lane quarter
    constexpr int kCw = C::BN / kWq;  // 32 packed columns per warp
    const int q = warp & 3;
    const int hcol = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const int u = 7 * (S + 1);  // S <= 4: sum_L v_L 2^(u - 7L) is exact in int64
    {
      const int t = threadIdx.x - 64;
      constexpr int ncl = BC ? C::BN / 2 : C::BN;
      if (t < ncl) {
        const int n = nt * ncl + t;
        long long o = -1;
        if (n < g.N) decomp_tc(g.gnC, n, o);
        sh->col_off[t] = o;
      }
      if (t < C::BN) sh->col_exp[t] = row_exp(g.expB[rowB0 + nt * C::BN + t]);
      asm volatile("bar.sync 1, %0;" ::"n"(32 * C::EPI) : "memory");
    }
    const int prow = mt * TC_BM + row;
    const int m = AC ? (prow >> 1) : prow;
    const bool odd = AC && (lane & 1);
    constexpr int NJ = BC ? 8 : 16;          // logical columns per 16 packed columns
    constexpr int rows_out = AC ? 16 : 32;    // logical rows of this warp
    constexpr int RS = NJ + 1;                // staging row stride (double2), padded
    double2* stage = reinterpret_cast<double2*>(sm) + (size_t)(warp - 2) * (32 * RS);
    const int lr = AC ? (lane >> 1) : lane;
    const uint32_t tl = (uint32_t)(q * 32) << 16;
    bool ok = !__any_sync(0xffffffffu, sh->abort != 0);
    if (ok) {
      const bool got = mbar_wait(smem_u32(&sh->accfull), 0u, kWaitLimit);
      if (!__all_sync(0xffffffffu, got)) {
        fail(sh, g.err, 4);
        ok = false;
      }
    }
    if (ok && __any_sync(0xffffffffu, sh->abort != 0)) ok = false;
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int ea = prow < g.rowsA_pad ? row_exp(g.expA[rowA0 + prow]) : 0;
      const int ebase = ea - u + (g.alpha_pow2 ? g.alpha_e : 0);
      const bool neg = g.alpha_pow2 && g.alpha_neg;
      long long coffm = 0;
      if (m < g.M) decomp_tc(g.gmC, m, coffm);
      double2* Cc = static_cast<double2*>(g.C) + (g.cc ? zb * g.bsC : 0);
      double* Cr = static_cast<double*>(g.C) + (g.cc ? 0 : zb * g.bsC);
      const int m0w = AC ? ((mt * TC_BM + q * 32) >> 1) : (mt * TC_BM + q * 32);
      const int nrows = min(rows_out, g.M - m0w);
      const bool red = g.acc || g.atomic;
      constexpr int RPP = 32 / NJ;  // rows per store pass
      constexpr int NPASS = rows_out / RPP;
      const int lc = lane % NJ, lrw = lane / NJ;
#pragma unroll 1
      for (int j0 = hcol * kCw; j0 < (hcol + 1) * kCw; j0 += 16) {
        long long a16[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) a16[j] = 0;
#pragma unroll
        for (int L0 = 2; L0 <= 5; L0 += 2) {
          if (L0 > S + 1) break;
          uint32_t lv[2][16];
#pragma unroll
          for (int i = 0; i < 2; ++i)
            if (L0 + i <= S + 1) tmem_ld16_nowait(tmem + tl + (uint32_t)((L0 + i - 2) * C::BN + j0), lv[i]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int L = L0 + i;
            if (L > S + 1) break;
            const int shl = u - 7 * L;  // >= 0 for L <= S + 1
#pragma unroll
            for (int j = 0; j < 16; ++j) a16[j] += (long long)__float2int_rn(__uint_as_float(lv[i][j])) << shl;
          }
        }
        __syncwarp();  // the previous group's stores have read the staging area
#pragma unroll
        for (int k = 0; k < NJ; ++k) {
          const int jj = (BC ? j0 / 2 : j0) + k;  // logical column within the tile
          long long re, im;
          if constexpr (BC) {
            const long long x0 = a16[2 * k], x1 = a16[2 * k + 1];
            if constexpr (AC) {
              const long long p0 = __shfl_xor_sync(0xffffffffu, x0, 1);
              const long long p1 = __shfl_xor_sync(0xffffffffu, x1, 1);
              const long long rr = odd ? p0 : x0, ri = odd ? p1 : x1, ir = odd ? x0 : p0, ii = odd ? x1 : p1;
              re = rr - ii;
              im = ri + ir;
            } else {
              re = x0;
              im = x1;
            }
          } else {
            const long long x = a16[k];
            if constexpr (AC) {
              const long long p = __shfl_xor_sync(0xffffffffu, x, 1);
              re = odd ? p : x;
              im = odd ? x : p;
            } else {
              re = x;
              im = 0;
            }
          }
          if (AC && ((k & 1) != (lane & 1))) continue;
          const int E = ebase + sh->col_exp[BC ? 2 * jj : jj];
          double vr, vi;
          if (g.alpha_pow2) {
            vr = scaled_i64_to_double(neg ? -re : re, E);
            vi = scaled_i64_to_double(neg ? -im : im, E);
          } else {
            const double dr = scaled_i64_to_double(re, E), di = scaled_i64_to_double(im, E);
            vr = g.ar * dr - g.ai * di;
            vi = g.ar * di + g.ai * dr;
          }
          stage[lr * RS + k] = make_double2(vr, vi);
        }
        __syncwarp();
        // store the group: every lane owns a (row, column) pair per pass
        const long long cn = sh->col_off[(BC ? j0 / 2 : j0) + lc];
#pragma unroll 4
        for (int p = 0; p < NPASS; ++p) {
          const int r = p * RPP + lrw;
          const long long cm = __shfl_sync(0xffffffffu, coffm, (AC ? 2 * r : r) & 31);
          if (r >= nrows || cn < 0) continue;
          const long long off = cm + cn;
          const double2 v = stage[r * RS + lc];
          if (g.cc) {
            if (red) {
              atomicAdd(&Cc[off].x, v.x);
              atomicAdd(&Cc[off].y, v.y);
            } else {
              Cc[off] = v;
            }
          } else {
            if (red)
              atomicAdd(&Cr[off], v.x);
            else
              Cr[off] = v.x;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------------------
// Persistent 64-column form for S <= 4 slices (TcPersist).  One CTA per SM
// walks the output tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... (each
// at most one exact K chunk, as in the 128-column form).  Two TMEM buffers of
// S level accumulators: the MMA issuer fills buffer j & 1 for its j-th tile
// once the drain warps have released it (accempty), the drain warps empty it
// once its MMAs are complete (accfull) and release it as soon as the levels
// are in registers, before they convert and store -- so a tile's drain runs
// under the next tile's loads and MMAs.  A and B slices have rings of their
// own (A1 .. AS and B1 .. BS per K block, products row by row, each slice
// released after its last product).
// ---------------------------------------------------------------------------
struct PersistShared {
  uint64_t fullA[TcPersist::RA], emptyA[TcPersist::RA];
  uint64_t fullB[TcPersist::RB], emptyB[TcPersist::RB];
  uint64_t accfull[2], accempty[2], done;
  uint32_t tmem;
  volatile int abort;
  int stop;                                 // the drain warps' common decision for a tile
  long long col_off[TcPersist::BN / 1];     // output offset of each logical column (-1: outside)
  int col_exp[TcPersist::BN];
};

struct TileCoord {
  int mt, nt, zb, kb0, kb1, rowA0, rowB0;
};

__device__ __forceinline__ TileCoord persist_tile(const TcArgs& g, int t, int mtiles, int ntiles) {
  TileCoord c;
  const int per = mtiles * ntiles;
  const int zs = t / per, rem = t - zs * per;
  if (g.m_fast) {
    c.mt = rem % mtiles;
    c.nt = rem / mtiles;
  } else {
    c.nt = rem % ntiles;
    c.mt = rem / ntiles;
  }
  c.zb = zs / g.nsplit;
  c.kb0 = (zs - c.zb * g.nsplit) * g.kb_per_split;
  c.kb1 = min(g.kblocks, c.kb0 + g.kb_per_split);
  c.rowA0 = g.bat_a ? c.zb * g.rowsA_pad : 0;
  c.rowB0 = g.bat_b ? c.zb * g.rowsB_pad : 0;
  return c;
}

template <bool AC, bool BC>
__global__ void __launch_bounds__(TcPersist::THREADS, 1)
    ozaki_persist_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                         const TcArgs g, int ntiles_total) {
  using C = TcPersist;
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t* ringA = sm;                                   // RA x 16 KB
  uint8_t* ringB = ringA + C::RA * C::A_SLOT;            // RB x 8 KB
  uint8_t* stg = ringB + C::RB * C::B_SLOT;              // EPI x STAGE_WARP
  PersistShared* sh = (PersistShared*)(stg + C::EPI * C::STAGE_WARP);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = g.S;
  const int ncols = g.tmem_cols;
  const int mtiles = g.rowsA_pad / TC_BM, ntiles = g.rowsB_pad / C::BN;
  const uint32_t buf_cols = (uint32_t)(S * C::BN);  // one buffer of S levels

  if (threadIdx.x == 0) {
    for (int i = 0; i < C::RA; ++i) {
      mbar_init(smem_u32(&sh->fullA[i]), 1);
      mbar_init(smem_u32(&sh->emptyA[i]), 1);
    }
    for (int i = 0; i < C::RB; ++i) {
      mbar_init(smem_u32(&sh->fullB[i]), 1);
      mbar_init(smem_u32(&sh->emptyB[i]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&sh->accfull[b]), 1);
      mbar_init(smem_u32(&sh->accempty[b]), 32 * C::EPI);
    }
    mbar_init(smem_u32(&sh->done), 1);
    sh->abort = 0;
    sh->stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = sh->tmem;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int ja = 0, jb = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles_total && ok && !sh->abort; t += gridDim.x) {
        const TileCoord c = persist_tile(g, t, mtiles, ntiles);
        for (int kb = c.kb0; kb < c.kb1 && ok && !sh->abort; ++kb)
          for (int i = 0; i < 2 * S; ++i) {
            const bool isA = i == 0 || i > S;  // A1, B1 .. BS, A2 .. AS
            const int j = isA ? ja : jb, R = isA ? C::RA : C::RB;
            const int st = j % R;
            const uint32_t ph = (uint32_t)((j / R) & 1);
            const uint32_t eb = smem_u32(isA ? &sh->emptyA[st] : &sh->emptyB[st]);
            if (!mbar_wait(eb, ph ^ 1u, kWaitLimit)) {
              fail(sh, g.err, 1);
              ok = false;
              break;
            }
            const uint32_t fb = smem_u32(isA ? &sh->fullA[st] : &sh->fullB[st]);
            if (isA) {
              mbar_expect_tx(fb, C::A_SLOT);
              tma3d(smem_u32(ringA + st * C::A_SLOT), &tmA, kb * TC_BK, c.rowA0 + c.mt * TC_BM, i == 0 ? 0 : i - S,
                    fb);
              ++ja;
            } else {
              mbar_expect_tx(fb, C::B_SLOT);
              tma3d(smem_u32(ringB + st * C::B_SLOT), &tmB, kb * TC_BK, c.rowB0 + c.nt * C::BN, i - 1, fb);
              ++jb;
            }
          }
      }
      // every issued load lands before the CTA exits
      for (int q = (ja > C::RA ? ja - C::RA : 0); q < ja; ++q)
        mbar_wait(smem_u32(&sh->fullA[q % C::RA]), (uint32_t)((q / C::RA) & 1), kWaitLimit);
      for (int q = (jb > C::RB ? jb - C::RB : 0); q < jb; ++q)
        mbar_wait(smem_u32(&sh->fullB[q % C::RB]), (uint32_t)((q / C::RB) & 1), kWaitLimit);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t id = idesc_bf16(TC_BM, C::BN);
      int ja = 0, jb = 0, jt = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles_total && ok && !sh->abort; t += gridDim.x, ++jt) {
        const TileCoord c = persist_tile(g, t, mtiles, ntiles);
        const int b = jt & 1, use = jt >> 1;
        if (use > 0 && !mbar_wait(smem_u32(&sh->accempty[b]), (uint32_t)((use - 1) & 1), kWaitLimit)) {
          fail(sh, g.err, 2);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dbuf = tmem + (uint32_t)b * buf_cols;
        bool first = true;
        for (int kb = c.kb0; kb < c.kb1 && ok; ++kb, ja += S, jb += S) {
          for (int s = 1; s <= S && ok; ++s) {
            const int qa = ja + s - 1;  // A_s
            if (!mbar_wait(smem_u32(&sh->fullA[qa % C::RA]), (uint32_t)((qa / C::RA) & 1), kWaitLimit)) {
              ok = false;
              break;
            }
            const uint64_t da = sdesc(smem_u32(ringA + (qa % C::RA) * C::A_SLOT));
            for (int tt = 1; tt <= S + 1 - s; ++tt) {
              const int qb = jb + tt - 1;  // B_tt
              if (s == 1 &&
                  !mbar_wait(smem_u32(&sh->fullB[qb % C::RB]), (uint32_t)((qb / C::RB) & 1), kWaitLimit)) {
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;");
              const uint64_t db = sdesc(smem_u32(ringB + (qb % C::RB) * C::B_SLOT));
              const uint32_t dacc = dbuf + (uint32_t)((s + tt - 2) * C::BN);
#pragma unroll
              for (int k = 0; k < TC_BK / 16; ++k) {
                const uint32_t accf = (first && s == 1 && k == 0) ? 0u : 1u;
                umma(dacc, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), id, accf);
              }
            }
            if (!ok) break;
            // A_s and B_(S+1-s) have had their last use in this K block
            umma_commit(smem_u32(&sh->emptyA[qa % C::RA]));
            umma_commit(smem_u32(&sh->emptyB[(jb + S - s) % C::RB]));
          }
          first = false;
        }
        if (!ok) {
          fail(sh, g.err, 3);
          break;
        }
        umma_commit(smem_u32(&sh->accfull[b]));
      }
      umma_commit(smem_u32(&sh->done));
      mbar_wait(smem_u32(&sh->done), 0, kWaitLimit);
    }
  } else {
    // ---------------- drain warps (2 .. 17): 16 columns each ----------------
    const int q = warp & 3;
    const int j0 = ((warp - 2) >> 2) * 16;  // this warp's packed columns
    const int row = q * 32 + lane;
    const bool odd = AC && (lane & 1);
    constexpr int NJ = BC ? 8 : 16;        // logical columns of the group
    constexpr int rows_out = AC ? 16 : 32;  // logical rows of this warp
    constexpr int RS = NJ + 1;              // staging row stride, padded
    constexpr bool REAL_ONLY = !AC && !BC;  // real operands: stage the real part only
    double2* stage2 = reinterpret_cast<double2*>(stg + (size_t)(warp - 2) * C::STAGE_WARP);
    double* stage1 = reinterpret_cast<double*>(stg + (size_t)(warp - 2) * C::STAGE_WARP);
    const int lr = AC ? (lane >> 1) : lane;
    const uint32_t tl = (uint32_t)(q * 32) << 16;
    const int u = 7 * (S + 1);
    const bool neg = g.alpha_pow2 && g.alpha_neg;
    const bool red = g.acc || g.atomic;
    constexpr int RPP = 32 / NJ;
    constexpr int NPASS = rows_out / RPP;
    const int lc = lane % NJ, lrw = lane / NJ;
    int jt = 0;
    for (int t = blockIdx.x; t < ntiles_total; t += gridDim.x, ++jt) {
      const TileCoord c = persist_tile(g, t, mtiles, ntiles);
      const int b = jt & 1, use = jt >> 1;
      // one decision for all drain warps, and the tile's column data
      asm volatile("bar.sync 1, %0;" ::"n"(32 * C::EPI) : "memory");
      const int td = threadIdx.x - 64;
      if (td == 0) sh->stop = sh->abort;
      {
        constexpr int ncl = BC ? C::BN / 2 : C::BN;
        if (td < ncl) {
          const int n = c.nt * ncl + td;
          long long o = -1;
          if (n < g.N) decomp_tc(g.gnC, n, o);
          sh->col_off[td] = o;
        }
        if (td < C::BN) sh->col_exp[td] = row_exp(g.expB[c.rowB0 + c.nt * C::BN + td]);
      }
      asm volatile("bar.sync 1, %0;" ::"n"(32 * C::EPI) : "memory");
      if (sh->stop) break;  // the same value for every drain warp
      const bool got = mbar_wait(smem_u32(&sh->accfull[b]), (uint32_t)(use & 1), kWaitLimit);
      if (!__all_sync(0xffffffffu, got)) {
        fail(sh, g.err, 4);
        continue;  // the next tile's decision stops every drain warp
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      long long a16[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) a16[j] = 0;
#pragma unroll
      for (int L0 = 2; L0 <= 5; L0 += 2) {
        if (L0 > S + 1) break;
        uint32_t lv[2][16];
#pragma unroll
        for (int i = 0; i < 2; ++i)
          if (L0 + i <= S + 1)
            tmem_ld16_nowait(tmem + tl + (uint32_t)b * buf_cols + (uint32_t)((L0 + i - 2) * C::BN + j0), lv[i]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int L = L0 + i;
          if (L > S + 1) break;
          const int shl = u - 7 * L;
#pragma unroll
          for (int j = 0; j < 16; ++j) a16[j] += (long long)__float2int_rn(__uint_as_float(lv[i][j])) << shl;
        }
      }
      // the levels are in registers: the MMAs of a later tile may refill this buffer
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(smem_u32(&sh->accempty[b]));
      const int prow = c.mt * TC_BM + row;
      const int m = AC ? (prow >> 1) : prow;
      const int ea = prow < g.rowsA_pad ? row_exp(g.expA[c.rowA0 + prow]) : 0;
      const int ebase = ea - u + (g.alpha_pow2 ? g.alpha_e : 0);
      long long coffm = 0;
      if (m < g.M) decomp_tc(g.gmC, m, coffm);
      double2* Cc = static_cast<double2*>(g.C) + (g.cc ? c.zb * g.bsC : 0);
      double* Cr = static_cast<double*>(g.C) + (g.cc ? 0 : c.zb * g.bsC);
      const int m0w = AC ? ((c.mt * TC_BM + q * 32) >> 1) : (c.mt * TC_BM + q * 32);
      const int nrows = min(rows_out, g.M - m0w);
      __syncwarp();  // the previous tile's stores have read the staging area
#pragma unroll
      for (int k = 0; k < NJ; ++k) {
        const int jj = (BC ? j0 / 2 : j0) + k;
        long long re, im;
        if constexpr (BC) {
          const long long x0 = a16[2 * k], x1 = a16[2 * k + 1];
          if constexpr (AC) {
            const long long p0 = __shfl_xor_sync(0xffffffffu, x0, 1);
            const long long p1 = __shfl_xor_sync(0xffffffffu, x1, 1);
            const long long rr = odd ? p0 : x0, ri = odd ? p1 : x1, ir = odd ? x0 : p0, ii = odd ? x1 : p1;
            re = rr - ii;
            im = ri + ir;
          } else {
            re = x0;
            im = x1;
          }
        } else {
          const long long x = a16[k];
          if constexpr (AC) {
            const long long p = __shfl_xor_sync(0xffffffffu, x, 1);
            re = odd ? p : x;
            im = odd ? x : p;
          } else {
            re = x;
            im = 0;
          }
        }
        if (AC && ((k & 1) != (lane & 1))) continue;
        const int E = ebase + sh->col_exp[BC ? 2 * jj : jj];
        double vr, vi;
        if (g.alpha_pow2) {
          vr = scaled_i64_to_double(neg ? -re : re, E);
          vi = scaled_i64_to_double(neg ? -im : im, E);
        } else {
          const double dr = scaled_i64_to_double(re, E), di = scaled_i64_to_double(im, E);
          vr = g.ar * dr - g.ai * di;
          vi = g.ar * di + g.ai * dr;
        }
        if constexpr (REAL_ONLY)
          stage1[lr * RS + k] = vr;
        else
          stage2[lr * RS + k] = make_double2(vr, vi);
      }
      __syncwarp();
      const long long cn = sh->col_off[(BC ? j0 / 2 : j0) + lc];
#pragma unroll 4
      for (int p = 0; p < NPASS; ++p) {
        const int r = p * RPP + lrw;
        const long long cm = __shfl_sync(0xffffffffu, coffm, (AC ? 2 * r : r) & 31);
        if (r >= nrows || cn < 0) continue;
        const long long off = cm + cn;
        const double2 v = REAL_ONLY ? make_double2(stage1[r * RS + lc], 0.0) : stage2[r * RS + lc];
        if (g.cc) {
          if (red) {
            atomicAdd(&Cc[off].x, v.x);
            if (!REAL_ONLY) atomicAdd(&Cc[off].y, v.y);
          } else {
            Cc[off] = v;
          }
        } else {
          if (red)
            atomicAdd(&Cr[off], v.x);
          else
            Cr[off] = v.x;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------------------
// Short contractions (K <= 64) of the mixed mode on the FP32 pipe: the same
// exact slice products as the tensor-core path, without packing.  One output
// tile per block: the block takes the binary exponents of its rows of A and
// columns of B over all of K (real and imaginary parts share one), cuts K
// chunks of both into S signed 7-bit digits in shared memory, and every
// thread accumulates the levels L = s + t of its 4 outputs with FP32 FMAs.  A complex level sum grows by at most
// 2 (2^14 + 2^13 + 2^13) = 2^16 per K index, so up to K = 64 every partial
// sum is an integer below 2^22, exact in FP32.  The epilogue recombines the
// levels in int64 and converts with the exponents, as the tensor-core drain
// does.  GB300's FP64 pipe runs about 2 FMA per clock per SM, its FP32 pipe
// 128: 60 FP32 FMAs per complex multiply-add still finish 4x sooner than 4
// FP64 ones, and the FP64 pipe stays free for the elementwise ops.
// ---------------------------------------------------------------------------
constexpr int kSimtMaxK = 64;

// Tile BM x BN (32 x 32, 16 x 64 or 64 x 16), 256 threads on a 16 x 16 grid,
// 4 outputs each: rows ty + 16 i, columns tx + 16 j.  Digits in shared memory
// per K index and row: S x (2 if complex) floats, contiguous, read as float2.
template <bool AC, bool BC, bool CC, int S, int BM, int BN>
__global__ void __launch_bounds__(256, 2) simt_slices_kernel(const GemmArgs g, int alpha_pow2, int alpha_e,
                                                             int alpha_neg) {
  constexpr int PA = AC ? 2 : 1, PB = BC ? 2 : 1;
  constexpr int SPA = (S * PA + 1) / 2 * 2, SPB = (S * PB + 1) / 2 * 2;  // floats per row, even
  // shared row strides: B's columns are read by the 16 tx values of a half
  // warp at once, so their stride is twice an odd number of floats (the 16
  // float2 reads fall in distinct bank pairs); A's rows by two ty values only
  constexpr int STA = SPA, STB = (SPB / 2) % 2 == 1 ? SPB : SPB + 2;
  constexpr int MI = BM / 16, NJ = BN / 16;
  static_assert(MI * NJ == 4, "four outputs per thread");
  constexpr int KC = (BM > 32 || BN > 32) ? 8 : 16;  // K chunk (static shared memory <= 48 KB)
  __shared__ __align__(8) float sa[KC][BM][STA];
  __shared__ __align__(8) float sb[KC][BN][STB];
  __shared__ long long aoff[BM], boff[BN], coffm[BM], coffn[BN];
  __shared__ long long kofa[kSimtMaxK], kofb[kSimtMaxK];
  __shared__ int ea[BM], eb[BN];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN, zb = blockIdx.z;
  const double* A = static_cast<const double*>(g.A) + (size_t)zb * g.bsA * PA;
  const double* B = static_cast<const double*>(g.B) + (size_t)zb * g.bsB * PB;
  auto dec = [](const ModeGroup& gr, int l, long long& o0, long long& o1) {
    o0 = 0;
    o1 = 0;
    for (int q = kMaxModes - 1; q >= 0; --q)
      if (q < gr.n) {
        const int r = l % gr.dim[q];
        l /= gr.dim[q];
        o0 += (long long)r * gr.s0[q];
        o1 += (long long)r * gr.s1[q];
      }
  };
  if (tid < BM) {
    long long o0 = -1, o1 = -1;
    if (m0 + tid < g.M) dec(g.gm, m0 + tid, o0, o1);
    aoff[tid] = o0;
    coffm[tid] = o1;
  } else if (tid < BM + BN) {
    const int c = tid - BM;
    long long o0 = -1, o1 = -1;
    if (n0 + c < g.N) dec(g.gn, n0 + c, o0, o1);
    boff[c] = o0;
    coffn[c] = o1;
  } else if (tid < BM + BN + g.K) {
    const int k = tid - BM - BN;
    dec(g.gk, k, kofa[k], kofb[k]);
  }
  __syncthreads();
  // exponents of the tile's rows of A and columns of B over all of K: every
  // thread takes elements (row, k) with independent loads, the maxima of the
  // bit patterns (the order of |x| for finite doubles) meet in shared memory
  constexpr unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull;
  __shared__ unsigned long long rmax[BM + BN];
  if (tid < BM + BN) rmax[tid] = 0ull;
  __syncthreads();
  for (int idx = tid; idx < (BM + BN) * g.K; idx += blockDim.x) {
    const int r = idx % (BM + BN), k = idx / (BM + BN);
    const bool isA = r < BM;
    const long long base = isA ? aoff[r] : boff[r - BM];
    if (base < 0) continue;
    const unsigned long long* bits =
        reinterpret_cast<const unsigned long long*>(isA ? static_cast<const void*>(A) : static_cast<const void*>(B));
    const int per = isA ? PA : PB;
    const long long el = base + (isA ? kofa[k] : kofb[k]);
    unsigned long long v = bits[per * el] & kAbs;
    if (per == 2) v = max(v, bits[2 * el + 1] & kAbs);
    if (v) atomicMax(&rmax[r], v);
  }
  __syncthreads();
  if (tid < BM + BN) {
    const unsigned long long mx = rmax[tid];
    const int E = (int)(mx >> 52);
    const int e = mx != 0 ? (E > 0 ? E - 1022 : -1022) : 0;
    if (tid < BM)
      ea[tid] = e;
    else
      eb[tid - BM] = e;
  }
  __syncthreads();
  const int tx = tid % 16, ty = tid / 16;
  float acc[MI][NJ][S][2];
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j)
#pragma unroll
      for (int L = 0; L < S; ++L) acc[i][j][L][0] = acc[i][j][L][1] = 0.f;
  constexpr int nbits = 7 * S;
  for (int kc = 0; kc < g.K; kc += KC) {
    // digits of the chunk: BM rows x KC of A, KC x BN columns of B
    for (int idx = tid; idx < (BM + BN) * KC; idx += blockDim.x) {
      const bool isA = idx < BM * KC;
      const int id2 = isA ? idx : idx - BM * KC;
      const int nr = isA ? BM : BN;
      const int r = id2 % nr, kk = id2 / nr, k = kc + kk;
      const long long base = isA ? aoff[r] : boff[r];
      const int per = isA ? PA : PB;
      double x[2] = {0.0, 0.0};
      if (base >= 0 && k < g.K) {
        const double* src = isA ? A : B;
        const long long el = base + (isA ? kofa[k] : kofb[k]);
        x[0] = src[per * el];
        if (per == 2) x[1] = src[2 * el + 1];
      }
      const int e = isA ? ea[r] : eb[r];
      float* dst = isA ? &sa[kk][r][0] : &sb[kk][r][0];
      for (int part = 0; part < per; ++part) {
        const unsigned long long f = fixed_point(x[part], e, nbits);
        const bool neg = __double_as_longlong(x[part]) < 0;  // sign bit: no FP64 compare
        int qd[S];
        balanced_digits(f, S, qd);
#pragma unroll
        for (int s = 0; s < S; ++s) dst[s * per + part] = small_int_to_float(neg ? -qd[s] : qd[s]);
      }
    }
    __syncthreads();
    const int kn = min(KC, g.K - kc);
    for (int kk = 0; kk < kn; ++kk) {
      float a[MI][SPA], b[NJ][SPB];
#pragma unroll
      for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int q = 0; q < SPA / 2; ++q) {
          const float2 v = *reinterpret_cast<const float2*>(&sa[kk][ty + 16 * i][2 * q]);
          a[i][2 * q] = v.x;
          a[i][2 * q + 1] = v.y;
        }
#pragma unroll
      for (int j = 0; j < NJ; ++j)
#pragma unroll
        for (int q = 0; q < SPB / 2; ++q) {
          const float2 v = *reinterpret_cast<const float2*>(&sb[kk][tx + 16 * j][2 * q]);
          b[j][2 * q] = v.x;
          b[j][2 * q + 1] = v.y;
        }
#pragma unroll
      for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
          for (int s = 0; s < S; ++s)
#pragma unroll
            for (int t = 0; t < S - s; ++t) {  // level s + t (0-based), s + t <= S - 1
              float& re = acc[i][j][s + t][0];
              float& im = acc[i][j][s + t][1];
              if constexpr (AC && BC) {
                re = fmaf(a[i][2 * s], b[j][2 * t], re);
                re = fmaf(-a[i][2 * s + 1], b[j][2 * t + 1], re);
                im = fmaf(a[i][2 * s], b[j][2 * t + 1], im);
                im = fmaf(a[i][2 * s + 1], b[j][2 * t], im);
              } else if constexpr (AC) {
                re = fmaf(a[i][2 * s], b[j][t], re);
                im = fmaf(a[i][2 * s + 1], b[j][t], im);
              } else if constexpr (BC) {
                re = fmaf(a[i][s], b[j][2 * t], re);
                im = fmaf(a[i][s], b[j][2 * t + 1], im);
              } else {
                re = fmaf(a[i][s], b[j][t], re);
              }
            }
    }
    __syncthreads();
  }
  // recombine the levels in int64 (0-based level l weighs 2^(-7(l + 2))) and store
  const int u = 7 * ((S < 5 ? S : 5) + 1);
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int r = ty + 16 * i, c = tx + 16 * j;
      if (m0 + r >= g.M || n0 + c >= g.N) continue;
      long long X[2] = {0, 0};
#pragma unroll
      for (int L = 0; L < S; ++L) {
        const int sh = u - 7 * (L + 2);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const long long v = (long long)__float2int_rn(acc[i][j][L][p]);
          X[p] += sh >= 0 ? (v << sh) : (v >> (-sh));
        }
      }
      const int E = ea[r] + eb[c] - u + (alpha_pow2 ? alpha_e : 0);
      double vr, vi;
      if (alpha_pow2) {
        vr = scaled_i64_to_double(alpha_neg ? -X[0] : X[0], E);
        vi = scaled_i64_to_double(alpha_neg ? -X[1] : X[1], E);
      } else {
        const double dr = scaled_i64_to_double(X[0], E), di = scaled_i64_to_double(X[1], E);
        vr = g.ar * dr - g.ai * di;
        vi = g.ar * di + g.ai * dr;
      }
      const long long off = coffm[r] + coffn[c];
      // accumulation as an L2 reduction (one writer per element)
      if constexpr (CC) {
        double2* C = static_cast<double2*>(g.C) + (size_t)zb * g.bsC;
        if (g.acc) {
          atomicAdd(&C[off].x, vr);
          atomicAdd(&C[off].y, vi);
        } else {
          C[off] = make_double2(vr, vi);
        }
      } else {
        double* C = static_cast<double*>(g.C) + (size_t)zb * g.bsC;
        if (g.acc)
          atomicAdd(&C[off], vr);
        else
          C[off] = vr;
      }
    }
}

template <bool AC, bool BC, bool CC, int S>
static void launch_simt_tile(int tile, const GemmArgs& g, int nb, int p2, int e2, int n2, cudaStream_t st) {
  const int bm = tile == 1 ? 16 : tile == 2 ? 64 : 32, bn = tile == 1 ? 64 : tile == 2 ? 16 : 32;
  dim3 grid((unsigned)((g.N + bn - 1) / bn), (unsigned)((g.M + bm - 1) / bm), (unsigned)nb);
  if (tile == 1)
    simt_slices_kernel<AC, BC, CC, S, 16, 64><<<grid, 256, 0, st>>>(g, p2, e2, n2);
  else if (tile == 2)
    simt_slices_kernel<AC, BC, CC, S, 64, 16><<<grid, 256, 0, st>>>(g, p2, e2, n2);
  else
    simt_slices_kernel<AC, BC, CC, S, 32, 32><<<grid, 256, 0, st>>>(g, p2, e2, n2);
}

template <bool AC, bool BC, bool CC>
static void launch_simt_typed(int tile, const GemmArgs& g, int nb, int S, int p2, int e2, int n2, cudaStream_t st) {
  if (S == 6)
    launch_simt_tile<AC, BC, CC, 6>(tile, g, nb, p2, e2, n2, st);
  else if (S == 5)
    launch_simt_tile<AC, BC, CC, 5>(tile, g, nb, p2, e2, n2, st);
  else
    launch_simt_tile<AC, BC, CC, 4>(tile, g, nb, p2, e2, n2, st);
}

bool simt_slices_supported(int K, int S) { return K >= 1 && K <= kSimtMaxK && S >= 4 && S <= 6; }

cudaError_t launch_simt_slices(const Op& op, const void* A, const void* B, void* C, cudaStream_t st) {
  GemmArgs g = op.g;
  g.A = A;
  g.B = B;
  g.C = C;
  const TcArgs& t = op.tc;
  if (!simt_slices_supported(g.K, t.S) || g.atomic) return cudaErrorInvalidValue;
  const int nb = g.nb < 1 ? 1 : g.nb;
  // the tile with the least padding: 32 x 32, 16 x 64, 64 x 16
  const long long M = g.M, N = g.N;
  const long long pad[3] = {((M + 31) / 32 * 32) * ((N + 31) / 32 * 32), ((M + 15) / 16 * 16) * ((N + 63) / 64 * 64),
                            ((M + 63) / 64 * 64) * ((N + 15) / 16 * 16)};
  int tile = 0;
  for (int q = 1; q < 3; ++q)
    if (pad[q] < pad[tile]) tile = q;
  const int bm = tile == 1 ? 16 : tile == 2 ? 64 : 32;
  if ((M + bm - 1) / bm > 65535 || nb > 65535) return cudaErrorInvalidConfiguration;
  const bool ac = op.dta == C64, bc = op.dtb == C64, cc = op.dtc == C64;
  if (!cc && (ac || bc)) return cudaErrorInvalidValue;
  if (ac && bc)
    launch_simt_typed<true, true, true>(tile, g, nb, t.S, t.alpha_pow2, t.alpha_e, t.alpha_neg, st);
  else if (ac)
    launch_simt_typed<true, false, true>(tile, g, nb, t.S, t.alpha_pow2, t.alpha_e, t.alpha_neg, st);
  else if (bc)
    launch_simt_typed<false, true, true>(tile, g, nb, t.S, t.alpha_pow2, t.alpha_e, t.alpha_neg, st);
  else if (cc)
    launch_simt_typed<false, false, true>(tile, g, nb, t.S, t.alpha_pow2, t.alpha_e, t.alpha_neg, st);
  else
    launch_simt_typed<false, false, false>(tile, g, nb, t.S, t.alpha_pow2, t.alpha_e, t.alpha_neg, st);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
bool tc_available() { return true; }

// the driver's tensor-map encoder, looked up once (thread-safe static init)
static PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        !p)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled unavailable");
  return fn;
}

// [S][rows_pad][K_pad] BF16, box = (64 K, box_rows rows, 1 slice).
// Encoded maps are cached by (address, layout): a packed buffer keeps its
// address for the life of its program.
static CUtensorMap slice_map(const void* base, int S, int rows_pad, int K_pad, int box_rows) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, int, int, int>, CUtensorMap> cache;
  const auto key = std::make_tuple(base, S, rows_pad, K_pad, box_rows);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)K_pad, (cuuint64_t)rows_pad, (cuuint64_t)S};
  cuuint64_t strides[2] = {(cuuint64_t)K_pad * 2, (cuuint64_t)K_pad * 2 * rows_pad};
  cuuint32_t box[3] = {TC_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                               es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = m;
  return m;
}

cudaError_t launch_pack(const PackArgs& p, cudaStream_t st) {
  if (p.nb < 1 || p.rows < 1 || p.rows_pad % (p.cplx ? 2 : 1) != 0 || p.rows * (p.cplx ? 2 : 1) > p.rows_pad ||
      p.K_pad % 2 != 0 || p.K > p.K_pad)
    return cudaErrorInvalidValue;
  const long long blocks = (long long)p.nb * p.rows;
  if (blocks > 0x7FFFFFFFLL) return cudaErrorInvalidConfiguration;
  if (p.K_pad <= 2048) {
    // rows held in registers, read once: up to 256 elements per warp (8 per
    // lane), up to eight warps per row
    auto go = [&](auto kern, int rows_per_block) {
      kern<<<(unsigned)((blocks + rows_per_block - 1) / rows_per_block), 256, 0, st>>>(p);
    };
    if (p.K_pad <= 64)
      go(pack_rows_regs_kernel<1, 1>, 8);
    else if (p.K_pad <= 128)
      go(pack_rows_regs_kernel<2, 1>, 8);
    else if (p.K_pad <= 256)
      go(pack_rows_regs_kernel<4, 1>, 8);
    else if (p.K_pad <= 512)
      go(pack_rows_regs_kernel<4, 2>, 4);
    else if (p.K_pad <= 1024)
      go(pack_rows_regs_kernel<4, 4>, 2);
    else
      go(pack_rows_regs_kernel<4, 8>, 1);
  } else {
    // long rows: a block per row; few long rows (the K = o v^2 operands)
    // take more threads per row so that the SMs still fill
    const int threads = (p.K_pad >= 4096 && blocks < 4 * 152) ? 1024 : 256;
    // the K offsets as a shared-memory table when they fit (64 KB, 32 bits)
    constexpr int kTabMax = 16384;
    constexpr int kMaxDev = 64;
    static std::once_flag once[kMaxDev];
    static cudaError_t attr_err[kMaxDev] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    std::call_once(once[dev], [dev] {
      attr_err[dev] = cudaFuncSetAttribute(pack_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kTabMax * (int)sizeof(int));
    });
    long long span = 0;  // largest K offset
    for (int q = 0; q < p.gk.n && q < kMaxModes; ++q) span += (long long)(p.gk.dim[q] - 1) * std::llabs(p.gk.s0[q]);
    const int tab = (attr_err[dev] == cudaSuccess && p.K <= kTabMax && span < (1LL << 31)) ? 1 : 0;
    const size_t smem = tab ? (size_t)p.K * sizeof(int) : 0;
    pack_kernel<<<(unsigned)blocks, threads, smem, st>>>(p, tab);
  }
  count_launch();
  return cudaGetLastError();
}

template <class C>
static cudaError_t launch_variant(const TcArgs& a0, const void* packA, const void* packB, cudaStream_t st) {
  // kernel attributes act on the current device's context: set them once
  // per device (engines on several host threads may launch their first
  // slice products together)
  constexpr int kMaxDev = 64;
  static std::once_flag once[kMaxDev];
  static cudaError_t attr_err[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  std::call_once(once[dev], [dev] {
    cudaError_t e = cudaFuncSetAttribute(ozaki_kernel<true, true, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<true, false, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<false, true, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<false, false, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    // all of L1 as shared memory, so that MINB CTAs fit on an SM
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<true, true, C>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<true, false, C>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<false, true, C>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(ozaki_kernel<false, false, C>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    attr_err[dev] = e;
  });
  if (attr_err[dev] != cudaSuccess) return attr_err[dev];
  TcArgs a = a0;
  if (a.S > C::STAGES) return cudaErrorInvalidValue;  // the ring holds one K block's slices
  int cols = 32;
  while (cols < (a.S + 2) * C::BN) cols *= 2;  // level accumulators + int64 partial sums
  if (cols > 512 / C::MINB) return cudaErrorInvalidValue;
  a.tmem_cols = cols;
  if (a.rowsB_pad % C::BN != 0) return cudaErrorInvalidValue;
  const CUtensorMap ma = slice_map(packA, a.S, (a.bat_a ? a.nb : 1) * a.rowsA_pad, a.kblocks * TC_BK, TC_BM);
  const CUtensorMap mb = slice_map(packB, a.S, (a.bat_b ? a.nb : 1) * a.rowsB_pad, a.kblocks * TC_BK, C::BN);
  // CTA order: the tiles of the smaller operand side vary fastest, so that
  // side stays in L2 while each tile of the larger side is read from DRAM
  // once (the N-fastest order re-read the 69 MB of packed amplitudes of the
  // 24-trajectory ladder for each of its 12 M strips: 430 MB per launch)
  const unsigned mtiles = (unsigned)(a.rowsA_pad / TC_BM), ntiles = (unsigned)(a.rowsB_pad / C::BN);
  a.m_fast = (a.rowsA_pad < a.rowsB_pad && ntiles <= 65535u) ? 1 : 0;
  dim3 grid(a.m_fast ? mtiles : ntiles, a.m_fast ? ntiles : mtiles, (unsigned)((long long)a.nb * a.nsplit));
  if (a.ac && a.bc)
    ozaki_kernel<true, true, C><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else if (a.ac)
    ozaki_kernel<true, false, C><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else if (a.bc)
    ozaki_kernel<false, true, C><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else
    ozaki_kernel<false, false, C><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  count_launch();
  return cudaGetLastError();
}

static cudaError_t launch_tile128(const TcArgs& a0, const void* packA, const void* packB, cudaStream_t st) {
  using C = TcTile128;
  constexpr int kMaxDev = 64;
  static std::once_flag once[kMaxDev];
  static cudaError_t attr_err[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  std::call_once(once[dev], [dev] {
    cudaError_t e = cudaSuccess;
    for (auto fn : {ozaki_tile128_kernel<true, true>, ozaki_tile128_kernel<true, false>,
                    ozaki_tile128_kernel<false, true>, ozaki_tile128_kernel<false, false>}) {
      if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    }
    attr_err[dev] = e;
  });
  if (attr_err[dev] != cudaSuccess) return attr_err[dev];
  TcArgs a = a0;
  // one exact K chunk per CTA, S level accumulators of 128 columns
  if (a.S < 1 || a.S > TC_TILE128_MAX_S || 2 * a.S > C::STAGES || a.kb_per_split > tc_chunk_kblocks(a.S))
    return cudaErrorInvalidValue;
  int cols = 32;
  while (cols < a.S * C::BN) cols *= 2;
  a.tmem_cols = cols;
  if (a.rowsB_pad % C::BN != 0 || a.rowsA_pad % TC_BM != 0) return cudaErrorInvalidValue;
  const CUtensorMap ma = slice_map(packA, a.S, (a.bat_a ? a.nb : 1) * a.rowsA_pad, a.kblocks * TC_BK, TC_BM);
  const CUtensorMap mb = slice_map(packB, a.S, (a.bat_b ? a.nb : 1) * a.rowsB_pad, a.kblocks * TC_BK, C::BN);
  const unsigned mtiles = (unsigned)(a.rowsA_pad / TC_BM), ntiles = (unsigned)(a.rowsB_pad / C::BN);
  a.m_fast = (a.rowsA_pad < a.rowsB_pad && ntiles <= 65535u) ? 1 : 0;
  if ((a.m_fast ? ntiles : mtiles) > 65535u || (long long)a.nb * a.nsplit > 65535LL) return cudaErrorInvalidConfiguration;
  dim3 grid(a.m_fast ? mtiles : ntiles, a.m_fast ? ntiles : mtiles, (unsigned)((long long)a.nb * a.nsplit));
  if (a.ac && a.bc)
    ozaki_tile128_kernel<true, true><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else if (a.ac)
    ozaki_tile128_kernel<true, false><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else if (a.bc)
    ozaki_tile128_kernel<false, true><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  else
    ozaki_tile128_kernel<false, false><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a);
  count_launch();
  return cudaGetLastError();
}

static cudaError_t launch_persist(const TcArgs& a0, const void* packA, const void* packB, cudaStream_t st) {
  using C = TcPersist;
  constexpr int kMaxDev = 64;
  static std::once_flag once[kMaxDev];
  static cudaError_t attr_err[kMaxDev] = {};
  static int sm_count[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  std::call_once(once[dev], [dev] {
    cudaError_t e = cudaDeviceGetAttribute(&sm_count[dev], cudaDevAttrMultiProcessorCount, dev);
    for (auto fn : {ozaki_persist_kernel<true, true>, ozaki_persist_kernel<true, false>,
                    ozaki_persist_kernel<false, true>, ozaki_persist_kernel<false, false>}) {
      if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    }
    attr_err[dev] = e;
  });
  if (attr_err[dev] != cudaSuccess) return attr_err[dev];
  TcArgs a = a0;
  // two TMEM buffers of S levels, one exact K chunk per tile
  if (a.S < 1 || a.S > TC_TILE128_MAX_S || a.kb_per_split > tc_chunk_kblocks(a.S)) return cudaErrorInvalidValue;
  int cols = 32;
  while (cols < 2 * a.S * C::BN) cols *= 2;
  a.tmem_cols = cols;
  if (a.rowsB_pad % C::BN != 0 || a.rowsA_pad % TC_BM != 0) return cudaErrorInvalidValue;
  const CUtensorMap ma = slice_map(packA, a.S, (a.bat_a ? a.nb : 1) * a.rowsA_pad, a.kblocks * TC_BK, TC_BM);
  const CUtensorMap mb = slice_map(packB, a.S, (a.bat_b ? a.nb : 1) * a.rowsB_pad, a.kblocks * TC_BK, C::BN);
  const long long mtiles = a.rowsA_pad / TC_BM, ntiles = a.rowsB_pad / C::BN;
  a.m_fast = a.rowsA_pad < a.rowsB_pad ? 1 : 0;
  const long long total = mtiles * ntiles * a.nb * a.nsplit;
  if (total > 0x7FFFFFFFLL) return cudaErrorInvalidConfiguration;
  const unsigned grid = (unsigned)std::min<long long>(total, std::max(sm_count[dev], 1));
  if (a.ac && a.bc)
    ozaki_persist_kernel<true, true><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a, (int)total);
  else if (a.ac)
    ozaki_persist_kernel<true, false><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a, (int)total);
  else if (a.bc)
    ozaki_persist_kernel<false, true><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a, (int)total);
  else
    ozaki_persist_kernel<false, false><<<grid, C::THREADS, C::SMEM, st>>>(ma, mb, a, (int)total);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ozaki(const TcArgs& a, const void* packA, const void* packB, cudaStream_t st) {
  if (a.nb < 1 || a.nsplit < 1 || (long long)a.nsplit * a.kb_per_split < a.kblocks) return cudaErrorInvalidValue;
  if (a.variant == 3) return launch_persist(a, packA, packB, st);
  if (a.variant == 2) return launch_tile128(a, packA, packB, st);
  return a.variant == 1 ? launch_variant<TcNarrow>(a, packA, packB, st) : launch_variant<TcWide>(a, packA, packB, st);
}

}  // namespace tdcc
