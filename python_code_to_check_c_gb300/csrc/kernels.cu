// FP64 kernels of the plain form: strided tensor contraction (GEMM over
// flattened mode groups), elementwise accumulate with antisymmetrisers, and
// the dipole trace.  All complex data is interleaved (double2).
#include <atomic>
#include <cstdio>
#include <type_traits>

#include "engine.h"

namespace tdcc {

static std::atomic<long long> g_launches{0};
void count_launch(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(); }

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
template <bool CPLX>
struct Elem;
template <>
struct Elem<true> {
  using T = double2;
};
template <>
struct Elem<false> {
  using T = double;
};

__device__ __forceinline__ double2 cz() { return make_double2(0.0, 0.0); }

__device__ __forceinline__ double2 as2(double x) { return make_double2(x, 0.0); }
__device__ __forceinline__ double2 as2(double2 x) { return x; }

// acc += a * b for the four real/complex combinations
__device__ __forceinline__ void mac(double2& c, double a, double b) { c.x = fma(a, b, c.x); }
__device__ __forceinline__ void mac(double2& c, double a, double2 b) {
  c.x = fma(a, b.x, c.x);
  c.y = fma(a, b.y, c.y);
}
__device__ __forceinline__ void mac(double2& c, double2 a, double b) {
  c.x = fma(a.x, b, c.x);
  c.y = fma(a.y, b, c.y);
}
__device__ __forceinline__ void mac(double2& c, double2 a, double2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}

__device__ __forceinline__ void decomp(const ModeGroup& g, int l, long long& o0, long long& o1) {
  o0 = 0;
  o1 = 0;
#pragma unroll
  for (int q = kMaxModes - 1; q >= 0; --q) {
    if (q < g.n) {
      const int d = g.dim[q];
      const int r = l % d;
      l /= d;
      o0 += (long long)r * g.s0[q];
      o1 += (long long)r * g.s1[q];
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 contraction: C[m,n] (+)= alpha * sum_k A[m,k] B[k,n]
// BM x BN output tile, K step 16, 256 threads, TM x TN outputs per thread
// (strided by BM/TM and BN/TN so shared-memory reads are conflict free).  On
// GB300 the FP64 pipe (~1.2 TFLOP/s) is the bound, so the tile shape is
// chosen per contraction to minimise padded (wasted) multiply-adds.
// ---------------------------------------------------------------------------
constexpr int GBK = 16;

template <bool AC, bool BC, bool CC, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(256) gemm_f64_kernel(const GemmArgs g) {
  static_assert((BM / TM) * (BN / TN) == 256, "256 threads");
  static_assert(256 % BM == 0 && 256 % BN == 0, "tile rows divide the CTA");
  using TA = typename Elem<AC>::T;
  using TB = typename Elem<BC>::T;
  constexpr int RX = BN / TN, RY = BM / TM;  // thread grid
  constexpr int LA = BM * GBK / 256, LB = BN * GBK / 256;
  __shared__ TA As[GBK][BM];
  __shared__ TB Bs[GBK][BN];

  const int tid = threadIdx.x;
  const int tx = tid % RX, ty = tid / RX;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int zb = blockIdx.z / g.nsplit;          // batch
  const int ks = blockIdx.z - zb * g.nsplit;     // K split
  const int kbeg = ks * g.kchunk;
  const int kend = min(g.K, kbeg + g.kchunk);

  const TA* A = static_cast<const TA*>(g.A) + zb * g.bsA;
  const TB* B = static_cast<const TB*>(g.B) + zb * g.bsB;

  // this thread's load row (A) / column (B) and their base offsets
  const int ar = tid % BM, ak0 = tid / BM;
  const int br = tid % BN, bk0 = tid / BN;
  const int am = m0 + ar, bn = n0 + br;
  long long aoff = 0, boff = 0, dummy;
  if (am < g.M) decomp(g.gm, am, aoff, dummy);
  if (bn < g.N) decomp(g.gn, bn, boff, dummy);

  double2 acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = cz();

  for (int k0 = kbeg; k0 < kend; k0 += GBK) {
#pragma unroll
    for (int r = 0; r < LA; ++r) {
      const int kk = ak0 + (256 / BM) * r;
      const int k = k0 + kk;
      TA av{};
      if (k < kend && am < g.M) {
        long long ka, kb;
        decomp(g.gk, k, ka, kb);
        av = A[aoff + ka];
      }
      As[kk][ar] = av;
    }
#pragma unroll
    for (int r = 0; r < LB; ++r) {
      const int kk = bk0 + (256 / BN) * r;
      const int k = k0 + kk;
      TB bv{};
      if (k < kend && bn < g.N) {
        long long ka, kb;
        decomp(g.gk, k, ka, kb);
        bv = B[boff + kb];
      }
      Bs[kk][br] = bv;
    }
    __syncthreads();
    // the last K step of a short K range stops at its end (K = o = 10 would
    // otherwise spend 6 of 16 multiply-adds on zero padding)
    const int kmax = min(GBK, kend - k0);
#pragma unroll 4
    for (int kk = 0; kk < kmax; ++kk) {
      TA a[TM];
      TB b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + RY * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + RX * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) mac(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }

  long long coffm[TM], coffn[TN];
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty + RY * i;
    coffm[i] = 0;
    if (m < g.M) decomp(g.gm, m, dummy, coffm[i]);
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int n = n0 + tx + RX * j;
    coffn[j] = 0;
    if (n < g.N) decomp(g.gn, n, dummy, coffn[j]);
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty + RY * i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = n0 + tx + RX * j;
      if (n >= g.N) continue;
      const double2 s = acc[i][j];
      const long long off = coffm[i] + coffn[j];
      if constexpr (CC) {
        double2* C = static_cast<double2*>(g.C) + zb * g.bsC;
        const double2 v = make_double2(g.ar * s.x - g.ai * s.y, g.ar * s.y + g.ai * s.x);
        if (g.atomic || g.acc) {  // L2 reductions (one writer per element unless split)
          atomicAdd(&C[off].x, v.x);
          atomicAdd(&C[off].y, v.y);
        } else {
          C[off] = v;
        }
      } else {
        double* C = static_cast<double*>(g.C) + zb * g.bsC;
        const double v = g.ar * s.x;
        if (g.atomic || g.acc)
          atomicAdd(&C[off], v);
        else
          C[off] = v;
      }
    }
  }
}

// tile shapes: {BM, BN}
const int kTiles[kNumTiles][2] = {{64, 64}, {32, 64}, {64, 32}, {32, 32}, {16, 16}, {16, 128}, {128, 16}};

bool tile_fits(int t, long long M) { return (M + kTiles[t][0] - 1) / kTiles[t][0] <= 65535; }  // grid.y

int choose_tile(long long M, long long N) {
  int best = 0;
  double bc = 1e300;
  for (int t = 0; t < kNumTiles; ++t) {
    if (!tile_fits(t, M)) continue;
    const long long bm = kTiles[t][0], bn = kTiles[t][1];
    // padded multiply-adds, with a small penalty for less operand reuse
    const double pen = (bm * bn >= 4096) ? 1.0 : (bm * bn >= 1024) ? 1.06 : 1.15;
    const double cost = (double)((M + bm - 1) / bm * bm) * (double)((N + bn - 1) / bn * bn) * pen;
    if (cost < bc) {
      bc = cost;
      best = t;
    }
  }
  return best;
}

template <bool AC, bool BC, bool CC>
static void launch_typed(int tile, dim3 grid, const GemmArgs& g, cudaStream_t st) {
  switch (tile) {
    case 0: gemm_f64_kernel<AC, BC, CC, 64, 64, 4, 4><<<grid, 256, 0, st>>>(g); break;
    case 1: gemm_f64_kernel<AC, BC, CC, 32, 64, 2, 4><<<grid, 256, 0, st>>>(g); break;
    case 2: gemm_f64_kernel<AC, BC, CC, 64, 32, 4, 2><<<grid, 256, 0, st>>>(g); break;
    case 3: gemm_f64_kernel<AC, BC, CC, 32, 32, 2, 2><<<grid, 256, 0, st>>>(g); break;
    case 5: gemm_f64_kernel<AC, BC, CC, 16, 128, 1, 8><<<grid, 256, 0, st>>>(g); break;
    case 6: gemm_f64_kernel<AC, BC, CC, 128, 16, 8, 1><<<grid, 256, 0, st>>>(g); break;
    default: gemm_f64_kernel<AC, BC, CC, 16, 16, 1, 1><<<grid, 256, 0, st>>>(g); break;
  }
}

cudaError_t launch_gemm(const Op& op, const void* A, const void* B, void* C, cudaStream_t st) {
  GemmArgs g = op.g;
  g.A = A;
  g.B = B;
  g.C = C;
  const int bm = kTiles[op.tile][0], bn = kTiles[op.tile][1];
  const int gx = (g.N + bn - 1) / bn, gy = (g.M + bm - 1) / bm;
  if (g.nb < 1) g.nb = 1;
  if (g.nsplit < 1) g.nsplit = 1;
  if ((long long)g.nsplit * g.kchunk < g.K) return cudaErrorInvalidValue;
  const long long gz = (long long)g.nb * g.nsplit;
  dim3 grid(gx, gy, (unsigned)gz);
  if (gy > 65535 || gz > 65535) return cudaErrorInvalidConfiguration;
  const bool ac = op.dta == C64, bc = op.dtb == C64, cc = op.dtc == C64;
  if (ac && bc)
    launch_typed<true, true, true>(op.tile, grid, g, st);
  else if (ac && !bc)
    launch_typed<true, false, true>(op.tile, grid, g, st);
  else if (!ac && bc)
    launch_typed<false, true, true>(op.tile, grid, g, st);
  else if (cc)
    launch_typed<false, false, true>(op.tile, grid, g, st);
  else
    launch_typed<false, false, false>(op.tile, grid, g, st);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// elementwise: C[idx] (+)= sum_t coef_t * A_t[idx] (* B_t[idx])
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 ld(const void* p, long long off, int cplx) {
  if (cplx) return static_cast<const double2*>(p)[off];
  return make_double2(static_cast<const double*>(p)[off], 0.0);
}

// c x for c = +-2^k from the bits of x, with no FP64 operation, where x and
// the product are normal; otherwise (and for infinities and NaNs) fma(c, x,
// +0), whose value the bit path also gives: a zero x gives +0, and a normal
// product is exact.  sgn = c's sign bit, k its unbiased exponent.
__device__ __forceinline__ double scale_pow2(double x, double c, unsigned long long sgn, int k) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long mag = u & 0x7FFFFFFFFFFFFFFFull;
  if (mag == 0ull) return 0.0;
  const int E = (int)(mag >> 52), Er = E + k;
  if (E == 0 || E == 2047 || Er <= 0 || Er >= 2047) return fma(c, x, 0.0);
  return __longlong_as_double((long long)((u ^ sgn) + ((unsigned long long)(long long)k << 52)));
}

template <typename IDX>
__global__ void __launch_bounds__(256) add_kernel(const AddArgs a) {
  const IDX stride = (IDX)gridDim.x * blockDim.x;
  // The first term starts the sum: when it is A alone with a real
  // coefficient +-2^k (the antisymmetrisers' +-1, the 1/2 and 1/4 of tau)
  // it takes no FP64 operation (the FP64 pipe is the one these sums wait on)
  const unsigned long long cb = (unsigned long long)__double_as_longlong(a.t[0].cr);
  const int ce = (int)((cb >> 52) & 0x7FF);
  const bool first_p2 = a.nt > 0 && a.t[0].B == nullptr && __double_as_longlong(a.t[0].ci) == 0 &&
                        (cb & 0x000FFFFFFFFFFFFFull) == 0ull && ce > 0 && ce < 2047;
  const unsigned long long csgn = cb & 0x8000000000000000ull;
  const int ck = ce - 1023;
  for (IDX idx = (IDX)blockIdx.x * blockDim.x + threadIdx.x; idx < (IDX)a.total; idx += stride) {
    // decode the (coalesced) index, last dimension fastest
    IDX l = idx;
    int ii[kAddDims];
#pragma unroll
    for (int q = kAddDims - 1; q >= 0; --q) {
      ii[q] = 0;
      if (q < a.nd) {
        const IDX d = (IDX)a.d[q];
        ii[q] = (int)(l % d);
        l /= d;
      }
    }
    double2 s = cz();
    int t0 = 0;
    if (first_p2) {
      long long oa = 0;
#pragma unroll
      for (int q = 0; q < kAddDims; ++q)
        if (q < a.nd) oa += (long long)ii[q] * a.t[0].sA[q];
      const double2 x = ld(a.t[0].A, oa, a.t[0].ac);
      s = make_double2(scale_pow2(x.x, a.t[0].cr, csgn, ck), scale_pow2(x.y, a.t[0].cr, csgn, ck));
      t0 = 1;
    }
    for (int t = t0; t < a.nt; ++t) {
      const AddTerm& T = a.t[t];
      long long oa = 0, ob = 0;
#pragma unroll
      for (int q = 0; q < kAddDims; ++q) {
        if (q < a.nd) {
          oa += (long long)ii[q] * T.sA[q];
          ob += (long long)ii[q] * T.sB[q];
        }
      }
      double2 x = ld(T.A, oa, T.ac);
      if (T.B) {
        const double2 y = ld(T.B, ob, T.bc);
        x = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
      }
      if (T.ci == 0.0) {  // real coefficients (almost all): half the FP64 operations
        s.x = fma(T.cr, x.x, s.x);
        s.y = fma(T.cr, x.y, s.y);
      } else {
        s.x += T.cr * x.x - T.ci * x.y;
        s.y += T.cr * x.y + T.ci * x.x;
      }
    }
    long long oc = 0;
#pragma unroll
    for (int q = 0; q < kAddDims; ++q)
      if (q < a.nd) oc += (long long)ii[q] * a.sC[q];
    // accumulation as an L2 reduction (no return value): one writer per
    // element, so the single addition c + s equals a read-modify-write, and
    // neither the load nor the add occupies the SM (its FP64 pipe is narrow)
    if (a.cc) {
      double2* C = static_cast<double2*>(a.C);
      if (a.acc) {
        atomicAdd(&C[oc].x, s.x);
        atomicAdd(&C[oc].y, s.y);
      } else {
        C[oc] = s;
      }
    } else {
      double* C = static_cast<double*>(a.C);
      if (a.acc)
        atomicAdd(&C[oc], s.x);
      else
        C[oc] = s.x;
    }
  }
}

cudaError_t launch_add(const AddArgs& a, cudaStream_t st) {
  if (a.total <= 0) return cudaSuccess;
  if (a.nd < 1 || a.nd > kAddDims) return cudaErrorInvalidValue;
  long long blocks = (a.total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  // 32-bit index arithmetic unless the index space needs 64 bits
  if (a.total + (long long)blocks * 256 < (1LL << 32))
    add_kernel<unsigned><<<(unsigned)blocks, 256, 0, st>>>(a);
  else
    add_kernel<unsigned long long><<<(unsigned)blocks, 256, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// reduction: out[o] (+)= c * sum_r X[o, r] (* Y[o, r]).  One warp per output
// element, lanes over the reduction index, fixed-order shuffle sum.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long red_off(const int* d, const long long* s, int nd, long long l) {
  long long off = 0;
#pragma unroll
  for (int q = kRedDims - 1; q >= 0; --q) {
    if (q < nd) {
      off += (l % d[q]) * s[q];
      l /= d[q];
    }
  }
  return off;
}

__global__ void __launch_bounds__(256) reduce_kernel(const ReduceArgs r) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < r.nout; w += nw) {
    const long long oo = red_off(r.dout, r.so_out, r.no, w);
    const long long ox = red_off(r.dout, r.so_x, r.no, w);
    const long long oy = red_off(r.dout, r.so_y, r.no, w);
    double sr = 0.0, si = 0.0;
    for (long long k = lane; k < r.nred; k += 32) {
      const double2 x = static_cast<const double2*>(r.X)[ox + red_off(r.dred, r.sr_x, r.nr, k)];
      double2 v = x;
      if (r.Y) {
        const long long yo = oy + red_off(r.dred, r.sr_y, r.nr, k);
        const double2 y = ld(r.Y, yo, r.ycplx);
        v = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
      }
      sr += v.x;
      si += v.y;
    }
    for (int dd = 16; dd > 0; dd >>= 1) {
      sr += __shfl_down_sync(0xffffffffu, sr, dd);
      si += __shfl_down_sync(0xffffffffu, si, dd);
    }
    if (lane == 0) {
      double2* out = static_cast<double2*>(r.out);
      const double vr = r.cr * sr - r.ci * si, vi = r.cr * si + r.ci * sr;
      if (r.acc) {
        double2 c = out[oo];
        c.x += vr;
        c.y += vi;
        out[oo] = c;
      } else {
        out[oo] = make_double2(vr, vi);
      }
    }
  }
}

cudaError_t launch_reduce(const ReduceArgs& r, cudaStream_t st) {
  if (r.nout <= 0) return cudaSuccess;
  if (r.no < 0 || r.no > kRedDims || r.nr < 0 || r.nr > kRedDims) return cudaErrorInvalidValue;
  long long blocks = (r.nout + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(r);
  count_launch();
  return cudaGetLastError();
}

struct TraceBatch {
  long long bs[4];  // batch strides of Dij, l1, Dai, Dab (elements)
  long long bsres;
};

// dipole trace: res[k] = sum_ij mu_k[i,j] rho[i,j], rho = [[Dij, l1],[Dai, Dab]]
// One CTA per dipole component; warp-shuffle + shared-memory reduction, so
// the sum order is fixed (deterministic).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) trace_kernel(int n, int o, const double* mu,
                                                     const double2* dij, const double2* l1,
                                                     const double2* dai, const double2* dab,
                                                     double2* res, TraceBatch tb) {
  const int k = blockIdx.x;
  const int z = blockIdx.y;  // trajectory
  dij += z * tb.bs[0];
  l1 += z * tb.bs[1];
  dai += z * tb.bs[2];
  dab += z * tb.bs[3];
  res += z * tb.bsres;
  const int v = n - o;
  const double* M = mu + (long long)k * n * n;
  double sr = 0.0, si = 0.0;
  const long long nn = (long long)n * n;
  for (long long e = threadIdx.x; e < nn; e += blockDim.x) {
    const int p = (int)(e / n), q = (int)(e % n);
    double2 r;
    if (p < o && q < o)
      r = dij[p * o + q];
    else if (p < o)
      r = l1[p * v + (q - o)];
    else if (q < o)
      r = dai[(p - o) * o + q];
    else
      r = dab[(long long)(p - o) * v + (q - o)];
    const double m = M[e];
    sr = fma(m, r.x, sr);
    si = fma(m, r.y, si);
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

cudaError_t launch_trace(int n, int o, int n_mu, const double* mu, const void* dij, const void* l1,
                         const void* dai, const void* dab, void* res, int nb, const long long* bs,
                         long long bsres, cudaStream_t st) {
  TraceBatch tb;
  for (int k = 0; k < 4; ++k) tb.bs[k] = nb > 1 ? bs[k] : 0;
  tb.bsres = nb > 1 ? bsres : 0;
  trace_kernel<<<dim3(n_mu, nb > 1 ? nb : 1), 1024, 0, st>>>(n, o, mu, static_cast<const double2*>(dij),
                                                             static_cast<const double2*>(l1),
                                                             static_cast<const double2*>(dai),
                                                             static_cast<const double2*>(dab),
                                                             static_cast<double2*>(res), tb);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdcc
