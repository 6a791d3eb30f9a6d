// HBM-bound kernels of the block-frozen RK4 propagator: field evaluation,
// Fock dressing, the fused stage axpys and the rounded final update.
// Reference: CCSD_Helper.py:1158-1240 (ft1/ft2/fL1/fL2, Runge_Kutta_solver).
#include <cmath>

#include "rk4.h"

namespace tdcc {

__device__ double2 field_value(const tdcc_field& f, double t) {
  switch (f.kind) {
    case TDCC_FIELD_SIN:
      return make_double2(f.A * sin(f.w0 * t), 0.0);
    case TDCC_FIELD_REFERENCE: {
      // cmath.exp(1j*w0*2*np.pi*t): phase evaluated as ((w0*2)*pi)*t
      const double th = ((f.w0 * 2.0) * 3.141592653589793) * t;
      return make_double2(f.A * cos(th), f.A * sin(th));
    }
    case TDCC_FIELD_ENVELOPE: {
      double env = 0.0;
      for (int k = 0; k < f.n_env; ++k) {
        const double d = (t - (f.env_t0 + k * f.env_dt)) / f.env_sigma;
        env += f.env_c[k] * exp(-0.5 * d * d);
      }
      return make_double2(f.A * sin(f.w0 * t) * env, 0.0);
    }
    default:
      return make_double2(0.0, 0.0);
  }
}

// ctx->t += dt (the reference advances t before the stages), then each
// trajectory's field at t, t + dt/2, t + dt.  One block: every thread reads
// the old time before thread 0 stores the new one.
__global__ void advance_field_kernel(StepCtx* ctx) {
  const double t = __dadd_rn(ctx->t, ctx->dt);
  const double dt = ctx->dt, h = dt / 2.0;
  const int b = threadIdx.x;
  if (b < ctx->nb) {
    const tdcc_field& f = ctx->fields[b];
    double2* E = ctx->E + 3 * b;
    E[0] = field_value(f, t);
    E[1] = field_value(f, __dadd_rn(t, h));
    E[2] = field_value(f, __dadd_rn(t, dt));
  }
  __syncthreads();
  if (threadIdx.x == 0) ctx->t = t;
}

// Fs[s][b] = fock - E[b][s] * mu[pol[b]]  for the three stage times
__global__ void dress_kernel(const StepCtx* ctx, const double* __restrict__ fock,
                             const double* __restrict__ mu, double2* __restrict__ Fs, int nn) {
  const int s = blockIdx.y, b = blockIdx.z;
  const int nb = ctx->nb;
  const double2 E = ctx->E[3 * b + s];
  const double* m = mu + (long long)ctx->pol[b] * nn;
  double2* out = Fs + ((long long)s * nb + b) * nn;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += gridDim.x * blockDim.x) {
    const double me = m[e];
    out[e] = make_double2(fock[e] - E.x * me, -(E.y * me));
  }
}

// Stage s (1..4) after k_s is known:
//   s=1: acc = k            ; yin = y0 + (dt/2) k
//   s=2: acc = acc + 2k     ; yin = y0 + (dt/2) k
//   s=3: acc = acc + 2k     ; yin = y0 + dt k
//   s=4: acc = acc + k
// Evaluation order and roundings follow numpy's for
// dt/6.0*(k1 + 2.0*k2 + 2.0*k3 + k4) and t + dt/2.0*k (no FMA contraction).
__global__ void rk4_stage_kernel(const double2* __restrict__ y0, const double2* __restrict__ k,
                                 double2* __restrict__ acc, double2* __restrict__ yin, long long n,
                                 int s, double h) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 kk = k[i];
    double2 a;
    if (s == 1) {
      a = kk;
    } else {
      a = acc[i];
      if (s == 4) {
        a.x = __dadd_rn(a.x, kk.x);
        a.y = __dadd_rn(a.y, kk.y);
      } else {
        a.x = __dadd_rn(a.x, __dmul_rn(2.0, kk.x));
        a.y = __dadd_rn(a.y, __dmul_rn(2.0, kk.y));
      }
    }
    acc[i] = a;
    if (s < 4) {
      const double2 y = y0[i];
      yin[i] = make_double2(__dadd_rn(y.x, __dmul_rn(h, kk.x)), __dadd_rn(y.y, __dmul_rn(h, kk.y)));
    }
  }
}

__device__ __forceinline__ double round_dec(double x, double scale) {
  // np.around(x, decimals): rint(x * 10**decimals) / 10**decimals
  return __ddiv_rn(rint(__dmul_rn(x, scale)), scale);
}

// ynew = round(y0, precs) + sign_i * (dt/6) * acc, sign_i = -i (T) or +i (Lambda)
__global__ void rk4_finish_kernel(const double2* __restrict__ y0, const double2* __restrict__ acc,
                                  double2* __restrict__ ynew, long long n, double dt6, int sign,
                                  double scale, int do_round) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 a = acc[i];
    const double dx = __dmul_rn(dt6, a.x), dy = __dmul_rn(dt6, a.y);
    // (-1j)*(dx + i dy) = dy - i dx ; (+1j)*(dx + i dy) = -dy + i dx
    const double2 d = sign < 0 ? make_double2(dy, -dx) : make_double2(-dy, dx);
    double2 y = y0[i];
    if (do_round) {
      y.x = round_dec(y.x, scale);
      y.y = round_dec(y.y, scale);
    }
    ynew[i] = make_double2(__dadd_rn(y.x, d.x), __dadd_rn(y.y, d.y));
  }
}

__global__ void record_mu_kernel(StepCtx* ctx, const double2* res, double2* traj, double* times) {
  const long long s = ctx->step;
  const int nb = ctx->nb, b = threadIdx.x;
  if (b < nb) {
    if (traj) traj[s * nb + b] = res[(long long)b * ctx->n_mu + ctx->pol[b]];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (times) times[s] = ctx->t;
    ctx->step = s + 1;
  }
}

// ---------------------------------------------------------------------------
// reverse-mode helpers (tdcc_adjoint)
// ---------------------------------------------------------------------------
// y = c x  (acc = 0) or y += c x  (acc = 1), complex c
__global__ void caxpy_kernel(double2* __restrict__ y, const double2* __restrict__ x, long long n, double cr, double ci,
                             int acc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    const double2 p = make_double2(cr * v.x - ci * v.y, cr * v.y + ci * v.x);
    if (acc) {
      double2 w = y[i];
      w.x += p.x;
      w.y += p.y;
      y[i] = w;
    } else {
      y[i] = p;
    }
  }
}

// g[b] += sum_e aF[b][e] * (-mu[pol[b]][e]): dJ/dE of one RK4 stage, per
// trajectory (F = fock - E mu_pol).  One block per trajectory, fixed-order sum.
__global__ void __launch_bounds__(256) field_grad_kernel(const double2* __restrict__ aF, const double* __restrict__ mu,
                                                         const int* __restrict__ pol, int nn, double2* __restrict__ g,
                                                         const RevCtx* rc, int stage) {
  const int b = blockIdx.x;
  if (rc) g += (rc->cur * 4 + stage) * (long long)gridDim.x;
  const double2* a = aF + (long long)b * nn;
  const double* m = mu + (long long)pol[b] * nn;
  double sr = 0.0, si = 0.0;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    sr -= a[e].x * m[e];
    si -= a[e].y * m[e];
  }
  __shared__ double wr[8], wi[8];
  for (int d = 16; d > 0; d >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, d);
    si += __shfl_down_sync(0xffffffffu, si, d);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    wr[w] = sr;
    wi[w] = si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      tr += wr[k];
      ti += wi[k];
    }
    g[b].x += tr;
    g[b].y += ti;
  }
}

// a_res[b][k] = (k == pol[b]) ? w : 0  (cotangent of the recorded dipole component)
__global__ void dipole_cotangent_kernel(double2* __restrict__ ares, const int* __restrict__ pol, int nb, int n_mu,
                                        const double* __restrict__ wts, const RevCtx* rc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double w = wts[rc->cur];
  if (i < nb * n_mu) ares[i] = make_double2((i % n_mu) == pol[i / n_mu] ? w : 0.0, 0.0);
}

__global__ void step_store_kernel(const StepCtx* ctx, const double2* __restrict__ src, double2* __restrict__ dst,
                                  long long stride, long long n) {
  double2* d = dst + ctx->step * stride;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = src[i];
}

static unsigned grid_for(long long n);

__global__ void rev_gather_kernel(const RevCtx* rc, GatherTable t) {
  const GatherCopy c = t.c[blockIdx.y];
  const double* src = c.src + (rc->cur % rc->K + c.koff) * c.stride8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < c.n8; i += (long long)gridDim.x * blockDim.x)
    c.dst[i] = src[i];
}

__global__ void rev_advance_kernel(RevCtx* rc) { rc->cur -= 1; }

cudaError_t launch_rev_gather(const RevCtx* rc, const GatherTable& t, cudaStream_t st) {
  if (t.n <= 0) return cudaSuccess;
  long long mx = 0;
  for (int j = 0; j < t.n; ++j) mx = t.c[j].n8 > mx ? t.c[j].n8 : mx;
  rev_gather_kernel<<<dim3(grid_for(mx), (unsigned)t.n), 256, 0, st>>>(rc, t);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rev_advance(RevCtx* rc, cudaStream_t st) {
  rev_advance_kernel<<<1, 1, 0, st>>>(rc);
  count_launch();
  return cudaGetLastError();
}

__global__ void act_store_kernel(const StepCtx* ctx, ActTable t, double* base, long long stride8) {
  const ActCopy c = t.c[blockIdx.y];
  double* d = base + ctx->step * stride8 + c.off8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < c.n8; i += (long long)gridDim.x * blockDim.x)
    d[i] = c.src[i];
}

cudaError_t launch_act_store(const StepCtx* ctx, const ActTable& t, double* base, long long stride8,
                             cudaStream_t st) {
  if (t.n <= 0) return cudaSuccess;
  long long mx = 0;
  for (int j = 0; j < t.n; ++j) mx = t.c[j].n8 > mx ? t.c[j].n8 : mx;
  dim3 grid(grid_for(mx), (unsigned)t.n);
  act_store_kernel<<<grid, 256, 0, st>>>(ctx, t, base, stride8);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_step_store(const StepCtx* ctx, const double2* src, double2* dst_base, long long stride, long long n,
                              cudaStream_t st) {
  step_store_kernel<<<grid_for(n), 256, 0, st>>>(ctx, src, dst_base, stride, n);
  count_launch();
  return cudaGetLastError();
}

__global__ void sum4_kernel(double2* __restrict__ y, const double2* x0, const double2* x1, const double2* x2,
                            const double2* x3, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = y[i];
    for (const double2* x : {x0, x1, x2, x3})
      if (x) {
        v.x += x[i].x;
        v.y += x[i].y;
      }
    y[i] = v;
  }
}

cudaError_t launch_sum4(double2* y, const double2* x0, const double2* x1, const double2* x2, const double2* x3,
                        long long n, cudaStream_t st) {
  sum4_kernel<<<grid_for(n), 256, 0, st>>>(y, x0, x1, x2, x3, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_caxpy(double2* y, const double2* x, long long n, double cr, double ci, int acc, cudaStream_t st) {
  caxpy_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n, cr, ci, acc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_field_grad(const double2* aF, const double* mu, const int* pol, int n, int nb, double2* g,
                              const RevCtx* rc, int stage, cudaStream_t st) {
  field_grad_kernel<<<nb, 256, 0, st>>>(aF, mu, pol, n * n, g, rc, stage);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_dipole_cotangent(double2* ares, const int* pol, int nb, int n_mu, const double* w,
                                    const RevCtx* rc, cudaStream_t st) {
  dipole_cotangent_kernel<<<(nb * n_mu + 127) / 128, 128, 0, st>>>(ares, pol, nb, n_mu, w, rc);
  count_launch();
  return cudaGetLastError();
}

static unsigned grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return (unsigned)b;
}

static unsigned warps_for(int nb) { return (unsigned)((nb + 31) / 32 * 32); }

cudaError_t launch_advance_field(StepCtx* ctx, int nb, cudaStream_t st) {
  if (nb < 1 || nb > kMaxTrajectories) return cudaErrorInvalidValue;
  advance_field_kernel<<<1, warps_for(nb), 0, st>>>(ctx);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_dress(const StepCtx* ctx, const double* fock, const double* mu, double2* Fs, int n,
                         int nb, cudaStream_t st) {
  const int nn = n * n;
  dim3 grid((nn + 255) / 256 > 64 ? 64 : (nn + 255) / 256, 3, nb);
  dress_kernel<<<grid, 256, 0, st>>>(ctx, fock, mu, Fs, nn);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rk4_stage(const double2* y0, const double2* k, double2* acc, double2* yin,
                             long long n, int s, double h, cudaStream_t st) {
  rk4_stage_kernel<<<grid_for(n), 256, 0, st>>>(y0, k, acc, yin, n, s, h);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rk4_finish(const double2* y0, const double2* acc, double2* ynew, long long n,
                              double dt6, int sign, double scale, int do_round, cudaStream_t st) {
  rk4_finish_kernel<<<grid_for(n), 256, 0, st>>>(y0, acc, ynew, n, dt6, sign, scale, do_round);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_record_mu(StepCtx* ctx, const double2* res, int nb, double2* traj, double* times,
                             cudaStream_t st) {
  if (nb < 1 || nb > kMaxTrajectories) return cudaErrorInvalidValue;
  record_mu_kernel<<<1, warps_for(nb), 0, st>>>(ctx, res, traj, times);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdcc
