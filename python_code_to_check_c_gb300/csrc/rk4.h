// Device-side step context and launchers of the RK4 kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/tdcc.h"
#include "engine.h"

namespace tdcc {

// Lives in device memory so that a captured step graph advances the time and
// evaluates the fields itself.  Trajectory b has its own field (fields[b])
// along its own dipole component (pol[b]); all share the time grid.
struct StepCtx {
  double t;        // time of the current step (after the reference's t += dt)
  double dt;
  long long step;  // steps taken (index into the trajectory)
  int nb;          // trajectories
  int n_mu;
  const tdcc_field* fields;  // device [nb]
  const int* pol;            // device [nb]
  double2* E;                // device [nb][3]: field at t, t + dt/2, t + dt
};

constexpr int kMaxTrajectories = 1024;

// Per-step stores for reverse mode, written inside the captured step graph:
// step k's state goes to y[b] + k * sy[b], the inputs of its stages 2..4 to
// st[b][q] + k * sst[b], its dressed Fock matrices to fs + k * sfs (k is the
// device step counter).
// act[b] (when set) receives the forward intermediates that block b's
// reverse-mode program reads: per step act_stride[b] 8-byte words, the
// prologue values first, then the stage values of stages 1..4.
struct StepStore {
  double2* y[4];
  long long sy[4];
  double2* st[4][3];
  long long sst[4];
  double2* fs;
  long long sfs;
  double* act[4];
  long long act_stride[4];
};

// One launch copies up to kMaxActCopies buffers: entry j sends n8 8-byte
// words from src to base + ctx->step * stride8 + off8.
constexpr int kMaxActCopies = 32;
struct ActCopy {
  const double* src;
  long long off8;
  long long n8;
};
struct ActTable {
  int n;
  ActCopy c[kMaxActCopies];
};
cudaError_t launch_act_store(const StepCtx* ctx, const ActTable& t, double* base, long long stride8,
                             cudaStream_t st);

// dst_base + ctx->step * stride  <-  src  (n elements)
cudaError_t launch_step_store(const StepCtx* ctx, const double2* src, double2* dst_base, long long stride, long long n,
                              cudaStream_t st);

cudaError_t launch_advance_field(StepCtx* ctx, int nb, cudaStream_t st);
// Fs[s][b] = fock - E[b][s] * mu[pol[b]]  (stage-major: [3][nb][n][n])
cudaError_t launch_dress(const StepCtx* ctx, const double* fock, const double* mu, double2* Fs, int n,
                         int nb, cudaStream_t st);
cudaError_t launch_rk4_stage(const double2* y0, const double2* k, double2* acc, double2* yin,
                             long long n, int s, double h, cudaStream_t st);
cudaError_t launch_rk4_finish(const double2* y0, const double2* acc, double2* ynew, long long n,
                              double dt6, int sign, double scale, int do_round, cudaStream_t st);
// Reverse-mode step counter: one captured reverse step serves every step of
// a run.  It reads the global step cur (index cur % K within its checkpoint
// segment of K steps) and ends by decrementing cur.
struct RevCtx {
  long long cur;
  long long K;
};
// One launch gathers up to kMaxGather buffers: entry j sends n8 8-byte words
// from src + (cur % K + koff) * stride8 to dst.
constexpr int kMaxGather = 32;
struct GatherCopy {
  const double* src;
  long long stride8;
  long long koff;
  double* dst;
  long long n8;
};
struct GatherTable {
  int n;
  GatherCopy c[kMaxGather];
};
cudaError_t launch_rev_gather(const RevCtx* rc, const GatherTable& t, cudaStream_t st);
cudaError_t launch_rev_advance(RevCtx* rc, cudaStream_t st);

// reverse-mode helpers: y (+)= c x; g[b] += sum aF[b] * (-mu[pol[b]]) with
// g = g_base + (cur * 4 + stage) * nb (g_base itself when rc is null); the
// dipole cotangent a_res[b][k] = w[cur] * (k == pol[b])
cudaError_t launch_caxpy(double2* y, const double2* x, long long n, double cr, double ci, int acc, cudaStream_t st);
// y += x0 + x1 + x2 + x3 in that order (null terms skipped)
cudaError_t launch_sum4(double2* y, const double2* x0, const double2* x1, const double2* x2, const double2* x3,
                        long long n, cudaStream_t st);
cudaError_t launch_field_grad(const double2* aF, const double* mu, const int* pol, int n, int nb, double2* g_base,
                              const RevCtx* rc, int stage, cudaStream_t st);
cudaError_t launch_dipole_cotangent(double2* ares, const int* pol, int nb, int n_mu, const double* w,
                                    const RevCtx* rc, cudaStream_t st);
// traj[step][b] = res[b][pol[b]]; step += 1
cudaError_t launch_record_mu(StepCtx* ctx, const double2* res, int nb, double2* traj, double* times,
                             cudaStream_t st);

}  // namespace tdcc
