// Device-side step context and launchers of the RK4 kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/tdcc.h"
#include "engine.h"

namespace tdcc {

// Lives in device memory so that a captured step graph advances the time and
// evaluates the field itself.
struct StepCtx {
  double t;        // time of the current step (after the reference's t += dt)
  double dt;
  tdcc_field field;
  double2 E[3];    // field at t, t + dt/2, t + dt
  long long step;  // steps taken (index into the trajectory)
};

cudaError_t launch_advance_field(StepCtx* ctx, cudaStream_t st);
cudaError_t launch_dress(const StepCtx* ctx, const double* fock, const double* muz, double2* Fs,
                         int n, cudaStream_t st);
cudaError_t launch_rk4_stage(const double2* y0, const double2* k, double2* acc, double2* yin,
                             long long n, int s, double h, cudaStream_t st);
cudaError_t launch_rk4_finish(const double2* y0, const double2* acc, double2* ynew, long long n,
                              double dt6, int sign, double scale, int do_round, cudaStream_t st);
cudaError_t launch_record_mu(StepCtx* ctx, const double2* res, int n_mu, double2* traj,
                             double* times, cudaStream_t st);

}  // namespace tdcc
