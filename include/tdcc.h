/*
 * tdcc.h -- C ABI of libtdcc.so, the GB300 (sm_103a) engine for the
 * time-dependent CCSD / CC2 hot path of yramis/python_code_to_check_C.
 *
 * The reference is pure Python (numpy + opt_einsum) and has no FFI; each
 * entry point below names the reference method it replaces (file:line in the
 * reference project).  A Python caller binds these with ctypes
 * (python_code_to_check_c_gb300/_lib.py); any other host language binds the
 * same symbols.
 *
 * Conventions
 *  - Return value: TDCC_OK (0) or a negative TDCC_ERR_* code; the message of
 *    the last failure on the calling thread is read with tdcc_last_error().
 *  - Every array is caller-owned DEVICE memory, C-contiguous:
 *      t1, l1 : complex128 [o][v]          (interleaved re, im doubles)
 *      t2, l2 : complex128 [o][o][v][v]
 *      F      : complex128 [n][n]          (Fock + field, n = o + v)
 *      tei    : float64    [n][n][n][n]    antisymmetrised <pq||rs>,
 *                                          occupied orbitals first
 *      fock   : float64    [n][n]
 *      mu     : float64    [n_mu][n][n]    dipole matrices (z is the last)
 *  - `stream` is a cudaStream_t (0 = legacy default stream).  Calls are
 *    asynchronous with respect to the host unless stated otherwise.
 *  - A tdcc_system is not thread-safe: use one per host thread.
 */
#ifndef TDCC_H
#define TDCC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tdcc_system_s* tdcc_system;

enum {
  TDCC_OK = 0,
  TDCC_ERR_ARG = -1,       /* bad size / pointer / enum value              */
  TDCC_ERR_CUDA = -2,      /* a CUDA runtime call failed                   */
  TDCC_ERR_ALLOC = -3,     /* device allocation failed                     */
  TDCC_ERR_STATE = -4,     /* call not valid in the current state          */
  TDCC_ERR_NONFINITE = -5, /* propagation produced NaN/Inf                 */
  TDCC_ERR_LIMIT = -6      /* size beyond a documented maximum             */
};

enum { TDCC_CCSD = 0, TDCC_CC2 = 1 };

/* residual blocks */
enum { TDCC_T1 = 0, TDCC_T2 = 1, TDCC_L1 = 2, TDCC_L2 = 3 };

/* contraction arithmetic */
enum {
  TDCC_PREC_FP64 = 0,      /* every contraction in FP64 (the plain form)   */
  TDCC_PREC_MIXED = 1      /* large contractions as split-BF16 tcgen05
                              products, FP64 everywhere else               */
};

/* external field E(t); the Fock matrix seen by a stage at time t is
   F(t) = fock - E(t) * mu_z  (mu_z = last dipole matrix).                 */
enum {
  TDCC_FIELD_NONE = 0,
  TDCC_FIELD_SIN = 1,       /* E = A sin(w0 t)                              */
  TDCC_FIELD_REFERENCE = 2, /* E = A exp(i 2 pi w0 t): the reference's Vt
                               (CCSD_Helper.py:1197-1200)                  */
  TDCC_FIELD_ENVELOPE = 3   /* E = A sin(w0 t) sum_k c_k exp(-(t-t_k)^2/(2 s^2)),
                               t_k = env_t0 + k * env_dt                   */
};

#define TDCC_MAX_ENVELOPE 64

typedef struct tdcc_field {
  int kind;
  double A;
  double w0;
  int n_env;                      /* number of envelope bumps (<= 64)       */
  double env_t0, env_dt, env_sigma;
  double env_c[TDCC_MAX_ENVELOPE];
} tdcc_field;

/* ABI version (increments on incompatible changes). */
int tdcc_version(void);

/* Copies the last error message of this thread into buf (NUL-terminated). */
int tdcc_last_error(char* buf, size_t len);

/* Number of kernels this library has launched in this process (all entry
   points, all devices).  Used by benchmarks to report launch counts.      */
long long tdcc_launch_count(void);

/* Builds a system from device-resident integrals (replaces
   CCSD_Helper.__init__ / TEI_MO / F_MO / Defd_dipole,
   CCSD_Helper.py:26-54, 57-93, 970-980).  tei/fock/mu are borrowed: they
   must stay valid until tdcc_system_destroy.  Allocates workspace lazily.  */
int tdcc_system_create(int o, int v, const double* tei, const double* fock,
                       const double* mu, int n_mu, tdcc_system* out);
int tdcc_system_destroy(tdcc_system s);

/* A system that advances nb (1..1024) trajectories over the same integrals
   together; no counterpart in the reference, which runs one trajectory per
   process.  Every per-trajectory array of the other entry points then holds
   nb copies back to back ([nb][...]): t1/t2/l1/l2 and their outputs, the
   dressed Fock matrix of tdcc_rhs ([nb][n][n]), mu_out ([nb][n_mu]) and the
   trajectories of tdcc_propagate ([nsteps][nb]).  Contractions with an
   integral operand run once for all trajectories (the trajectory index
   joins the GEMM's row or column modes); products of two per-trajectory
   operands run as batched products.  tdcc_ground_state needs nb = 1 (make
   a single-trajectory system over the same integrals for it).             */
int tdcc_system_create_batched(int o, int v, const double* tei, const double* fock,
                               const double* mu, int n_mu, int nb, tdcc_system* out);
int tdcc_system_batch(tdcc_system s);   /* nb of the system (0 for NULL) */

/* Per-trajectory fields for tdcc_rk4_step / tdcc_propagate called with
   field = NULL: fields (HOST tdcc_field[nb]) and pol (HOST int[nb], the
   dipole component 0..n_mu-1 each field couples to and whose expectation
   value tdcc_propagate records; NULL = the last component).  fields = NULL
   clears them.  A non-NULL field argument overrides them: that field for
   every trajectory, along the last component.                             */
int tdcc_set_fields(tdcc_system s, const tdcc_field* fields, const int* pol);

/* Selects the contraction arithmetic (TDCC_PREC_*) and, for the mixed mode,
   the number of BF16 slices per operand (2..6; 7 bits each).  With up to 4
   slices the tensor-core products take the 128-column tile or, for one or
   two K blocks, the persistent 64-column form; with 5 or 6 the 64-column
   tile.  4 slices keep |d mu| within 1e-8 a.u. of the FP64 form over 2000
   steps of the o=10, v=38 system; strongly correlated systems need 5.    */
int tdcc_set_precision(tdcc_system s, int mode, int slices);

/* Ground-state amplitudes by Jacobi sweeps with eigh(F) denominators and
   DIIS, on the device.  Replaces DIIS_solver / DIIS_solver_Lam
   (CCSD_Helper.py:347-416, 702-776) and DIIS_solver_CC2 /
   DIIS_solver_Lam_CC2 (CC2_Helper.py:179-248, 324-400) with the same
   storage pattern (including the CC2 Lambda order, CC2_Helper.py:382).
   mode 0: T amplitudes, t1/t2 updated in place (l1, l2 may be NULL);
   mode 1: Lambda amplitudes, l1/l2 updated in place, t1/t2 fixed.
   eps: HOST double[n], the ascending eigenvalues of the Fock matrix.
   Stops when |dE| < e_min (the reference's test; it uses 1e-15) or, if
   r_tol > 0, when a sweep's max |residual| < r_tol, or after maxiter.
   energy: correlation energy (mode 0) or pseudo-energy E1 + E2 (mode 1).
   Synchronous; allocates its vector store for the duration of the call. */
int tdcc_ground_state(tdcc_system s, int method, int mode, void* t1, void* t2, void* l1, void* l2,
                      const double* eps, int maxsize, int maxiter, double e_min, double r_tol,
                      double* energy, int* niter, void* stream);

/* Mixed mode routing: contractions with at least min_macs multiply-adds, a
   contracted extent K >= min_k and output extents M, N >= min_mn (per
   launch, trajectories folded in) run on the tensor cores (defaults 2^18,
   32, 1); the rest stay FP64.  (0, 1, 1) sends every contraction to the
   tensor cores, which tests use at small sizes.                           */
int tdcc_set_tc_policy(tdcc_system s, long long min_macs, int min_k, int min_mn);

/* Mixed mode, contractions the tensor cores leave out: those with K <= max_k
   and at least min_macs multiply-adds run as the same exact BF16-digit slice
   products on the FP32 pipe (defaults 64 and 2^14; max_k = 0 keeps them
   FP64).  GB300's FP64 pipe is narrow and shared with the elementwise ops. */
int tdcc_set_simt_policy(tdcc_system s, int max_k, long long min_macs);

/* Workspace buffer sharing (no counterpart in the reference): a program whose
   workspace slots add up to more than min_bytes lets slots with disjoint
   lifetimes within one phase share memory (fewer bytes, some ops ordered
   that could otherwise run concurrently).  min_bytes < 0: the default
   (1 GiB); 0: always.  Reverse mode (tdcc_adjoint) turns sharing off for the
   system, as it reads every forward value after a stage ran.             */
int tdcc_set_memory_sharing(tdcc_system s, long long min_bytes);

/* Reverse mode's forward intermediates (no counterpart in the reference):
   mode 1 keeps, per step of a checkpoint segment, the intermediates each
   block's reverse-mode program reads (written by the captured forward step);
   mode 0 runs each stage's forward ops again before its reverse; mode -1
   (default) keeps them when the records need at most half the free device
   memory.  Both give the same gradients up to summation order.          */
int tdcc_set_adjoint_store(tdcc_system s, int mode);

/* Synchronises the device and reports TDCC_ERR_CUDA if a kernel of this
   system recorded an error (a tensor-core kernel whose bounded wait
   expired); clears the flag.                                              */
int tdcc_check_errors(tdcc_system s);

/* Bytes of device workspace currently held by the system.                 */
long long tdcc_workspace_bytes(tdcc_system s);

/* One right-hand side.  Replaces, by (method, block):
     CCSD T1 : CCSD_Helper.T1eq_rhs      (CCSD_Helper.py:177-196)
     CCSD T2 : CCSD_Helper.T2eq_rhs      (CCSD_Helper.py:268-309)
     CCSD L1 : CCSD_Helper.lam_1eq_rhs   (CCSD_Helper.py:555-581)
     CCSD L2 : CCSD_Helper.lam2eq_rhs    (CCSD_Helper.py:610-648)
     CC2  T1 : CCSD_Helper.T1eq_rhs      (used by CC2, CC2_Helper.py:463)
     CC2  T2 : CC2_Helper.T2eq_rhs_CC2   (CC2_Helper.py:12-47)
     CC2  L1 : CC2_Helper.L1eq_rhs_CC2   (CC2_Helper.py:50-125)
     CC2  L2 : CC2_Helper.L2eq_rhs_CC2   (CC2_Helper.py:128-175)
   Inputs not used by a block may be NULL (T blocks ignore l1, l2).
   `out` has the shape of the block's amplitude.                          */
int tdcc_rhs(tdcc_system s, int method, int block, const void* t1, const void* t2,
             const void* l1, const void* l2, const void* F, void* out, void* stream);

/* Correlated one-particle density blocks and the dipole expectation value
   sum_pq mu^k_pq rho_pq for every dipole component k (replaces
   CCSD_Helper.dipole_moment, Dij/Dab/Dai, CCSD_Helper.py:984-1006,
   1066-1092).  mu_out: device complex128[n_mu].                           */
int tdcc_dipole(tdcc_system s, const void* t1, const void* t2, const void* l1,
                const void* l2, void* mu_out, void* stream);

/* One step of the block-frozen RK4 propagator (the loop body of
   CCSD_Helper.Runge_Kutta_solver, CCSD_Helper.py:1206-1240, and of
   CC2_Helper.Runge_Kutta_solver_CC2, CC2_Helper.py:451-472, with
   ft1/ft2/fL1/fL2 at CCSD_Helper.py:1158-1187 and CC2_Helper.py:412-433).
   t_prev is the time before the step; the stages see the field at
   t = t_prev + dt, t + dt/2, t + dt (the reference advances t first).
   The new state round(old, precs) + delta is written to the *_out arrays
   (which may alias the inputs).  If mu_out is not NULL the dipole of the
   new state is written there (complex128[nb][n_mu]).  field: see
   tdcc_set_fields.                                                        */
int tdcc_rk4_step(tdcc_system s, int method, const void* t1, const void* t2,
                  const void* l1, const void* l2, void* t1_out, void* t2_out,
                  void* l1_out, void* l2_out, double t_prev, double dt, int precs,
                  const tdcc_field* field, void* mu_out, void* stream);

/* nsteps RK4 steps with the state resident on the device and the step
   captured once in a CUDA graph.  The state arrays are read at entry and
   overwritten with the final state.  mu_traj (device complex128[nsteps][nb])
   receives after every step each trajectory's dipole component along its
   field (mu_z for a single trajectory).  Synchronous: returns after the
   last step completed (TDCC_ERR_NONFINITE if a final dipole is not
   finite).                                                                */
int tdcc_propagate(tdcc_system s, int method, void* t1, void* t2, void* l1, void* l2,
                   double t0, double dt, int nsteps, int precs,
                   const tdcc_field* field, void* mu_traj, void* stream);

/* Gradient of a dipole-response objective with respect to the field, by
   reverse mode through tdcc_propagate's steps (no counterpart in the
   reference).  J_b = sum_n w[n] Re mu_b(t_n) over the recorded dipole of
   trajectory b after step n (n = 0..nsteps-1, the trajectory tdcc_propagate
   records).  Writes J_out[b] (host double[nb]) and gE_host (host
   complex128 as interleaved doubles, [nsteps][4][nb]): the derivative of J_b
   with respect to the field value at each right-hand-side evaluation of step
   n -- RK4 stage s = 0..3 at t, t + dt/2, t + dt/2, t + dt with t the step's
   time (t0 advanced n + 1 times by dt) -- so that for any real parameter
   theta of the field dJ_b/dtheta = sum_{n,s} Re(gE[n][s][b] dE_b(tau)/dtheta).
   If a_t1..a_l2 are not NULL they receive dJ/d(initial state) (conjugated:
   conj(dJ/dRe + i dJ/dIm)).  The forward runs the captured step graphs and
   keeps the state every `checkpoint` steps; the backward recomputes each
   segment on the step graphs (storing per step the state, the stage inputs
   and the dressed Fock matrices) and runs the generated reverse-mode
   programs (the vector-Jacobian products of the right-hand sides) stage by
   stage.  checkpoint >= nsteps: the forward pass itself keeps every step
   and nothing is recomputed (memory: nsteps x (4 states + Fock)).  The rounding of the state (precs >= 0)
   is taken as the identity; precs < 0 makes the map smooth.  Synchronous;
   allocates its checkpoint and segment storage for the duration of the call.
   Fields: `field` for every trajectory, or tdcc_set_fields when NULL.      */
int tdcc_adjoint(tdcc_system s, int method, const void* t1, const void* t2, const void* l1,
                 const void* l2, double t0, double dt, int nsteps, int precs,
                 const tdcc_field* field, const double* w_host, int checkpoint,
                 double* J_out, double* gE_host, void* a_t1, void* a_t2, void* a_l1,
                 void* a_l2, void* stream);

/* Autotuner (no counterpart in the reference): runs one step from the given
   state to fill the workspaces, then times every contraction of the
   method's programs under candidate launch shapes -- FP64 kernel: tile shape
   x split-K on/off; tensor-core kernel: K splits -- and keeps the fastest
   (reps timed launches each, CUDA events).  Recomputes the per-system
   constants afterwards and drops the captured step graphs.  n_tuned: ops
   changed; ms_before / ms_after: summed per-launch times of all
   contractions (one pass of every op).  Any pointer output may be NULL.   */
int tdcc_autotune(tdcc_system s, int method, const void* t1, const void* t2, const void* l1,
                  const void* l2, int reps, int* n_tuned, double* ms_before, double* ms_after,
                  void* stream);

/* Reverse-mode op list of (method, block) as JSON (like tdcc_program_json):
   forward slots [0, nfwd), adjoint slots after them, "adj_of" maps each
   forward slot to its adjoint slot (-1: not differentiable).  No GPU.     */
long long tdcc_adjoint_program_json(int o, int v, int method, int block, int n_mu, int nb,
                                    char* buf, size_t len);

/* Antisymmetrised two-electron integrals from density-fitting factors, on
   the device (the integral provider; the reference reads psi4's
   mo_spin_eri, CCSD_Helper.py:57-93):
     tei[p,q,r,s] = sum_Q B[Q,p,r] B[Q,q,s] - sum_Q B[Q,p,s] B[Q,q,r]
   B: device float64 [nq][n][n]; tei: device float64 [n][n][n][n] (written).
   FP64 GEMM over Q, then an in-place antisymmetrisation.                   */
int tdcc_tei_from_df(const double* B, int n, int nq, double* tei, void* stream);

/* Dipole spectrum (Plots.py:20-25): the discrete Fourier transforms of
   Re mu(t) and Im mu(t), each fftshift-ed:
     Yr[j] = sum_n Re mu[n] exp(-2 pi i k n / N),  k = (j + N - N/2) mod N
   (Yi likewise with Im mu), N = nsteps, mu[n * stride] device complex128;
   Yr, Yi: device complex128 [N].  energy_ev (host [N], may be NULL): the
   reference's axis (j - N/2) / (N dt) * 2 pi * 27.211 eV.                 */
int tdcc_spectrum(const void* mu, long long nsteps, long long stride, double dt, void* Yr, void* Yi,
                  double* energy_ev, void* stream);

/* Dipole expectation value like tdcc_dipole, but without allocating any
   device memory and without a tdcc_system.  No counterpart in the reference
   (its dipole_moment, CCSD_Helper.py:1066, allocates numpy temporaries).
   For callers that cannot call cudaMalloc: code that runs inside someone
   else's stream capture, plugins whose host framework owns all device
   memory, processes that must not grow after start-up.
   Scratch: a static device array of 3.375 MiB (221,184 complex128) that
   every device loading the library keeps until exit; limits o <= 64 and
   v <= 256 (larger: TDCC_ERR_LIMIT).  The first call on a device looks up
   the array's device address (cudaGetSymbolAddress) with that device
   current; make that first call before any stream capture.  The address is
   kept for the life of the process: a device reset (cudaDeviceReset) in
   between is not supported.  All calls share the one array: calls whose GPU
   work overlaps (different streams or threads) race and give wrong results
   -- serialise them.  Inputs as in
   tdcc_dipole; mu: device float64 [n_mu][n][n]; mu_out: device
   complex128[n_mu].                                                       */
int tdcc_dipole_noalloc(int o, int v, const void* t1, const void* t2, const void* l1,
                        const void* l2, const double* mu, int n_mu, void* mu_out,
                        void* stream);

/* Writes a JSON description of the op list that computes (method, block)
   for sizes (o, v) and nb trajectories: buffer slots, and per op the GEMM
   mode groups / strides / batch strides or the elementwise terms, plus
   whether the op runs once per RK4 step or in every stage.  block = 4
   selects the density / dipole program.  Needs no GPU (used by the CPU
   tests to check the programs; no counterpart in the reference).  Returns
   the JSON length; TDCC_ERR_LIMIT if buf is too small.                    */
long long tdcc_program_json(int o, int v, int method, int block, int n_mu, int nb, char* buf,
                            size_t len);

/* Per-kernel timing record of tdcc_profile_step. */
typedef struct tdcc_op_record {
  char tag[96];   /* "<program>:<einsum>" or the kernel's role               */
  int kind;       /* 0 contraction, 1 elementwise, 2 trace, 3 RK4 / field    */
  int block;      /* 0..3 = T1, T2, L1, L2 block; 4 = density; 5 = step      */
  int stage;      /* 0 = prologue (once per step), 1..4 = RK4 stage          */
  int backend;    /* contractions: 0 FP64 CUDA cores, 1 tensor cores         */
  double flops;   /* real floating-point operations of the op               */
  double bytes;   /* compulsory bytes read + written by the op              */
  double ms;      /* device time from CUDA events on the launching stream    */
} tdcc_op_record;

/* Runs one RK4 step eagerly on a single stream with a CUDA-event pair around
   every kernel and returns one record per launch (diagnostics and the
   benchmark's roofline figures; no counterpart in the reference).  The state
   is not modified.  Synchronous.                                          */
int tdcc_profile_step(tdcc_system s, int method, const void* t1, const void* t2,
                      const void* l1, const void* l2, double t_prev, double dt,
                      int precs, const tdcc_field* field, tdcc_op_record* recs,
                      int max_recs, int* n_recs);

#ifdef __cplusplus
}
#endif

#endif /* TDCC_H */
