// extern "C" entry points of libtdcc.so (declared in include/tdcc.h).
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tdcc.h"
#include "engine.h"
#include "gemm_tc.h"
#include "ground.h"
#include "post.h"
#include "rk4.h"

#include <algorithm>

namespace tdcc {

static thread_local std::string g_err;
void set_error(const std::string& m) { g_err = m; }

void build_t1(Program& p);
void build_t2_ccsd(Program& p);
void build_t2_cc2(Program& p);
void build_l1_ccsd(Program& p);
void build_l2_ccsd(Program& p);
void build_l1_cc2(Program& p);
void build_l2_cc2(Program& p, const View& ones_v);
void build_density(Program& p, int n_mu);

// Tensor-core backend hooks (gemm_tc.cu); FP64 only when not compiled in.
bool tc_available();

struct ProgInst {
  std::unique_ptr<Program> prog;
  std::vector<void*> bases;
  size_t nfwd = 0;           // reverse-mode programs: slots [0, nfwd) are the forward program's
  // reverse-mode programs of the RHS blocks: the forward slots they read that
  // forward ops write once per step (prologue) or once per stage, with their
  // offsets (8-byte words) in one step's activation record
  std::vector<int> act_slot;
  std::vector<char> act_stage;
  std::vector<long long> act_off8;
  long long act_pro8 = 0, act_stage8 = 0;
  long long act_step8() const { return act_pro8 + 4 * act_stage8; }
  std::vector<void*> owned;  // this program's workspace allocations
  long long bytes = 0;
  bool setup_done = false;   // integral-only ops (e.g. packed integral blocks) ran
  DagExec dag;               // streams/events for concurrent execution of the ops
  // runs the integral-only ops once, eagerly, on `st`
  cudaError_t setup(cudaStream_t st) {
    if (setup_done) return cudaSuccess;
    const cudaError_t e = prog->run(bases, st, Program::SETUP);
    if (e == cudaSuccess) setup_done = true;
    return e;
  }
  ~ProgInst() {
    dag.destroy();
    for (void* p : owned) cudaFree(p);
  }
  // every slot an op of the program touches must be bound (checked on the
  // host before each run: an unbound slot would be a null device pointer)
  std::vector<int> used;
  void check_bound() {
    if (used.empty()) {
      std::vector<char> u(prog->slots.size(), 0);
      for (const auto& op : prog->ops) {
        for (int r : op.reads)
          if (r >= 0) u[r] = 1;
        if (op.write >= 0) u[op.write] = 1;
      }
      for (size_t i = 0; i < u.size(); ++i)
        if (u[i]) used.push_back((int)i);
    }
    for (int i : used)
      if (!bases[i]) throw std::runtime_error("unbound buffer slot " + prog->slots[i].name + " in " + prog->name);
  }
  // phase ops as a dependency DAG (serially, in program order, when timed)
  cudaError_t exec(cudaStream_t st, Program::Phase ph, std::vector<Program::Timed>* timed = nullptr) {
    check_bound();
    // TDCC_SERIAL=1 issues every op in program order on `st` (debugging aid)
    static const bool serial = [] {
      const char* e = getenv("TDCC_SERIAL");
      return e && e[0] == '1';
    }();
    if (timed || serial) return prog->run(bases, st, ph, timed);
    return prog->run_dag(bases, st, ph, dag);
  }
};

// Buffer sharing costs concurrency (shared buffers order otherwise independent
// ops), so it is used only where memory matters: programs whose workspace
// slots add up to more than this.
constexpr long long kShareMinBytes = 1LL << 30;
long long workspace_estimate(const Program& p) {
  long long b = 0;
  for (size_t i = kNumFixedSlots; i < p.slots.size(); ++i)
    if (!p.slots[i].fixed) b += p.slots[i].numel * elem_bytes(p.slots[i].dt);
  return b;
}

// contractions with at least this many multiply-adds, K >= kTcMinK and both
// output extents (per launch: M and N of the batched GEMM) >= kTcMinMN use
// the tensor-core slice products in the mixed-precision mode.  No output
// limit by default: contractions with 10 x 10 or 1 x N outputs pack mostly
// padding and take longer alone than in FP64, but the step runs its ops
// concurrently and the FP64 pipe is the shared bottleneck there (o=10, v=38:
// a limit of 16 cost 14 % with 24 trajectories, 8 % with one).
constexpr long long kTcMinMacs = 1LL << 18;
constexpr int kTcMinK = 32;
constexpr int kTcMinMN = 1;
// contractions the tensor cores leave out with K <= 64 and at least 2^14
// multiply-adds run as slice products on the FP32 pipe (mixed mode)
constexpr int kSimtMaxKDefault = 64;
constexpr long long kSimtMinMacs = 1LL << 14;

}  // namespace tdcc

using namespace tdcc;

struct tdcc_system_s {
  Dims dims;
  const double* tei = nullptr;
  const double* fock = nullptr;
  const double* mu = nullptr;
  int n_mu = 0;
  int prec_mode = TDCC_PREC_FP64;
  int slices = 5;
  long long tc_min_macs = kTcMinMacs;  // tensor-core routing policy
  int tc_min_k = kTcMinK;
  int tc_min_mn = kTcMinMN;
  int simt_max_k = kSimtMaxKDefault;   // short contractions on the FP32 pipe (mixed mode)
  long long simt_min_macs = kSimtMinMacs;
  int device = 0;
  int nb = 1;                       // trajectories advanced together
  bool share_mem = true;            // workspace slots with disjoint lifetimes share memory (off once
                                    // reverse mode is used: it reads every forward value after a stage)
  long long share_min = -1;         // sharing threshold in bytes (-1: kShareMinBytes)
  int adj_store = -1;               // reverse mode keeps forward intermediates (1), recomputes them
                                    // (0), or keeps them when they fit (-1)
  std::vector<tdcc_field> h_fields; // per-trajectory fields (tdcc_set_fields)
  std::vector<int> h_pol;
  std::unique_ptr<ProgInst> rhs[2][4];
  std::unique_ptr<ProgInst> dens;
  std::unique_ptr<ProgInst> adjp[2][5];  // reverse-mode programs (block 4: density)
  std::vector<int> adj_of[2][5];         // adjoint slot of each forward slot
  std::vector<void*> owned;
  long long ws_bytes = 0;

  // RK4 machinery
  bool rk_ready = false;
  StepCtx* ctx = nullptr;          // device
  tdcc_field* d_fields = nullptr;  // device [nb]
  int* d_pol = nullptr;            // device [nb]
  double2* d_E = nullptr;          // device [nb][3]
  double2* Fs = nullptr;           // 3 x nb x n x n dressed Fock matrices
  double2* kbuf[4] = {};
  double2* acc[4] = {};
  double2* yin[4] = {};
  double2* st[2][4] = {};          // ping-pong state buffers
  double2* res = nullptr;          // dipole components
  cudaStream_t main = nullptr;
  cudaStream_t bs[4] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[4] = {}, ev_user = nullptr;
  // captured step graphs (A->B, B->A)
  cudaGraphExec_t gexec[2] = {};
  int g_method = -1, g_precs = -999, g_prec_mode = -1;
  double g_dt = 0.0;
  double2* g_traj = nullptr;
  bool g_store_set = false;        // the captured graphs write per-step stores
  StepStore g_store{};
  long long g_nodes[2] = {0, 0};   // kernel nodes per captured step graph

  // elements of block b for one trajectory / for all trajectories
  long long nel(int b) const {
    const long long o = dims.o, v = dims.v;
    return (b == TDCC_T1 || b == TDCC_L1) ? o * v : o * o * v * v;
  }
  long long nelb(int b) const { return nel(b) * nb; }
};

namespace {

#define CK(x)                                                                      \
  do {                                                                             \
    cudaError_t e__ = (x);                                                         \
    if (e__ != cudaSuccess) {                                                      \
      throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(e__)); \
    }                                                                              \
  } while (0)

void* dalloc(tdcc_system s, size_t bytes) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error("cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  }
  s->owned.push_back(p);
  s->ws_bytes += (long long)bytes;
  return p;
}

void bind_fixed(tdcc_system s, std::vector<void*>& b) {
  b[S_TEI] = const_cast<double*>(s->tei);
  b[S_MU] = const_cast<double*>(s->mu);
}

ProgInst& get_rhs(tdcc_system s, int method, int block) {
  auto& slot = s->rhs[method][block];
  if (slot) return *slot;
  auto pi = std::make_unique<ProgInst>();
  static const char* names[2][4] = {{"ccsd_t1", "ccsd_t2", "ccsd_l1", "ccsd_l2"},
                                    {"cc2_t1", "cc2_t2", "cc2_l1", "cc2_l2"}};
  pi->prog = std::make_unique<Program>(s->dims, names[method][block]);
  Program& p = *pi->prog;
  if (block == TDCC_T1)
    build_t1(p);
  else if (method == TDCC_CCSD && block == TDCC_T2)
    build_t2_ccsd(p);
  else if (method == TDCC_CCSD && block == TDCC_L1)
    build_l1_ccsd(p);
  else if (method == TDCC_CCSD && block == TDCC_L2)
    build_l2_ccsd(p);
  else if (block == TDCC_T2)
    build_t2_cc2(p);
  else if (block == TDCC_L1)
    build_l1_cc2(p);
  else
    build_l2_cc2(p, p.ones("ones_v", s->dims.v));
  p.batch(s->nb);
  p.select_backend(s->prec_mode, s->tc_min_macs, s->slices, s->tc_min_k, s->tc_min_mn, s->simt_max_k,
                          s->simt_min_macs);
  // the block's own amplitude and the dressed Fock vary across RK4 stages
  p.analyse({S_T1 + block, S_F});
  if (s->share_mem && workspace_estimate(p) > (s->share_min < 0 ? kShareMinBytes : s->share_min)) p.plan_memory();
  pi->bases.assign(p.slots.size(), nullptr);
  pi->bytes = p.allocate(pi->bases, pi->owned);
  s->ws_bytes += pi->bytes;
  bind_fixed(s, pi->bases);
  pi->dag.init(p.ops.size(), 4);
  slot = std::move(pi);
  return *slot;
}

ProgInst& get_density(tdcc_system s) {
  if (s->dens) return *s->dens;
  auto pi = std::make_unique<ProgInst>();
  pi->prog = std::make_unique<Program>(s->dims, "density");
  build_density(*pi->prog, s->n_mu);
  pi->prog->batch(s->nb);
  pi->prog->select_backend(s->prec_mode, s->tc_min_macs, s->slices, s->tc_min_k, s->tc_min_mn, s->simt_max_k,
                          s->simt_min_macs);
  pi->prog->analyse({});
  if (s->share_mem && workspace_estimate(*pi->prog) > (s->share_min < 0 ? kShareMinBytes : s->share_min))
    pi->prog->plan_memory();
  pi->bases.assign(pi->prog->slots.size(), nullptr);
  pi->bytes = pi->prog->allocate(pi->bases, pi->owned);
  s->ws_bytes += pi->bytes;
  bind_fixed(s, pi->bases);
  pi->dag.init(pi->prog->ops.size(), 4);
  s->dens = std::move(pi);
  return *s->dens;
}

void build_program(Program& p, int method, int block, int n_mu, int nb);
struct ActPlan {
  std::vector<int> slot;          // forward slots kept
  std::vector<char> stage;        // 1: one value per stage, 0: one per step
  std::vector<long long> off8;    // offset (8-byte words) in the step's prologue or stage part
  long long pro8 = 0, stage8 = 0; // words of the prologue part and of one stage part
};
ActPlan plan_activations(const Program& adj, size_t nfwd, const Program& fwd);
void reset_programs(tdcc_system s);

// Reverse-mode program of (method, block); block 4 = density.  Its slots
// [0, nfwd) are bound to the forward instance's buffers before every run.
ProgInst& get_adj(tdcc_system s, int method, int block) {
  auto& slot = s->adjp[method][block];
  if (slot) return *slot;
  if (s->share_mem) {  // rebuild the forward programs with a buffer per slot
    reset_programs(s);
    s->share_mem = false;
  }
  if (block == 4)
    get_density(s);
  else
    get_rhs(s, method, block);
  Program f(s->dims, "fwd");
  build_program(f, method, block, s->n_mu, s->nb);
  auto pi = std::make_unique<ProgInst>();
  pi->prog = std::make_unique<Program>(s->dims, "adj");
  build_adjoint(f, *pi->prog, s->adj_of[method][block]);
  pi->prog->select_backend(s->prec_mode, s->tc_min_macs, s->slices, s->tc_min_k, s->tc_min_mn, s->simt_max_k,
                          s->simt_min_macs);
  pi->nfwd = f.slots.size();
  pi->bases.assign(pi->prog->slots.size(), nullptr);
  pi->bytes = pi->prog->allocate(pi->bases, pi->owned, pi->nfwd, true);
  s->ws_bytes += pi->bytes;
  pi->setup_done = true;  // no integral-only ops in a reverse-mode program
  pi->dag.init(pi->prog->ops.size(), 4);
  if (block < 4) {
    const ActPlan ap = plan_activations(*pi->prog, pi->nfwd, *get_rhs(s, method, block).prog);
    pi->act_slot = ap.slot;
    pi->act_stage = ap.stage;
    pi->act_off8 = ap.off8;
    pi->act_pro8 = ap.pro8;
    pi->act_stage8 = ap.stage8;
  }
  slot = std::move(pi);
  return *slot;
}

// The activation record of one RK4 step for reverse mode: the forward slots
// that the reverse-mode program reads and that forward ops write outside the
// integral-only setup.  A slot written by a stage op holds one value per
// stage; the others one per step.  Binding the reverse-mode program to the
// record gives it the values the forward step computed, so it need not run
// the forward ops again.  `nfwd`: the forward slots (the reverse-mode
// program's first slots).
ActPlan plan_activations(const Program& adj, size_t nfwd, const Program& fwd) {
  std::vector<char> rd(nfwd, 0), pro(nfwd, 0), stg(nfwd, 0);
  for (const Op& op : adj.ops)
    for (int r : op.reads)
      if (r >= 0 && r < (int)nfwd) rd[r] = 1;
  for (const Op& op : fwd.ops) {
    if (op.write < 0 || op.write >= (int)nfwd) continue;
    if (Program::in_phase(op, Program::STAGE))
      stg[op.write] = 1;
    else if (Program::in_phase(op, Program::PROLOGUE))
      pro[op.write] = 1;
  }
  ActPlan ap;
  for (int pass = 0; pass < 2; ++pass)
    for (size_t i = 0; i < nfwd; ++i) {
      if (!rd[i] || !(pro[i] || stg[i]) || (pass == 1) != (stg[i] != 0)) continue;
      const SlotInfo& si = fwd.slots[i];
      const long long w = (si.numel * elem_bytes(si.dt) + 7) / 8;
      long long& acc = pass ? ap.stage8 : ap.pro8;
      ap.slot.push_back((int)i);
      ap.stage.push_back((char)pass);
      ap.off8.push_back(acc);
      acc += (w + 31) / 32 * 32;  // 256-byte aligned entries
    }
  return ap;
}

// copies of one phase's activations (stage 0: prologue) into the step store
void store_activations(const StepCtx* ctx, const ProgInst& ai, const ProgInst& pi, const StepStore& ss, int b,
                       int stage, cudaStream_t st) {
  ActTable t{};
  const long long base = stage == 0 ? 0 : ai.act_pro8 + (stage - 1) * ai.act_stage8;
  for (size_t j = 0; j < ai.act_slot.size(); ++j) {
    if ((ai.act_stage[j] != 0) != (stage != 0)) continue;
    const int sl = ai.act_slot[j];
    const SlotInfo& si = pi.prog->slots[sl];
    t.c[t.n++] = {static_cast<const double*>(pi.bases[sl]), base + ai.act_off8[j],
                  (si.numel * elem_bytes(si.dt) + 7) / 8};
    if (t.n == kMaxActCopies) {
      CK(launch_act_store(ctx, t, ss.act[b], ss.act_stride[b], st));
      t.n = 0;
    }
  }
  CK(launch_act_store(ctx, t, ss.act[b], ss.act_stride[b], st));
}

void ensure_rk(tdcc_system s) {
  if (s->rk_ready) return;
  const long long n = s->dims.n;
  s->ctx = static_cast<StepCtx*>(dalloc(s, sizeof(StepCtx)));
  s->d_fields = static_cast<tdcc_field*>(dalloc(s, s->nb * sizeof(tdcc_field)));
  s->d_pol = static_cast<int*>(dalloc(s, s->nb * sizeof(int)));
  s->d_E = static_cast<double2*>(dalloc(s, 3 * s->nb * sizeof(double2)));
  s->Fs = static_cast<double2*>(dalloc(s, 3 * s->nb * n * n * sizeof(double2)));
  for (int b = 0; b < 4; ++b) {
    const size_t bytes = s->nelb(b) * sizeof(double2);
    s->kbuf[b] = static_cast<double2*>(dalloc(s, bytes));
    s->acc[b] = static_cast<double2*>(dalloc(s, bytes));
    s->yin[b] = static_cast<double2*>(dalloc(s, bytes));
    s->st[0][b] = static_cast<double2*>(dalloc(s, bytes));
    s->st[1][b] = static_cast<double2*>(dalloc(s, bytes));
  }
  s->res = static_cast<double2*>(dalloc(s, (size_t)s->nb * s->n_mu * sizeof(double2)));
  CK(cudaStreamCreateWithFlags(&s->main, cudaStreamNonBlocking));
  for (int b = 0; b < 4; ++b) {
    CK(cudaStreamCreateWithFlags(&s->bs[b], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&s->ev_join[b], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&s->ev_user, cudaEventDisableTiming));
  s->rk_ready = true;
}

// Optional per-launch timing (tdcc_profile_step).
struct Prof {
  struct Rec {
    std::string tag;
    int kind, block, stage, backend;
    double flops, bytes;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  void add_prog(const std::vector<Program::Timed>& tm, int block, int stage) {
    for (const auto& t : tm) {
      const Op& op = *t.op;
      const int kind = (op.kind == OP_GEMM || op.kind == OP_TCGEMM) ? 0
                       : (op.kind == OP_ADD || op.kind == OP_PACK) ? 1
                                                                   : 2;
      recs.push_back({op.tag, kind, block, stage, op.backend, (double)op.flops, (double)op.bytes, t.a, t.b});
    }
  }
};

template <class F>
void timed_launch(Prof* pf, cudaStream_t st, const char* tag, int block, int stage, double bytes, F&& fn) {
  if (!pf) {
    CK(fn());
    return;
  }
  Prof::Rec r{tag, 3, block, stage, 0, 0.0, bytes, nullptr, nullptr};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, st);
  CK(fn());
  cudaEventRecord(r.b, st);
  pf->recs.push_back(r);
}

// One RK4 block (ft1/ft2/fL1/fL2): prologue once, four stages, final update.
void run_block(tdcc_system s, int method, int b, double2* const in[4], double2* out_b, double dt,
               int precs, cudaStream_t st, Prof* pf = nullptr, double2* const* store = nullptr,
               const StepStore* ss = nullptr) {
  ProgInst& pi = get_rhs(s, method, b);
  Program& p = *pi.prog;
  auto& B = pi.bases;
  for (int k = 0; k < 4; ++k) B[S_T1 + k] = in[k];
  B[S_OUT] = s->kbuf[b];
  const long long n = s->nelb(b);
  const long long nn = (long long)s->dims.n * s->dims.n * s->nb;  // one stage's dressed Fock matrices
  std::vector<Program::Timed> tm;
  B[S_F] = s->Fs;
  CK(pi.setup(st));
  CK(pi.exec(st, Program::PROLOGUE, pf ? &tm : nullptr));
  if (pf) pf->add_prog(tm, b, 0);
  const ProgInst* act = ss && ss->act[b] ? s->adjp[method][b].get() : nullptr;
  if (act) store_activations(s->ctx, *act, pi, *ss, b, 0, st);
  for (int stage = 1; stage <= 4; ++stage) {
    B[S_T1 + b] = stage == 1 ? in[b] : s->yin[b];
    B[S_F] = s->Fs + (stage == 1 ? 0 : stage < 4 ? 1 : 2) * nn;
    tm.clear();
    CK(pi.exec(st, Program::STAGE, pf ? &tm : nullptr));
    if (pf) pf->add_prog(tm, b, stage);
    if (act) store_activations(s->ctx, *act, pi, *ss, b, stage, st);
    const double h = stage < 3 ? dt / 2.0 : dt;
    timed_launch(pf, st, "rk4_stage_axpy", b, stage, (double)n * 16 * (stage == 1 ? 3 : stage == 4 ? 3 : 5),
                 [&] { return launch_rk4_stage(in[b], s->kbuf[b], s->acc[b], s->yin[b], n, stage, h, st); });
    // the input of stage + 1 (reverse mode recomputes each stage from it)
    if (store && stage < 4)
      CK(cudaMemcpyAsync(store[stage - 1], s->yin[b], n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    if (ss && stage < 4) CK(launch_step_store(s->ctx, s->yin[b], ss->st[b][stage - 1], ss->sst[b], n, st));
  }
  const int sign = (b == TDCC_T1 || b == TDCC_T2) ? -1 : +1;
  const double scale = precs >= 0 ? std::pow(10.0, (double)precs) : 1.0;
  timed_launch(pf, st, "rk4_round_update", b, 4, (double)n * 16 * 3, [&] {
    return launch_rk4_finish(in[b], s->acc[b], out_b, n, dt / 6.0, sign, scale, precs >= 0 ? 1 : 0, st);
  });
}

// Full step on s->main: field, dressing, 4 concurrent blocks, dipole of the
// new state.  `in` and `out` must not alias.  With a profiler everything
// runs serially on s->main.
void run_step(tdcc_system s, int method, double2* const in[4], double2* const out[4], double dt,
              int precs, double2* traj, Prof* pf = nullptr, double2* const* store = nullptr,
              double2* fs_store = nullptr, const StepStore* ss = nullptr) {
  cudaStream_t m = s->main;
  const long long nn = (long long)s->dims.n * s->dims.n;
  timed_launch(pf, m, "advance_field", 5, 0, 0.0, [&] { return launch_advance_field(s->ctx, s->nb, m); });
  timed_launch(pf, m, "dress_fock", 5, 0, (double)nn * (8 + 8 * s->nb + 3 * 16 * s->nb),
               [&] { return launch_dress(s->ctx, s->fock, s->mu, s->Fs, s->dims.n, s->nb, m); });
  if (fs_store)
    CK(cudaMemcpyAsync(fs_store, s->Fs, 3 * (size_t)s->nb * nn * sizeof(double2), cudaMemcpyDeviceToDevice, m));
  if (ss) {
    CK(launch_step_store(s->ctx, s->Fs, ss->fs, ss->sfs, 3 * (long long)s->nb * nn, m));
    for (int b = 0; b < 4; ++b) CK(launch_step_store(s->ctx, in[b], ss->y[b], ss->sy[b], s->nelb(b), m));
  }
  if (pf) {
    for (int b = 0; b < 4; ++b) run_block(s, method, b, in, out[b], dt, precs, m, pf);
  } else {
    CK(cudaEventRecord(s->ev_fork, m));
    for (int b = 0; b < 4; ++b) {
      CK(cudaStreamWaitEvent(s->bs[b], s->ev_fork, 0));
      run_block(s, method, b, in, out[b], dt, precs, s->bs[b], nullptr, store ? store + 3 * b : nullptr, ss);
      CK(cudaEventRecord(s->ev_join[b], s->bs[b]));
    }
    for (int b = 0; b < 4; ++b) CK(cudaStreamWaitEvent(m, s->ev_join[b], 0));
  }
  ProgInst& d = get_density(s);
  for (int k = 0; k < 4; ++k) d.bases[S_T1 + k] = out[k];
  d.bases[S_RES] = s->res;
  std::vector<Program::Timed> tm;
  CK(d.exec(m, Program::ALL, pf ? &tm : nullptr));
  if (pf) pf->add_prog(tm, 4, 0);
  timed_launch(pf, m, "record_mu", 5, 0, 0.0,
               [&] { return launch_record_mu(s->ctx, s->res, s->nb, traj, nullptr, m); });
}

// Time, step counter and the trajectories' fields: `f` for every trajectory
// (along the last dipole component) when given, else the fields of
// tdcc_set_fields, else no field.
void set_ctx(tdcc_system s, double t, double dt, const tdcc_field* f, cudaStream_t st) {
  StepCtx h;
  memset(&h, 0, sizeof(h));
  h.t = t;
  h.dt = dt;
  h.step = 0;
  h.nb = s->nb;
  h.n_mu = s->n_mu;
  h.fields = s->d_fields;
  h.pol = s->d_pol;
  h.E = s->d_E;
  std::vector<tdcc_field> fl(s->nb);
  std::vector<int> pol(s->nb, s->n_mu - 1);
  if (f) {
    for (auto& x : fl) x = *f;
  } else if ((int)s->h_fields.size() == s->nb) {
    fl = s->h_fields;
    pol = s->h_pol;
  } else {
    for (auto& x : fl) {
      memset(&x, 0, sizeof(x));
      x.kind = TDCC_FIELD_NONE;
    }
  }
  CK(cudaMemcpyAsync(s->ctx, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s->d_fields, fl.data(), fl.size() * sizeof(tdcc_field), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s->d_pol, pol.data(), pol.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
}

int fail(int code, const std::string& m) {
  set_error(m);
  return code;
}

// drops the right-hand-side programs (and their workspace) and the captured
// step graphs; they are rebuilt on next use
// Every program instance a system can hold: the right-hand sides, the
// density / dipole program and the reverse-mode programs.  Code that must
// visit all of them (error flags, resets) goes through this one list.
std::vector<std::unique_ptr<ProgInst>*> all_programs(tdcc_system s) {
  std::vector<std::unique_ptr<ProgInst>*> v;
  for (auto& mrow : s->rhs)
    for (auto& pi : mrow) v.push_back(&pi);
  v.push_back(&s->dens);
  for (auto& mrow : s->adjp)
    for (auto& pi : mrow) v.push_back(&pi);
  return v;
}

void reset_programs(tdcc_system s) {
  cudaDeviceSynchronize();
  for (auto* slot : all_programs(s))
    if (*slot) {
      s->ws_bytes -= (*slot)->bytes;
      slot->reset();
    }
  for (auto& g : s->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

bool valid_method(int m) { return m == TDCC_CCSD || m == TDCC_CC2; }

}  // namespace

extern "C" {

int tdcc_version(void) { return 1; }

int tdcc_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return TDCC_ERR_ARG;
  strncpy(buf, g_err.c_str(), len - 1);
  buf[len - 1] = '\0';
  return TDCC_OK;
}

long long tdcc_launch_count(void) { return launch_count(); }

int tdcc_system_create(int o, int v, const double* tei, const double* fock, const double* mu,
                       int n_mu, tdcc_system* out) {
  return tdcc_system_create_batched(o, v, tei, fock, mu, n_mu, 1, out);
}

int tdcc_system_create_batched(int o, int v, const double* tei, const double* fock, const double* mu,
                               int n_mu, int nb, tdcc_system* out) {
  if (!out) return fail(TDCC_ERR_ARG, "out is NULL");
  if (nb < 1 || nb > kMaxTrajectories) return fail(TDCC_ERR_ARG, "nb must be 1..1024");
  *out = nullptr;
  if (o < 1 || v < 1) return fail(TDCC_ERR_ARG, "o and v must be >= 1");
  if ((long long)(o + v) * (o + v) * (o + v) * (o + v) >= (1LL << 40))
    return fail(TDCC_ERR_LIMIT, "n^4 too large");
  if (!tei || !fock || !mu) return fail(TDCC_ERR_ARG, "tei/fock/mu must be device pointers");
  if (n_mu < 1 || n_mu > 3) return fail(TDCC_ERR_ARG, "n_mu must be 1..3");
  auto* s = new tdcc_system_s;
  s->dims = Dims{o, v, o + v};
  s->tei = tei;
  s->fock = fock;
  s->mu = mu;
  s->n_mu = n_mu;
  s->nb = nb;
  cudaGetDevice(&s->device);
  *out = s;
  return TDCC_OK;
}

int tdcc_system_batch(tdcc_system s) { return s ? s->nb : 0; }

int tdcc_set_fields(tdcc_system s, const tdcc_field* fields, const int* pol) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!fields) {
    s->h_fields.clear();
    s->h_pol.clear();
    return TDCC_OK;
  }
  std::vector<int> p(s->nb, s->n_mu - 1);
  for (int b = 0; b < s->nb; ++b) {
    if (fields[b].kind < TDCC_FIELD_NONE || fields[b].kind > TDCC_FIELD_ENVELOPE)
      return fail(TDCC_ERR_ARG, "bad field kind for trajectory " + std::to_string(b));
    if (fields[b].n_env < 0 || fields[b].n_env > TDCC_MAX_ENVELOPE)
      return fail(TDCC_ERR_ARG, "bad envelope size for trajectory " + std::to_string(b));
    if (pol) {
      if (pol[b] < 0 || pol[b] >= s->n_mu) return fail(TDCC_ERR_ARG, "polarisation out of range");
      p[b] = pol[b];
    }
  }
  s->h_fields.assign(fields, fields + s->nb);
  s->h_pol = p;
  return TDCC_OK;
}

int tdcc_system_destroy(tdcc_system s) {
  if (!s) return TDCC_OK;
  cudaDeviceSynchronize();
  for (auto& g : s->gexec)
    if (g) cudaGraphExecDestroy(g);
  if (s->rk_ready) {
    cudaStreamDestroy(s->main);
    for (int b = 0; b < 4; ++b) {
      cudaStreamDestroy(s->bs[b]);
      cudaEventDestroy(s->ev_join[b]);
    }
    cudaEventDestroy(s->ev_fork);
    cudaEventDestroy(s->ev_user);
  }
  for (void* p : s->owned) cudaFree(p);
  delete s;
  return TDCC_OK;
}

int tdcc_set_precision(tdcc_system s, int mode, int slices) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (mode != TDCC_PREC_FP64 && mode != TDCC_PREC_MIXED) return fail(TDCC_ERR_ARG, "bad precision mode");
  if (mode == TDCC_PREC_MIXED && !tc_available())
    return fail(TDCC_ERR_STATE, "tensor-core backend not built into this library");
  if (mode == TDCC_PREC_MIXED && (slices < 2 || slices > 6)) return fail(TDCC_ERR_ARG, "slices must be 2..6");
  if (mode == TDCC_PREC_FP64) slices = s->slices;
  if (mode == s->prec_mode && slices == s->slices) return TDCC_OK;
  reset_programs(s);
  s->prec_mode = mode;
  s->slices = slices;
  return TDCC_OK;
}

int tdcc_set_memory_sharing(tdcc_system s, long long min_bytes) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (min_bytes == s->share_min) return TDCC_OK;
  reset_programs(s);
  s->share_min = min_bytes;
  return TDCC_OK;
}

int tdcc_set_adjoint_store(tdcc_system s, int mode) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (mode < -1 || mode > 1) return fail(TDCC_ERR_ARG, "mode must be -1, 0 or 1");
  s->adj_store = mode;
  return TDCC_OK;
}

int tdcc_set_simt_policy(tdcc_system s, int max_k, long long min_macs) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (max_k < 0 || max_k > 64 || min_macs < 0) return fail(TDCC_ERR_ARG, "0 <= max_k <= 64 and min_macs >= 0 required");
  if (max_k == s->simt_max_k && min_macs == s->simt_min_macs) return TDCC_OK;
  reset_programs(s);
  s->simt_max_k = max_k;
  s->simt_min_macs = min_macs;
  return TDCC_OK;
}

int tdcc_set_tc_policy(tdcc_system s, long long min_macs, int min_k, int min_mn) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (min_macs < 0 || min_k < 1 || min_mn < 1)
    return fail(TDCC_ERR_ARG, "min_macs >= 0, min_k >= 1 and min_mn >= 1 required");
  if (min_macs == s->tc_min_macs && min_k == s->tc_min_k && min_mn == s->tc_min_mn) return TDCC_OK;
  reset_programs(s);
  s->tc_min_macs = min_macs;
  s->tc_min_k = min_k;
  s->tc_min_mn = min_mn;
  return TDCC_OK;
}

int tdcc_ground_state(tdcc_system s, int method, int mode, void* t1, void* t2, void* l1, void* l2,
                      const double* eps_host, int maxsize, int maxiter, double e_min, double r_tol,
                      double* energy, int* niter, void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (mode != 0 && mode != 1) return fail(TDCC_ERR_ARG, "mode must be 0 (T) or 1 (Lambda)");
  if (!t1 || !t2 || (mode == 1 && (!l1 || !l2)) || !eps_host || !energy || !niter)
    return fail(TDCC_ERR_ARG, "NULL argument");
  if (maxsize < 1 || maxsize > 14 || maxiter < 1) return fail(TDCC_ERR_ARG, "need 1 <= maxsize <= 14, maxiter >= 1");
  if (s->nb != 1)
    return fail(TDCC_ERR_STATE, "ground state needs a single-trajectory system (nb = 1) over the same integrals");
  std::vector<void*> mem;
  struct Guard {
    std::vector<void*>& m;
    ~Guard() {
      for (void* p : m) cudaFree(p);
    }
  } guard{mem};
  try {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int o = s->dims.o, v = s->dims.v, n = s->dims.n;
    const long long n1 = (long long)o * v, n2 = n1 * n1;
    auto alloc = [&](size_t bytes) {
      void* p = nullptr;
      CK(cudaMalloc(&p, bytes));
      mem.push_back(p);
      return p;
    };
    auto c2 = [&](long long cnt) { return static_cast<double2*>(alloc((size_t)cnt * sizeof(double2))); };
    double* eps = static_cast<double*>(alloc((size_t)n * sizeof(double)));
    CK(cudaMemcpyAsync(eps, eps_host, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
    double2* Fc = c2((long long)n * n);
    CK(g_to_complex(Fc, s->fock, (long long)n * n, st));
    double2 *r1 = c2(n1), *r2 = c2(n2), *x1 = c2(n1), *x2 = c2(n2), *o1 = c2(n1), *o2 = c2(n2);
    double2* res = c2(64);
    const int ns = maxsize + 2, ne = maxsize + 1;
    std::vector<double2*> S1(ns), S2(ns), E1(ne), E2(ne);
    for (int k = 0; k < ns; ++k) {
      S1[k] = c2(n1);
      S2[k] = c2(n2);
    }
    for (int k = 0; k < ne; ++k) {
      E1[k] = c2(n1);
      E2[k] = c2(n2);
    }
    auto d2d = [&](void* dst, const void* src, long long bytes) {
      CK(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToDevice, st));
    };
    d2d(x1, mode == 0 ? t1 : l1, n1 * 16);
    d2d(x2, mode == 0 ? t2 : l2, n2 * 16);
    ProgInst& P1 = get_rhs(s, method, mode == 0 ? TDCC_T1 : TDCC_L1);
    ProgInst& P2 = get_rhs(s, method, mode == 0 ? TDCC_T2 : TDCC_L2);
    double last_res = INFINITY;
    auto rhs = [&](ProgInst& P, double2* out) {
      auto& B = P.bases;
      B[S_T1] = mode == 0 ? (void*)x1 : t1;
      B[S_T2] = mode == 0 ? (void*)x2 : t2;
      B[S_L1] = mode == 1 ? (void*)x1 : (l1 ? l1 : (void*)x1);
      B[S_L2] = mode == 1 ? (void*)x2 : (l2 ? l2 : (void*)x2);
      B[S_F] = Fc;
      B[S_OUT] = out;
      CK(P.setup(st));
      CK(P.exec(st, Program::DYNAMIC));
    };
    // one Jacobi sweep: both residuals at the current amplitudes, then update
    auto update = [&]() {
      rhs(P1, r1);
      rhs(P2, r2);
      if (r_tol > 0.0) {
        double2 h;
        CK(g_maxabs(r1, n1, r2, n2, res + 63, st));
        CK(cudaMemcpyAsync(&h, res + 63, sizeof(h), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        last_res = h.x;
      }
      CK(g_jacobi(x1, r1, eps, o, v, 2, n1, st));
      CK(g_jacobi(x2, r2, eps, o, v, 4, n2, st));
    };
    auto energy_of = [&]() {
      double2 h[2];
      CK(g_energy(s->tei, s->fock, x1, x2, o, v, mode, res, st));
      CK(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      return h[0].x + h[1].x;
    };
    // buffer bookkeeping for the rolling stores (front = oldest)
    std::vector<int> s1q, s2q, e1q, e2q, s1free, s2free, efree;
    for (int k = ns - 1; k >= 0; --k) {
      s1free.push_back(k);
      s2free.push_back(k);
    }
    for (int k = ne - 1; k >= 0; --k) efree.push_back(k);
    auto take = [](std::vector<int>& fr) {
      const int k = fr.back();
      fr.pop_back();
      return k;
    };
    auto push_s1 = [&](const double2* x) {
      const int k = take(s1free);
      d2d(S1[k], x, n1 * 16);
      s1q.push_back(k);
    };
    auto push_s2 = [&](const double2* x) {
      const int k = take(s2free);
      d2d(S2[k], x, n2 * 16);
      s2q.push_back(k);
    };
    auto push_e = [&](const double2* a1, const double2* b1, const double2* a2, const double2* b2) {
      const int k = take(efree);
      CK(g_sub(E1[k], a1, b1, n1, st));
      CK(g_sub(E2[k], a2, b2, n2, st));
      e1q.push_back(k);
    };
    // (DIIS_solver, CCSD_Helper.py:347-370): first sweep, then maxsize more
    update();
    push_s1(x1);
    push_s2(x2);
    for (int k = 1; k <= maxsize; ++k) {
      update();
      push_s1(x1);
      push_s2(x2);
      push_e(S1[s1q[k]], S1[s1q[k - 1]], S2[s2q[k]], S2[s2q[k - 1]]);
    }
    const int m1 = maxsize + 1;
    std::vector<double> Bm(m1 * m1, -1.0);
    Bm[m1 * m1 - 1] = 0.0;
    const bool early_l1 = (method == TDCC_CC2 && mode == 1);  // CC2_Helper.py:382
    double E = 0.0;
    int it = 0;
    for (int z = 1; z < maxiter; ++z) {
      const double e_old = energy_of();
      // B[a][b] = <e_b, e_a> (t1 part + t2 part), symmetric
      std::vector<std::pair<int, int>> pairs;
      for (int a = 0; a < maxsize; ++a)
        for (int b = a; b < maxsize; ++b) pairs.push_back({a, b});
      for (size_t p0 = 0; p0 < pairs.size(); p0 += 32) {
        DotPairs dp{};
        const size_t cnt = std::min<size_t>(32, pairs.size() - p0);
        for (size_t q = 0; q < cnt; ++q) {
          const int a = pairs[p0 + q].first, b = pairs[p0 + q].second;
          dp.a[2 * q] = E1[e1q[b]];
          dp.b[2 * q] = E1[e1q[a]];
          dp.n[2 * q] = n1;
          dp.a[2 * q + 1] = E2[e1q[b]];
          dp.b[2 * q + 1] = E2[e1q[a]];
          dp.n[2 * q + 1] = n2;
        }
        dp.count = (int)(2 * cnt);
        CK(g_dots(dp, res, st));
        std::vector<double2> h(2 * cnt);
        CK(cudaMemcpyAsync(h.data(), res, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (size_t q = 0; q < cnt; ++q) {
          const int a = pairs[p0 + q].first, b = pairs[p0 + q].second;
          const double val = h[2 * q].x + h[2 * q + 1].x;
          Bm[a * m1 + b] = val;
          Bm[b * m1 + a] = val;
        }
      }
      // solve B c = (0, ..., 0, -1) by Gaussian elimination, partial pivoting
      std::vector<double> M = Bm, rhsv(m1, 0.0);
      rhsv[m1 - 1] = -1.0;
      for (int col = 0; col < m1; ++col) {
        int piv = col;
        for (int r = col + 1; r < m1; ++r)
          if (std::fabs(M[r * m1 + col]) > std::fabs(M[piv * m1 + col])) piv = r;
        if (M[piv * m1 + col] == 0.0) throw std::runtime_error("singular DIIS matrix");
        if (piv != col) {
          for (int c = 0; c < m1; ++c) std::swap(M[col * m1 + c], M[piv * m1 + c]);
          std::swap(rhsv[col], rhsv[piv]);
        }
        for (int r = col + 1; r < m1; ++r) {
          const double f = M[r * m1 + col] / M[col * m1 + col];
          for (int c = col; c < m1; ++c) M[r * m1 + c] -= f * M[col * m1 + c];
          rhsv[r] -= f * rhsv[col];
        }
      }
      std::vector<double> cvec(m1);
      for (int r = m1 - 1; r >= 0; --r) {
        double acc = rhsv[r];
        for (int c = r + 1; c < m1; ++c) acc -= M[r * m1 + c] * cvec[c];
        cvec[r] = acc / M[r * m1 + r];
      }
      // extrapolate x = sum_a c_a stored[a+1]
      std::vector<const double2*> src1, src2;
      std::vector<double> coef;
      for (int a = 0; a < maxsize; ++a) {
        src1.push_back(S1[s1q[a + 1]]);
        src2.push_back(S2[s2q[a + 1]]);
        coef.push_back(cvec[a]);
      }
      CK(g_lincomb(x1, src1, coef, n1, st));
      CK(g_lincomb(x2, src2, coef, n2, st));
      d2d(o1, x1, n1 * 16);
      d2d(o2, x2, n2 * 16);
      E = energy_of();
      ++it;
      if (std::fabs(E - e_old) < e_min) break;
      if (early_l1) {
        push_s1(x1);
        update();
        push_s2(x2);
      } else {
        update();
        push_s1(x1);
        push_s2(x2);
      }
      push_e(x1, o1, x2, o2);
      s1free.push_back(s1q.front());
      s1q.erase(s1q.begin());
      s2free.push_back(s2q.front());
      s2q.erase(s2q.begin());
      efree.push_back(e1q.front());
      e1q.erase(e1q.begin());
      if (r_tol > 0.0 && last_res < r_tol) break;
    }
    d2d(mode == 0 ? t1 : l1, x1, n1 * 16);
    d2d(mode == 0 ? t2 : l2, x2, n2 * 16);
    CK(cudaStreamSynchronize(st));
    *energy = E;
    *niter = it;
  } catch (const std::exception& ex) {
    cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

int tdcc_check_errors(tdcc_system s) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  const cudaError_t ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) return fail(TDCC_ERR_CUDA, std::string("device error: ") + cudaGetErrorString(ce));
  for (auto* slot : all_programs(s)) {
    auto& pi = *slot;
    if (!pi || pi->prog->err_slot < 0) continue;
    int flag = 0;
    void* p = pi->bases[pi->prog->err_slot];
    if (cudaMemcpy(&flag, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(TDCC_ERR_CUDA, "reading the tensor-core error flag failed");
    if (flag) {
      const int zero = 0;
      cudaMemcpy(p, &zero, sizeof(int), cudaMemcpyHostToDevice);
      return fail(TDCC_ERR_CUDA, "tensor-core kernel in " + pi->prog->name + " gave up waiting (code " +
                                     std::to_string(flag) + ")");
    }
  }
  return TDCC_OK;
}

long long tdcc_workspace_bytes(tdcc_system s) { return s ? s->ws_bytes : 0; }

int tdcc_rhs(tdcc_system s, int method, int block, const void* t1, const void* t2, const void* l1,
             const void* l2, const void* F, void* out, void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (block < 0 || block > 3) return fail(TDCC_ERR_ARG, "bad block");
  if (!t1 || !t2 || !F || !out) return fail(TDCC_ERR_ARG, "t1/t2/F/out must not be NULL");
  if (block >= TDCC_L1 && (!l1 || !l2)) return fail(TDCC_ERR_ARG, "Lambda blocks need l1 and l2");
  try {
    ProgInst& pi = get_rhs(s, method, block);
    auto& B = pi.bases;
    B[S_T1] = const_cast<void*>(t1);
    B[S_T2] = const_cast<void*>(t2);
    B[S_L1] = const_cast<void*>(l1);
    B[S_L2] = const_cast<void*>(l2);
    B[S_F] = const_cast<void*>(F);
    B[S_OUT] = out;
    cudaError_t e = pi.setup(static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = pi.exec(static_cast<cudaStream_t>(stream), Program::DYNAMIC);
    if (e != cudaSuccess) return TDCC_ERR_CUDA;
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

int tdcc_dipole(tdcc_system s, const void* t1, const void* t2, const void* l1, const void* l2,
                void* mu_out, void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!t1 || !t2 || !l1 || !l2 || !mu_out) return fail(TDCC_ERR_ARG, "NULL argument");
  try {
    ProgInst& d = get_density(s);
    d.bases[S_T1] = const_cast<void*>(t1);
    d.bases[S_T2] = const_cast<void*>(t2);
    d.bases[S_L1] = const_cast<void*>(l1);
    d.bases[S_L2] = const_cast<void*>(l2);
    d.bases[S_RES] = mu_out;
    if (d.exec(static_cast<cudaStream_t>(stream), Program::ALL) != cudaSuccess)
      return TDCC_ERR_CUDA;
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

int tdcc_rk4_step(tdcc_system s, int method, const void* t1, const void* t2, const void* l1,
                  const void* l2, void* t1_out, void* t2_out, void* l1_out, void* l2_out,
                  double t_prev, double dt, int precs, const tdcc_field* field, void* mu_out,
                  void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (!t1 || !t2 || !l1 || !l2 || !t1_out || !t2_out || !l1_out || !l2_out)
    return fail(TDCC_ERR_ARG, "NULL state pointer");
  if (!(dt > 0.0)) return fail(TDCC_ERR_ARG, "dt must be > 0");
  if (precs > 22) return fail(TDCC_ERR_ARG, "precs must be <= 22 (negative: no rounding)");
  try {
    ensure_rk(s);
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    CK(cudaEventRecord(s->ev_user, user));
    CK(cudaStreamWaitEvent(s->main, s->ev_user, 0));
    set_ctx(s, t_prev, dt, field, s->main);
    double2* in[4] = {(double2*)t1, (double2*)t2, (double2*)l1, (double2*)l2};
    double2* tmp[4] = {s->st[1][0], s->st[1][1], s->st[1][2], s->st[1][3]};
    run_step(s, method, in, tmp, dt, precs, nullptr);
    void* outs[4] = {t1_out, t2_out, l1_out, l2_out};
    for (int b = 0; b < 4; ++b)
      CK(cudaMemcpyAsync(outs[b], tmp[b], s->nelb(b) * sizeof(double2), cudaMemcpyDeviceToDevice, s->main));
    if (mu_out)
      CK(cudaMemcpyAsync(mu_out, s->res, (size_t)s->nb * s->n_mu * sizeof(double2), cudaMemcpyDeviceToDevice,
                         s->main));
    CK(cudaEventRecord(s->ev_user, s->main));
    CK(cudaStreamWaitEvent(user, s->ev_user, 0));
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

}  // extern "C"

namespace {
// tdcc_propagate, optionally copying the state at steps 0, ck_every, 2 ck_every, ...
// (before those steps) into ck[4 * j + block].
int propagate_impl(tdcc_system s, int method, void* t1, void* t2, void* l1, void* l2, double t0, double dt,
                   int nsteps, int precs, const tdcc_field* field, void* mu_traj, void* stream, int ck_every,
                   double2* const* ck, const StepStore* ss = nullptr) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (!t1 || !t2 || !l1 || !l2 || !mu_traj) return fail(TDCC_ERR_ARG, "NULL argument");
  if (nsteps < 0) return fail(TDCC_ERR_ARG, "nsteps < 0");
  if (!(dt > 0.0)) return fail(TDCC_ERR_ARG, "dt must be > 0");
  if (precs > 22) return fail(TDCC_ERR_ARG, "precs must be <= 22");
  try {
    ensure_rk(s);
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    CK(cudaEventRecord(s->ev_user, user));
    CK(cudaStreamWaitEvent(s->main, s->ev_user, 0));
    void* st_user[4] = {t1, t2, l1, l2};
    for (int b = 0; b < 4; ++b)
      CK(cudaMemcpyAsync(s->st[0][b], st_user[b], s->nelb(b) * sizeof(double2), cudaMemcpyDeviceToDevice, s->main));
    set_ctx(s, t0, dt, field, s->main);
    // (re)capture the two ping-pong step graphs when the configuration changed
    if (s->g_method != method || s->g_dt != dt || s->g_precs != precs || s->g_prec_mode != s->prec_mode ||
        s->g_traj != mu_traj || !s->gexec[0] || s->g_store_set != (ss != nullptr) ||
        (ss && memcmp(&s->g_store, ss, sizeof(StepStore)) != 0)) {
      for (auto& g : s->gexec)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
      // build programs (allocations) before capture
      for (int b = 0; b < 4; ++b) CK(get_rhs(s, method, b).setup(s->main));
      CK(cudaStreamSynchronize(s->main));
      get_density(s);
      const long long before_capture = launch_count();
      for (int k = 0; k < 2; ++k) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(s->main, cudaStreamCaptureModeThreadLocal));
        try {
          run_step(s, method, s->st[k], s->st[1 - k], dt, precs, (double2*)mu_traj, nullptr, nullptr, nullptr, ss);
        } catch (...) {
          cudaStreamEndCapture(s->main, &graph);
          throw;
        }
        CK(cudaStreamEndCapture(s->main, &graph));
        size_t nn = 0;
        CK(cudaGraphGetNodes(graph, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
        long long kn = 0;
        for (auto nd : nodes) {
          cudaGraphNodeType ty;
          CK(cudaGraphNodeGetType(nd, &ty));
          if (ty == cudaGraphNodeTypeKernel) ++kn;
        }
        s->g_nodes[k] = kn;
        CK(cudaGraphInstantiate(&s->gexec[k], graph, 0));
        cudaGraphDestroy(graph);
      }
      count_launch(before_capture - launch_count());  // captured, not executed
      s->g_method = method;
      s->g_dt = dt;
      s->g_precs = precs;
      s->g_prec_mode = s->prec_mode;
      s->g_traj = (double2*)mu_traj;
      s->g_store_set = ss != nullptr;
      if (ss) s->g_store = *ss;
    }
    // the step graphs run on the caller's stream, so its events bracket them
    CK(cudaEventRecord(s->ev_user, s->main));
    CK(cudaStreamWaitEvent(user, s->ev_user, 0));
    for (int i = 0; i < nsteps; ++i) {
      if (ck && i % ck_every == 0)
        for (int b = 0; b < 4; ++b)
          CK(cudaMemcpyAsync(ck[4 * (i / ck_every) + b], s->st[i & 1][b], s->nelb(b) * sizeof(double2),
                             cudaMemcpyDeviceToDevice, user));
      CK(cudaGraphLaunch(s->gexec[i & 1], user));
      count_launch(s->g_nodes[i & 1]);
    }
    const int fin = nsteps & 1;
    for (int b = 0; b < 4; ++b)
      CK(cudaMemcpyAsync(st_user[b], s->st[fin][b], s->nelb(b) * sizeof(double2), cudaMemcpyDeviceToDevice, user));
    CK(cudaStreamSynchronize(user));
    if (nsteps > 0) {
      std::vector<double2> last(s->nb);
      CK(cudaMemcpy(last.data(), (double2*)mu_traj + (long long)(nsteps - 1) * s->nb, s->nb * sizeof(double2),
                    cudaMemcpyDeviceToHost));
      for (int b = 0; b < s->nb; ++b)
        if (!std::isfinite(last[b].x) || !std::isfinite(last[b].y))
          return fail(TDCC_ERR_NONFINITE, "dipole of trajectory " + std::to_string(b) +
                                              " is not finite after propagation");
    }
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

}  // namespace

extern "C" {

int tdcc_propagate(tdcc_system s, int method, void* t1, void* t2, void* l1, void* l2, double t0,
                   double dt, int nsteps, int precs, const tdcc_field* field, void* mu_traj,
                   void* stream) {
  return propagate_impl(s, method, t1, t2, l1, l2, t0, dt, nsteps, precs, field, mu_traj, stream, 1, nullptr);
}

int tdcc_autotune(tdcc_system s, int method, const void* t1, const void* t2, const void* l1, const void* l2,
                  int reps, int* n_tuned, double* ms_before, double* ms_after, void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (!t1 || !t2 || !l1 || !l2) return fail(TDCC_ERR_ARG, "NULL state pointer");
  if (reps < 1) reps = 3;
  int tuned = 0;
  double before = 0.0, after = 0.0;
  try {
    ensure_rk(s);
    cudaStream_t user = static_cast<cudaStream_t>(stream), m = s->main;
    CK(cudaEventRecord(s->ev_user, user));
    CK(cudaStreamWaitEvent(m, s->ev_user, 0));
    // one eager step fills every workspace with realistic values
    tdcc_field none;
    memset(&none, 0, sizeof(none));
    none.kind = TDCC_FIELD_NONE;
    set_ctx(s, 0.0, 1e-3, &none, m);
    double2* in[4] = {(double2*)t1, (double2*)t2, (double2*)l1, (double2*)l2};
    double2* tmp[4] = {s->st[1][0], s->st[1][1], s->st[1][2], s->st[1][3]};
    run_step(s, method, in, tmp, 1e-3, -1, nullptr);
    CK(cudaStreamSynchronize(m));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto time_op = [&](ProgInst& pi, const Op& op) {
      CK(pi.prog->launch_op(op, pi.bases, m));  // warm
      CK(cudaEventRecord(e0, m));
      for (int r = 0; r < reps; ++r) CK(pi.prog->launch_op(op, pi.bases, m));
      CK(cudaEventRecord(e1, m));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      return (double)ms / reps;
    };
    std::vector<ProgInst*> progs;
    for (int b = 0; b < 4; ++b) progs.push_back(&get_rhs(s, method, b));
    progs.push_back(&get_density(s));
    for (ProgInst* pip : progs) {
      ProgInst& pi = *pip;
      pi.check_bound();
      for (Op& op : pi.prog->ops) {
        if (op.kind == OP_GEMM && op.backend == GB_FP64) {
          const double t_cur = time_op(pi, op);
          double best = t_cur;
          Op best_op = op;
          for (int tile = 0; tile < kNumTiles; ++tile)
            for (int split = 0; split < 2; ++split) {
              if (!tile_fits(tile, op.g.M)) continue;
              Op c = op;
              Program::plan_gemm(c, split == 1 && op.zeroed, tile);
              if (c.tile == op.tile && c.g.nsplit == op.g.nsplit) continue;
              const double t = time_op(pi, c);
              if (t < best * 0.97) {
                best = t;
                best_op = c;
              }
            }
          before += t_cur;
          after += best;
          if (best_op.tile != op.tile || best_op.g.nsplit != op.g.nsplit) {
            op = best_op;
            ++tuned;
          }
        } else if (op.kind == OP_TCGEMM) {
          const double t_cur = time_op(pi, op);
          double best = t_cur;
          TcArgs best_a = op.tc;
          for (int variant = 0; variant < 4; ++variant) {
            if (variant == 1 && op.tc.S > TcNarrow::STAGES) continue;
            if (variant == 2 && (op.tc.S > TC_TILE128_MAX_S || op.tc.rowsB_pad % TcTile128::BN != 0)) continue;
            if (variant == 3 && op.tc.S > TC_TILE128_MAX_S) continue;
            for (int sp : {0, 1, 2, 3, 4, 6, 8, 12, 16, 24, 32}) {  // 0: the current split
              Op c = op;
              c.tc.variant = variant;
              if (sp > 0) {
                if (!op.zeroed || sp > op.tc.kblocks) continue;
                c.tc.kb_per_split = (c.tc.kblocks + sp - 1) / sp;
                c.tc.nsplit = (c.tc.kblocks + c.tc.kb_per_split - 1) / c.tc.kb_per_split;
                c.tc.atomic = c.tc.nsplit > 1 ? 1 : 0;
                if (c.tc.nsplit == op.tc.nsplit) continue;
                if (!c.tc.atomic && !c.tc.acc) continue;  // plain store needs one writer per element
              }
              // the 128-column and persistent tiles accumulate at most one exact K chunk each
              if ((variant == 2 || variant == 3) && c.tc.kb_per_split > tc_chunk_kblocks(c.tc.S)) continue;
              if (c.tc.variant == op.tc.variant && c.tc.nsplit == op.tc.nsplit) continue;
              const double t = time_op(pi, c);
              if (t < best * 0.97) {
                best = t;
                best_a = c.tc;
              }
            }
          }
          before += t_cur;
          after += best;
          if (best_a.nsplit != op.tc.nsplit || best_a.variant != op.tc.variant) {
            op.tc = best_a;
            ++tuned;
          }
        }
      }
      // tuned ops ran on live workspaces: recompute the per-system constants
      pi.setup_done = false;
      CK(pi.setup(m));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto& g : s->gexec)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    CK(cudaStreamSynchronize(m));
    CK(cudaEventRecord(s->ev_user, m));
    CK(cudaStreamWaitEvent(user, s->ev_user, 0));
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  if (n_tuned) *n_tuned = tuned;
  if (ms_before) *ms_before = before;
  if (ms_after) *ms_after = after;
  return TDCC_OK;
}

int tdcc_adjoint(tdcc_system s, int method, const void* t1, const void* t2, const void* l1, const void* l2,
                 double t0, double dt, int nsteps, int precs, const tdcc_field* field, const double* w_host,
                 int checkpoint, double* J_out, double* gE_host, void* a_t1, void* a_t2, void* a_l1, void* a_l2,
                 void* stream) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (!t1 || !t2 || !l1 || !l2 || !w_host || !J_out || !gE_host) return fail(TDCC_ERR_ARG, "NULL argument");
  if (nsteps < 1 || !(dt > 0.0)) return fail(TDCC_ERR_ARG, "nsteps >= 1 and dt > 0 required");
  if (checkpoint < 1) return fail(TDCC_ERR_ARG, "checkpoint interval must be >= 1");
  if (precs > 22) return fail(TDCC_ERR_ARG, "precs must be <= 22");
  const int K = std::min(checkpoint, nsteps), nseg = (nsteps + K - 1) / K;
  const int nb = s->nb, n_mu = s->n_mu, n = s->dims.n;
  const long long nn = (long long)n * n;
  std::vector<void*> mem;
  struct Guard {
    std::vector<void*>& m;
    ~Guard() {
      cudaDeviceSynchronize();
      for (void* p : m) cudaFree(p);
    }
  } guard{mem};
  auto alloc = [&](size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error("cudaMalloc of " + std::to_string(bytes) + " bytes failed (adjoint)");
    }
    mem.push_back(p);
    return static_cast<double2*>(p);
  };
  try {
    ensure_rk(s);
    for (int b = 0; b < 4; ++b) {
      get_adj(s, method, b);
      CK(get_rhs(s, method, b).setup(s->main));
    }
    get_adj(s, method, 4);
    cudaStream_t user = static_cast<cudaStream_t>(stream), m = s->main;
    CK(cudaEventRecord(s->ev_user, user));
    CK(cudaStreamWaitEvent(m, s->ev_user, 0));
    auto nel = [&](int b) { return (size_t)s->nelb(b); };
    const size_t maxel = nel(1);
    // ---- working memory for the call ----
    // segment store: per step the state, the inputs of stages 2..4 and the
    // dressed Fock matrices, written by the captured step graphs
    std::vector<double2*> ck(4 * nseg), y(4), ay(4);
    if (nseg > 1)
      for (int j = 0; j < nseg; ++j)
        for (int b = 0; b < 4; ++b) ck[4 * j + b] = alloc(nel(b) * 16);
    for (int b = 0; b < 4; ++b) y[b] = alloc(nel(b) * 16);
    StepStore ss{};
    for (int b = 0; b < 4; ++b) {
      ss.sy[b] = ss.sst[b] = (long long)nel(b);
      ss.y[b] = alloc((size_t)(K + 1) * nel(b) * 16);  // + the state after the segment
      for (int q = 0; q < 3; ++q) ss.st[b][q] = alloc((size_t)K * nel(b) * 16);
    }
    ss.sfs = 3LL * nb * nn;
    ss.fs = alloc((size_t)K * ss.sfs * 16);
    // the four blocks' reverse passes run concurrently, each with its own
    // scratch, its contributions to every block's cotangent (summed at the
    // join in block order) and its slice of dJ/dE
    double2 *ak[4][4], *akin[4], *aY[4], *aF[4], *contrib[4][4];
    for (int b = 0; b < 4; ++b) {
      ay[b] = alloc(nel(b) * 16);
      for (int st = 0; st < 4; ++st) ak[b][st] = alloc(maxel * 16);
      akin[b] = alloc(maxel * 16);
      aY[b] = alloc(maxel * 16);
      aF[b] = alloc((size_t)nb * nn * 16);
      for (int q = 0; q < 4; ++q)
        contrib[b][q] = (q == b || s->adj_of[method][b][S_T1 + q] >= 0) ? alloc(nel(q) * 16) : nullptr;
    }
    double2* ares = alloc((size_t)nb * n_mu * 16);
    const size_t gEn = (size_t)nsteps * 4 * nb;  // one block's dJ/dE
    double2* gE = alloc(4 * gEn * 16);
    double2* traj = alloc((size_t)nsteps * nb * 16);
    double2* straj = alloc((size_t)K * nb * 16);
    // activation records (forward intermediates per step) when they fit;
    // otherwise each stage's forward ops run again before its reverse
    bool use_act = false;
    if (s->adj_store != 0) {
      long long act8 = 0;
      for (int b = 0; b < 4; ++b) act8 += get_adj(s, method, b).act_step8();
      size_t fr = 0, tot = 0;
      CK(cudaMemGetInfo(&fr, &tot));
      use_act = s->adj_store == 1 || (double)K * act8 * 8 <= 0.5 * (double)fr;
      for (int b = 0; b < 4 && use_act; ++b) {
        const long long w = get_adj(s, method, b).act_step8();
        ss.act_stride[b] = w;
        ss.act[b] = w ? reinterpret_cast<double*>(alloc((size_t)K * w * 8)) : nullptr;
      }
    }
    CK(cudaMemsetAsync(gE, 0, 4 * gEn * 16, m));
    const void* in[4] = {t1, t2, l1, l2};
    for (int b = 0; b < 4; ++b) CK(cudaMemcpyAsync(y[b], in[b], nel(b) * 16, cudaMemcpyDeviceToDevice, m));
    CK(cudaStreamSynchronize(m));

    // ---- forward on the captured step graphs: one segment keeps every step,
    //      otherwise checkpoints every K steps ----
    const int rc = nseg == 1 ? propagate_impl(s, method, y[0], y[1], y[2], y[3], t0, dt, nsteps, precs, field, traj, m,
                                              1, nullptr, &ss)
                             : propagate_impl(s, method, y[0], y[1], y[2], y[3], t0, dt, nsteps, precs, field, traj, m,
                                              K, ck.data());
    if (rc != TDCC_OK) return rc;
    {
      std::vector<double2> ht((size_t)nsteps * nb);
      CK(cudaMemcpy(ht.data(), traj, ht.size() * 16, cudaMemcpyDeviceToHost));
      for (int b = 0; b < nb; ++b) {
        double J = 0.0;
        for (int i = 0; i < nsteps; ++i) J += w_host[i] * ht[(size_t)i * nb + b].x;
        J_out[b] = J;
      }
    }

    // ---- backward: one captured graph per reverse step (with and without
    //      the objective's dipole term), replayed for every step; it gathers
    //      step k's stored values into fixed buffers, so one graph serves all
    //      steps (k and the global step come from a device counter) ----
    for (int b = 0; b < 4; ++b) CK(cudaMemsetAsync(ay[b], 0, nel(b) * 16, m));
    const double c6 = dt / 6.0;
    const double wst[4] = {1.0, 2.0, 2.0, 1.0};
    const double hst[4] = {0.0, dt / 2.0, dt / 2.0, dt};  // Y(s) = y + h_s k_(s-1)
    double2 *gy[4], *gyn[4], *gst[4][3];
    double* gact[4] = {nullptr, nullptr, nullptr, nullptr};
    GatherTable gt{};
    auto gather = [&](const void* src, long long stride8, long long koff, void* dst, long long n8) {
      if (gt.n == kMaxGather) throw std::runtime_error("reverse step gathers too many buffers");
      gt.c[gt.n++] = {static_cast<const double*>(src), stride8, koff, static_cast<double*>(dst), n8};
    };
    for (int b = 0; b < 4; ++b) {
      const long long w8 = (long long)nel(b) * 2;
      gy[b] = alloc(nel(b) * 16);
      gyn[b] = alloc(nel(b) * 16);
      gather(ss.y[b], ss.sy[b] * 2, 0, gy[b], w8);
      gather(ss.y[b], ss.sy[b] * 2, 1, gyn[b], w8);
      for (int q = 0; q < 3; ++q) {
        gst[b][q] = alloc(nel(b) * 16);
        gather(ss.st[b][q], ss.sst[b] * 2, 0, gst[b][q], w8);
      }
      if (use_act && ss.act[b]) {
        gact[b] = reinterpret_cast<double*>(alloc((size_t)ss.act_stride[b] * 8));
        gather(ss.act[b], ss.act_stride[b], 0, gact[b], ss.act_stride[b]);
      }
    }
    double2* gF = alloc((size_t)ss.sfs * 16);
    gather(ss.fs, ss.sfs * 2, 0, gF, ss.sfs * 2);
    RevCtx* rctx = reinterpret_cast<RevCtx*>(alloc(sizeof(RevCtx)));
    double* wdev = reinterpret_cast<double*>(alloc((size_t)nsteps * 8));
    CK(cudaMemcpyAsync(wdev, w_host, (size_t)nsteps * 8, cudaMemcpyHostToDevice, m));
    const RevCtx rc_h{nsteps - 1, K};
    CK(cudaMemcpyAsync(rctx, &rc_h, sizeof(RevCtx), cudaMemcpyHostToDevice, m));
    CK(cudaStreamSynchronize(m));

    auto reverse_step = [&](bool dipole) {
      CK(launch_rev_gather(rctx, gt, m));
      if (dipole) {  // the objective's dipole term at y_(n+1)
        ProgInst& d = get_density(s);
        ProgInst& ad = get_adj(s, method, 4);
        const auto& aof = s->adj_of[method][4];
        for (int q = 0; q < 4; ++q) d.bases[S_T1 + q] = gyn[q];
        d.bases[S_RES] = s->res;
        CK(d.exec(m, Program::ALL));
        for (size_t i = 0; i < ad.nfwd; ++i) ad.bases[i] = d.bases[i];
        CK(launch_dipole_cotangent(ares, s->d_pol, nb, n_mu, wdev, rctx, m));
        ad.bases[aof[S_RES]] = ares;
        for (int q = 0; q < 4; ++q)
          if (aof[S_T1 + q] >= 0) ad.bases[aof[S_T1 + q]] = ay[q];
        CK(ad.exec(m, Program::ALL));
      }
      // step adjoint: ay (of y_(n+1)) -> ay (of y_n); rounding taken as the
      // identity.  Block b's update reads y_n only, so the four block
      // reverse passes are independent.
      CK(cudaEventRecord(s->ev_fork, m));
      for (int b = 0; b < 4; ++b) {
        cudaStream_t sb = s->bs[b];
        CK(cudaStreamWaitEvent(sb, s->ev_fork, 0));
        ProgInst& pi = get_rhs(s, method, b);
        ProgInst& ai = get_adj(s, method, b);
        const auto& aof = s->adj_of[method][b];
        for (int q = 0; q < 4; ++q)
          if (contrib[b][q]) CK(cudaMemsetAsync(contrib[b][q], 0, nel(q) * 16, sb));
        auto& B = pi.bases;
        for (int q = 0; q < 4; ++q) B[S_T1 + q] = gy[q];
        B[S_OUT] = s->kbuf[b];
        B[S_F] = gF;
        if (!use_act) CK(pi.exec(sb, Program::PROLOGUE));
        // a_k(s) = c w_s a_out, c = -i dt/6 (T) or +i dt/6 (Lambda)
        const double ci = (b == TDCC_T1 || b == TDCC_T2) ? -c6 : c6;
        for (int st = 0; st < 4; ++st) CK(launch_caxpy(ak[b][st], ay[b], nel(b), 0.0, wst[st] * ci, 0, sb));
        for (int st = 4; st >= 1; --st) {
          B[S_T1 + b] = st == 1 ? gy[b] : gst[b][st - 2];
          B[S_F] = gF + (size_t)(st == 1 ? 0 : st < 4 ? 1 : 2) * nb * nn;
          if (!use_act) CK(pi.exec(sb, Program::STAGE));
          for (size_t i = 0; i < ai.nfwd; ++i) ai.bases[i] = B[i];
          if (use_act)
            for (size_t j = 0; j < ai.act_slot.size(); ++j)
              ai.bases[ai.act_slot[j]] =
                  gact[b] + ai.act_off8[j] + (ai.act_stage[j] ? ai.act_pro8 + (st - 1) * ai.act_stage8 : 0);
          CK(cudaMemcpyAsync(akin[b], ak[b][st - 1], nel(b) * 16, cudaMemcpyDeviceToDevice, sb));
          ai.bases[aof[S_OUT]] = akin[b];
          CK(cudaMemsetAsync(aY[b], 0, nel(b) * 16, sb));
          if (aof[S_T1 + b] >= 0) ai.bases[aof[S_T1 + b]] = aY[b];
          if (aof[S_F] >= 0) {
            CK(cudaMemsetAsync(aF[b], 0, (size_t)nb * nn * 16, sb));
            ai.bases[aof[S_F]] = aF[b];
          }
          for (int q = 0; q < 4; ++q)
            if (q != b && aof[S_T1 + q] >= 0) ai.bases[aof[S_T1 + q]] = contrib[b][q];
          CK(ai.exec(sb, Program::STAGE));
          if (aof[S_F] >= 0) CK(launch_field_grad(aF[b], s->mu, s->d_pol, n, nb, gE + b * gEn, rctx, st - 1, sb));
          CK(launch_caxpy(contrib[b][b], aY[b], nel(b), 1.0, 0.0, 1, sb));
          if (st > 1) CK(launch_caxpy(ak[b][st - 2], aY[b], nel(b), hst[st - 1], 0.0, 1, sb));
        }
        CK(ai.exec(sb, Program::PROLOGUE));
        CK(cudaEventRecord(s->ev_join[b], sb));
      }
      for (int b = 0; b < 4; ++b) CK(cudaStreamWaitEvent(m, s->ev_join[b], 0));
      for (int q = 0; q < 4; ++q)
        CK(launch_sum4(ay[q], contrib[0][q], contrib[1][q], contrib[2][q], contrib[3][q], nel(q), m));
      CK(launch_rev_advance(rctx, m));
    };
    struct Graphs {
      cudaGraphExec_t g[2] = {nullptr, nullptr};
      ~Graphs() {
        for (auto x : g)
          if (x) cudaGraphExecDestroy(x);
      }
    } rg;
    bool need[2] = {false, false};
    for (int i = 0; i < nsteps; ++i) need[w_host[i] != 0.0] = true;
    long long per_step[2] = {0, 0};  // kernels per replay
    for (int dip = 0; dip < 2; ++dip) {
      if (!need[dip]) continue;
      const long long before_capture = launch_count();
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(m, cudaStreamCaptureModeThreadLocal));
      try {
        reverse_step(dip != 0);
      } catch (...) {
        cudaStreamEndCapture(m, &graph);
        throw;
      }
      CK(cudaStreamEndCapture(m, &graph));
      CK(cudaGraphInstantiate(&rg.g[dip], graph, 0));
      cudaGraphDestroy(graph);
      per_step[dip] = launch_count() - before_capture;
      count_launch(-per_step[dip]);  // captured, not executed
    }
    for (int j = nseg - 1; j >= 0; --j) {
      const int k0 = j * K, kn = std::min(K, nsteps - k0);
      if (nseg > 1) {
        // recompute the segment on the step graphs, filling the store; y ends
        // as the state after the segment
        double tk = t0;
        for (int i = 0; i < k0; ++i) tk += dt;  // the forward's time accumulation
        for (int b = 0; b < 4; ++b)
          CK(cudaMemcpyAsync(y[b], ck[4 * j + b], nel(b) * 16, cudaMemcpyDeviceToDevice, m));
        const int rs = propagate_impl(s, method, y[0], y[1], y[2], y[3], tk, dt, kn, precs, field, straj, m, 1,
                                      nullptr, &ss);
        if (rs != TDCC_OK) return rs;
      }
      // the state after the segment follows its last stored step
      for (int b = 0; b < 4; ++b)
        CK(cudaMemcpyAsync(ss.y[b] + (size_t)kn * ss.sy[b], y[b], nel(b) * 16, cudaMemcpyDeviceToDevice, m));
      for (int k = kn - 1; k >= 0; --k) {
        const int dip = w_host[k0 + k] != 0.0;
        CK(cudaGraphLaunch(rg.g[dip], m));
        count_launch(per_step[dip]);
      }
    }
    void* aout[4] = {a_t1, a_t2, a_l1, a_l2};
    for (int b = 0; b < 4; ++b)
      if (aout[b]) CK(cudaMemcpyAsync(aout[b], ay[b], nel(b) * 16, cudaMemcpyDeviceToDevice, m));
    std::vector<double2> hg(4 * gEn);
    CK(cudaMemcpyAsync(hg.data(), gE, 4 * gEn * 16, cudaMemcpyDeviceToHost, m));
    CK(cudaStreamSynchronize(m));
    for (size_t i = 0; i < gEn; ++i) {
      double re = 0.0, im = 0.0;
      for (int b = 0; b < 4; ++b) {
        re += hg[b * gEn + i].x;
        im += hg[b * gEn + i].y;
      }
      gE_host[2 * i] = re;
      gE_host[2 * i + 1] = im;
    }
    CK(cudaEventRecord(s->ev_user, m));
    CK(cudaStreamWaitEvent(user, s->ev_user, 0));
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

int tdcc_profile_step(tdcc_system s, int method, const void* t1, const void* t2, const void* l1,
                      const void* l2, double t_prev, double dt, int precs, const tdcc_field* field,
                      tdcc_op_record* recs, int max_recs, int* n_recs) {
  if (!s) return fail(TDCC_ERR_ARG, "null system");
  if (!valid_method(method)) return fail(TDCC_ERR_ARG, "bad method");
  if (!t1 || !t2 || !l1 || !l2 || !recs || !n_recs || max_recs < 0) return fail(TDCC_ERR_ARG, "NULL argument");
  if (!(dt > 0.0)) return fail(TDCC_ERR_ARG, "dt must be > 0");
  Prof pf;
  try {
    ensure_rk(s);
    CK(cudaDeviceSynchronize());
    set_ctx(s, t_prev, dt, field, s->main);
    double2* in[4] = {(double2*)t1, (double2*)t2, (double2*)l1, (double2*)l2};
    double2* tmp[4] = {s->st[1][0], s->st[1][1], s->st[1][2], s->st[1][3]};
    run_step(s, method, in, tmp, dt, precs, nullptr, &pf);
    CK(cudaStreamSynchronize(s->main));
  } catch (const std::exception& ex) {
    for (auto& r : pf.recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  int k = 0;
  for (auto& r : pf.recs) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    if (k < max_recs) {
      tdcc_op_record& o = recs[k];
      memset(&o, 0, sizeof(o));
      strncpy(o.tag, r.tag.c_str(), sizeof(o.tag) - 1);
      o.kind = r.kind;
      o.block = r.block;
      o.stage = r.stage;
      o.backend = r.backend;
      o.flops = r.flops;
      o.bytes = r.bytes;
      o.ms = ms;
    }
    ++k;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  *n_recs = k;
  return TDCC_OK;
}

int tdcc_tei_from_df(const double* B, int n, int nq, double* tei, void* stream) {
  if (!B || !tei) return fail(TDCC_ERR_ARG, "NULL argument");
  if (n < 1 || nq < 1 || (long long)n * n > 0x7fffffffLL) return fail(TDCC_ERR_ARG, "bad sizes");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  try {
    // X[p,q,r,s] = sum_Q B[Q,p,r] B[Q,q,s]: M modes (p, r), N modes (q, s), K = Q
    const long long n2 = (long long)n * n, n3 = n2 * n;
    Op op;
    op.kind = OP_GEMM;
    op.tag = "tei_from_df";
    op.dta = op.dtb = op.dtc = R64;
    GemmArgs& g = op.g;
    g.M = (int)n2;
    g.N = (int)n2;
    g.K = nq;
    g.gm.n = 2;
    g.gm.dim[0] = g.gm.dim[1] = n;
    g.gm.s0[0] = n;
    g.gm.s0[1] = 1;
    g.gm.s1[0] = n3;
    g.gm.s1[1] = n;
    g.gn.n = 2;
    g.gn.dim[0] = g.gn.dim[1] = n;
    g.gn.s0[0] = n;
    g.gn.s0[1] = 1;
    g.gn.s1[0] = n2;
    g.gn.s1[1] = 1;
    g.gk.n = 1;
    g.gk.dim[0] = nq;
    g.gk.s0[0] = n2;
    g.gk.s1[0] = n2;
    g.ar = 1.0;
    g.ai = 0.0;
    g.acc = 0;
    g.nb = 1;
    Program::plan_gemm(op, false);
    CK(launch_gemm(op, B, B, tei, st));
    CK(launch_tei_antisym(tei, n, st));
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

int tdcc_spectrum(const void* mu, long long nsteps, long long stride, double dt, void* Yr, void* Yi,
                  double* energy_ev, void* stream) {
  if (!mu || !Yr || !Yi) return fail(TDCC_ERR_ARG, "NULL argument");
  if (nsteps < 1 || nsteps > 0x7fffffffLL || stride < 1) return fail(TDCC_ERR_ARG, "bad sizes");
  if (!(dt > 0.0)) return fail(TDCC_ERR_ARG, "dt must be > 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  try {
    void* tw = nullptr;
    CK(cudaMallocAsync(&tw, (size_t)nsteps * 16, st));
    const cudaError_t e = launch_spectrum(static_cast<const double2*>(mu), nsteps, stride,
                                          static_cast<double2*>(tw), static_cast<double2*>(Yr),
                                          static_cast<double2*>(Yi), st);
    cudaFreeAsync(tw, st);
    CK(e);
    if (energy_ev)
      for (long long j = 0; j < nsteps; ++j)
        energy_ev[j] = (double)(j - nsteps / 2) / ((double)nsteps * dt) * (2.0 * M_PI) * 27.211;
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// program introspection (no GPU needed)
// ---------------------------------------------------------------------------
namespace {

void build_program(Program& p, int method, int block, int n_mu, int nb = 1) {
  if (block == 4)
    build_density(p, n_mu);
  else if (block == TDCC_T1)
    build_t1(p);
  else if (method == TDCC_CCSD && block == TDCC_T2)
    build_t2_ccsd(p);
  else if (method == TDCC_CCSD && block == TDCC_L1)
    build_l1_ccsd(p);
  else if (method == TDCC_CCSD && block == TDCC_L2)
    build_l2_ccsd(p);
  else if (block == TDCC_T2)
    build_t2_cc2(p);
  else if (block == TDCC_L1)
    build_l1_cc2(p);
  else
    build_l2_cc2(p, p.ones("ones_v", p.dims.v));
  p.batch(nb);
  if (block == 4)
    p.analyse({});
  else
    p.analyse({S_T1 + block, S_F});
  p.plan_memory();  // introspection shows the buffer sharing the runtime uses
}

std::string jarr(const long long* x, int n) {
  std::string s = "[";
  for (int i = 0; i < n; ++i) s += (i ? "," : "") + std::to_string(x[i]);
  return s + "]";
}
std::string jarr(const int* x, int n) {
  std::string s = "[";
  for (int i = 0; i < n; ++i) s += (i ? "," : "") + std::to_string(x[i]);
  return s + "]";
}
std::string jnum(double x) {
  char b[64];
  snprintf(b, sizeof(b), "%.17g", x);
  return b;
}
std::string jgroup(const ModeGroup& g) {
  return "{\"n\":" + std::to_string(g.n) + ",\"dim\":" + jarr(g.dim, g.n) + ",\"s0\":" + jarr(g.s0, g.n) +
         ",\"s1\":" + jarr(g.s1, g.n) + "}";
}

std::string program_json(const Program& p) {
  std::string j = "{\"name\":\"" + p.name + "\",\"slots\":[";
  for (size_t i = 0; i < p.slots.size(); ++i) {
    const auto& s = p.slots[i];
    j += (i ? "," : "") + std::string("{\"name\":\"") + s.name + "\",\"dt\":" + std::to_string(s.dt) +
         ",\"numel\":" + std::to_string(s.numel) + ",\"numel1\":" + std::to_string(s.numel1) +
         ",\"buf\":" + std::to_string(i < p.slot_buf.size() ? p.slot_buf[i] : (int)i) +
         ",\"batched\":" + (s.batched ? "true" : "false") + ",\"fixed\":" + (s.fixed ? "true" : "false") +
         ",\"ones\":" + (s.init.empty() ? "false" : "true") + "}";
  }
  j += "],\"ops\":[";
  for (size_t i = 0; i < p.ops.size(); ++i) {
    const Op& op = p.ops[i];
    j += i ? "," : "";
    // phase flags, then the slots the op reads and writes (dependency analysis)
    const std::string var = std::string(op.varying ? "true" : "false") + ",\"const\":" +
                            (op.is_const ? "true" : "false") + ",\"reads\":" +
                            jarr(op.reads.data(), (int)op.reads.size()) + ",\"write\":" + std::to_string(op.write);
    if (op.kind == OP_GEMM) {
      const GemmArgs& g = op.g;
      j += "{\"kind\":\"gemm\",\"tag\":\"" + op.tag + "\",\"varying\":" + var +
           ",\"sa\":" + std::to_string(op.sa) + ",\"oa\":" + std::to_string(op.oa) + ",\"dta\":" + std::to_string(op.dta) +
           ",\"sb\":" + std::to_string(op.sb) + ",\"ob\":" + std::to_string(op.ob) + ",\"dtb\":" + std::to_string(op.dtb) +
           ",\"sc\":" + std::to_string(op.sc) + ",\"oc\":" + std::to_string(op.oc) + ",\"dtc\":" + std::to_string(op.dtc) +
           ",\"M\":" + std::to_string(g.M) + ",\"N\":" + std::to_string(g.N) + ",\"K\":" + std::to_string(g.K) +
           ",\"gm\":" + jgroup(g.gm) + ",\"gn\":" + jgroup(g.gn) + ",\"gk\":" + jgroup(g.gk) +
           ",\"ar\":" + jnum(g.ar) + ",\"ai\":" + jnum(g.ai) + ",\"acc\":" + std::to_string(g.acc) +
           ",\"atomic\":" + std::to_string(g.atomic) + ",\"nsplit\":" + std::to_string(g.nsplit) +
           ",\"kchunk\":" + std::to_string(g.kchunk) + ",\"nb\":" + std::to_string(g.nb) +
           ",\"bsA\":" + std::to_string(g.bsA) + ",\"bsB\":" + std::to_string(g.bsB) +
           ",\"bsC\":" + std::to_string(g.bsC) + ",\"flops\":" + std::to_string(op.flops) + "}";
    } else if (op.kind == OP_ADD) {
      const AddArgs& a = op.a;
      j += "{\"kind\":\"add\",\"varying\":" + var + ",\"sc\":" + std::to_string(op.add_sc) +
           ",\"oc\":" + std::to_string(op.add_oc) + ",\"cc\":" + std::to_string(a.cc) +
           ",\"acc\":" + std::to_string(a.acc) + ",\"d\":" + jarr(a.d, a.nd) + ",\"sC\":" + jarr(a.sC, a.nd) +
           ",\"terms\":[";
      for (int t = 0; t < a.nt; ++t) {
        const AddTerm& T = a.t[t];
        j += (t ? "," : "") + std::string("{\"sa\":") + std::to_string(op.add_slots[t][0]) +
             ",\"oa\":" + std::to_string(op.add_off[t][0]) + ",\"ac\":" + std::to_string(T.ac) +
             ",\"sA\":" + jarr(T.sA, a.nd) + ",\"sb\":" + std::to_string(op.add_slots[t][1]) +
             ",\"ob\":" + std::to_string(op.add_off[t][1]) + ",\"bc\":" + std::to_string(T.bc) +
             ",\"sB\":" + jarr(T.sB, a.nd) + ",\"cr\":" + jnum(T.cr) + ",\"ci\":" + jnum(T.ci) + "}";
      }
      j += "]}";
    } else if (op.kind == OP_REDUCE) {
      const ReduceArgs& r = op.rd;
      j += "{\"kind\":\"reduce\",\"tag\":\"" + op.tag + "\",\"varying\":" + var +
           ",\"out\":" + std::to_string(op.rd_out) + ",\"oout\":" + std::to_string(op.rd_oout) +
           ",\"x\":" + std::to_string(op.rd_x) + ",\"ox\":" + std::to_string(op.rd_ox) +
           ",\"y\":" + std::to_string(op.rd_y) + ",\"oy\":" + std::to_string(op.rd_oy) +
           ",\"ycplx\":" + std::to_string(r.ycplx) + ",\"dout\":" + jarr(r.dout, r.no) +
           ",\"dred\":" + jarr(r.dred, r.nr) + ",\"so_out\":" + jarr(r.so_out, r.no) +
           ",\"so_x\":" + jarr(r.so_x, r.no) + ",\"so_y\":" + jarr(r.so_y, r.no) +
           ",\"sr_x\":" + jarr(r.sr_x, r.nr) + ",\"sr_y\":" + jarr(r.sr_y, r.nr) +
           ",\"cr\":" + jnum(r.cr) + ",\"ci\":" + jnum(r.ci) + ",\"acc\":" + std::to_string(r.acc) + "}";
    } else {
      j += "{\"kind\":\"trace\",\"varying\":" + var + ",\"slots\":" + jarr(op.tr_slots, 4) +
           ",\"n_mu\":" + std::to_string(op.tr_n_mu) + ",\"nb\":" + std::to_string(op.tr_nb) +
           ",\"bs\":" + jarr(op.tr_bs, 4) + ",\"bsres\":" + std::to_string(op.tr_bsres) + "}";
    }
  }
  return j + "]}";
}

}  // namespace

extern "C" long long tdcc_adjoint_program_json(int o, int v, int method, int block, int n_mu, int nb, char* buf,
                                               size_t len) {
  if (o < 1 || v < 1 || !valid_method(method) || block < 0 || block > 4 || n_mu < 1 || n_mu > 3 || nb < 1)
    return fail(TDCC_ERR_ARG, "bad arguments");
  try {
    Program p(Dims{o, v, o + v}, "introspect");
    build_program(p, method, block, n_mu, nb);
    Program a(p.dims, "introspect_adj");
    std::vector<int> adj_of;
    build_adjoint(p, a, adj_of);
    std::string j = program_json(a);
    j.pop_back();  // '}'
    j += ",\"nfwd\":" + std::to_string(p.slots.size()) + ",\"adj_of\":" + jarr(adj_of.data(), (int)adj_of.size());
    if (block < 4) {  // the activation record the step graph keeps for this program
      const ActPlan ap = plan_activations(a, p.slots.size(), p);
      std::vector<int> st(ap.stage.begin(), ap.stage.end());
      j += ",\"act\":{\"pro8\":" + std::to_string(ap.pro8) + ",\"stage8\":" + std::to_string(ap.stage8) +
           ",\"slots\":" + jarr(ap.slot.data(), (int)ap.slot.size()) + ",\"stage\":" +
           jarr(st.data(), (int)st.size()) + ",\"off8\":" + jarr(ap.off8.data(), (int)ap.off8.size()) + "}";
    }
    j += "}";
    if (!buf || len < j.size() + 1) return fail(TDCC_ERR_LIMIT, "buffer too small: need " + std::to_string(j.size() + 1));
    memcpy(buf, j.c_str(), j.size() + 1);
    return (long long)j.size();
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_ARG, ex.what());
  }
}

extern "C" long long tdcc_program_json(int o, int v, int method, int block, int n_mu, int nb, char* buf,
                                       size_t len) {
  if (o < 1 || v < 1 || !valid_method(method) || block < 0 || block > 4 || n_mu < 1 || n_mu > 3 || nb < 1)
    return fail(TDCC_ERR_ARG, "bad arguments");
  try {
    Program p(Dims{o, v, o + v}, "introspect");
    build_program(p, method, block, n_mu, nb);
    const std::string j = program_json(p);
    if (!buf || len < j.size() + 1) return fail(TDCC_ERR_LIMIT, "buffer too small: need " + std::to_string(j.size() + 1));
    memcpy(buf, j.c_str(), j.size() + 1);
    return (long long)j.size();
  } catch (const std::exception& ex) {
    return fail(TDCC_ERR_ARG, ex.what());
  }
}
