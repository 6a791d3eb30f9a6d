// Internal engine of libtdcc.so: strided tensor views, the contraction /
// elementwise op records, and "programs" (ordered op lists with symbolic
// buffer slots) that the residual builders emit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace tdcc {

enum DType : int { R64 = 0, C64 = 1, U8 = 2 };

inline long long elem_bytes(int dt) { return dt == C64 ? 16 : dt == R64 ? 8 : 1; }

// ---------------------------------------------------------------------------
// Kernel argument blocks (passed by value to the kernels)
// ---------------------------------------------------------------------------
constexpr int kMaxModes = 4;

// A group of tensor modes flattened into one GEMM dimension.  s0/s1 are the
// element strides of each mode in the two tensors that carry the group
// (M: A and C, N: B and C, K: A and B).  The last mode varies fastest.
struct ModeGroup {
  int n;
  int dim[kMaxModes];
  long long s0[kMaxModes];
  long long s1[kMaxModes];
};

struct GemmArgs {
  const void* A;
  const void* B;
  void* C;
  int M, N, K;
  ModeGroup gm, gn, gk;
  double ar, ai;   // alpha
  int acc;         // C += alpha*AB (else C = alpha*AB)
  int kchunk;      // K range per split
  int atomic;      // split-K: accumulate with atomics (C pre-initialised)
  int nsplit;      // K splits; blockIdx.z = batch * nsplit + split
  int nb;          // batch count (independent products, one per trajectory)
  long long bsA, bsB, bsC;  // batch strides in elements (0: shared operand)
};

constexpr int kMaxAddTerms = 6;
constexpr int kAddDims = 6;

struct AddTerm {
  const void* A;   // never null
  const void* B;   // optional second factor (elementwise product), may be null
  long long sA[kAddDims];
  long long sB[kAddDims];
  int ac, bc;      // A / B complex?
  double cr, ci;   // coefficient
};

// Elementwise iteration space: nd dimensions (last fastest), merged where
// every operand is contiguous across neighbours.
struct AddArgs {
  void* C;
  int nd;
  long long sC[kAddDims];
  int d[kAddDims];
  long long total;
  int cc;          // C complex?
  int acc;         // C += sum (else C = sum)
  int nt;
  AddTerm t[kMaxAddTerms];
};

// ---------------------------------------------------------------------------
// Views and programs
// ---------------------------------------------------------------------------
// Fixed slots bound by the caller of a program at run time.
enum Slot : int {
  S_TEI = 0,   // R64 [n,n,n,n]
  S_F,         // C64 [n,n]  dressed Fock of the stage
  S_T1, S_T2, S_L1, S_L2,  // C64 amplitudes
  S_OUT,       // C64 residual output
  S_MU,        // R64 [n_mu,n,n]
  S_RES,       // C64 small result vector (dipole components)
  kNumFixedSlots
};

struct View {
  int slot = -1;
  long long off = 0;
  int dt = C64;
  int nd = 0;
  int d[4] = {1, 1, 1, 1};
  long long s[4] = {0, 0, 0, 0};

  View swap(int a, int b) const {
    View r = *this;
    std::swap(r.d[a], r.d[b]);
    std::swap(r.s[a], r.s[b]);
    return r;
  }
  long long numel() const {
    long long x = 1;
    for (int i = 0; i < nd; ++i) x *= d[i];
    return x;
  }
};

struct Term {
  double cr = 1.0, ci = 0.0;
  View A;
  View B;  // slot -1: absent
};

enum OpKind { OP_GEMM = 0, OP_ADD = 1, OP_TRACE = 2, OP_PACK = 3, OP_TCGEMM = 4, OP_REDUCE = 5 };

// out[o] (+)= c * sum_r X[o, r] (* Y[o, r]) over strided index spaces: the
// adjoint of an elementwise term whose operand is broadcast (outer products,
// scaled rows).  Complex X and out; Y complex or real, or absent.
constexpr int kRedDims = 6;
struct ReduceArgs {
  void* out;
  const void* X;
  const void* Y;
  int no, nr;                 // output / reduction dimensions
  int dout[kRedDims], dred[kRedDims];
  long long so_out[kRedDims], so_x[kRedDims], so_y[kRedDims];  // strides of the output dims
  long long sr_x[kRedDims], sr_y[kRedDims];                    // strides of the reduction dims
  long long nout, nred;
  int ycplx;
  double cr, ci;
  int acc;
};

// Tensor-core backend argument blocks (gemm_tc.cu).
struct PackArgs {
  const void* src;   // FP64 tensor (real or interleaved complex)
  int cplx;
  ModeGroup gr;      // row modes, strides in s0 (elements of src)
  ModeGroup gk;      // K modes, strides in s0
  int rows;          // logical rows (M or N) per batch
  int K;
  int rows_pad;      // packed rows per batch (x2 for complex), multiple of the tile
  int K_pad;         // multiple of the K tile
  int S;             // slices
  int nb;            // batches: packed rows of batch z start at z * rows_pad
  long long bs;      // batch stride of src in elements
  void* out;         // [S][nb * rows_pad][K_pad] BF16
  int* exps;         // [nb * rows_pad]
};

struct TcArgs {
  int M, N;                 // logical output extents (per batch)
  int rowsA_pad, rowsB_pad; // packed rows per batch
  int nb, nsplit;           // blockIdx.z = batch * nsplit + split
  int variant;              // 0: 64-wide tile, one CTA per SM; 1: 32-wide, two per SM; 2: 128-wide; 3: persistent 64-wide
  int m_fast;               // launch order: M tiles fastest (set by the launcher)
  int bat_a, bat_b;         // A / B packed per batch (else shared by all batches)
  long long bsC;            // output batch stride in elements
  int kblocks, kb_per_split;
  int S;
  int tmem_cols;
  int ac, bc, cc;           // A, B, C complex?
  const int* expA;
  const int* expB;
  ModeGroup gmC, gnC;       // output offsets: strides in s0
  void* C;
  double ar, ai;
  int alpha_pow2;           // alpha = (-1)^alpha_neg 2^alpha_e exactly (folded into exponents)
  int alpha_e, alpha_neg;
  int acc, atomic;
  int* err;
};

// GB_SIMT: exact BF16-digit slice products on the FP32 pipe for short
// contractions of the mixed mode (gemm_tc.cu)
enum GemmBackend { GB_FP64 = 0, GB_TC = 1, GB_SIMT = 2 };

struct Op {
  OpKind kind;
  std::string tag;
  // GEMM
  int sa = -1, sb = -1, sc = -1;
  long long oa = 0, ob = 0, oc = 0;
  int dta = C64, dtb = C64, dtc = C64;
  GemmArgs g{};
  int backend = GB_FP64;
  int tile = 0;            // FP64 tile shape index (kTiles)
  bool zeroed = false;     // C is zeroed (or accumulated into) before: split-K allowed
  long long flops = 0;     // real flops of this contraction
  long long bytes = 0;     // compulsory bytes read + written
  // ADD
  AddArgs a{};
  int add_slots[kMaxAddTerms][2];
  long long add_off[kMaxAddTerms][2];
  int add_sc = -1;
  long long add_oc = 0;
  // TRACE: res[k] = sum over 4 density blocks of mu_k * rho (see kernels)
  int tr_slots[4];
  int tr_n_mu = 0;
  int tr_nb = 1;           // trajectories; strides of the four density blocks and of res
  long long tr_bs[4] = {0, 0, 0, 0};
  long long tr_bsres = 0;
  // PACK: operand slot/offset/type -> packed slot (exponents at pk_exp_off bytes)
  PackArgs pk{};
  int pk_src = -1, pk_dt = R64, pk_dst = -1;
  long long pk_off = 0, pk_exp_off = 0;
  // REDUCE: out / X / Y slots and offsets
  ReduceArgs rd{};
  int rd_out = -1, rd_x = -1, rd_y = -1;
  long long rd_oout = 0, rd_ox = 0, rd_oy = 0;
  // TCGEMM: packed A / B slots, output C, error-flag slot
  TcArgs tc{};
  int tc_pa = -1, tc_pb = -1, tc_err = -1;
  long long tc_expa_off = 0, tc_expb_off = 0;
  // dependency analysis
  std::vector<int> reads;
  int write = -1;
  bool varying = true;
  bool is_const = false;   // depends on the integrals only: run once per system
};

struct SlotInfo {
  std::string name;
  int dt;
  long long numel;           // all trajectories (numel1 * nb when batched)
  bool fixed;
  std::vector<double> init;  // uploaded at allocation (constant slots)
  bool batched = false;      // one copy per trajectory, [nb][numel1]
  long long numel1 = 0;      // elements of one copy (the batch stride)
};

struct Dims {  // system sizes
  int o, v, n;
};

// Streams and per-op events for executing a program as a dependency DAG.
struct DagExec {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> ev;     // one per op
  std::vector<cudaEvent_t> tails;  // one per stream (join)
  cudaEvent_t fork = nullptr;
  void init(size_t nops, int nstreams);
  void destroy();
};

class Program {
 public:
  Program(Dims dims, std::string name);

  Dims dims;
  std::string name;
  std::vector<SlotInfo> slots;
  std::vector<Op> ops;
  long long flops_total = 0;

  // views of fixed slots
  View G(const char* blk) const;             // TEI block, e.g. "oovv"
  View Fb(const char* blk) const;            // dressed Fock block "ov"
  View amp(int slot) const;                  // T1/T2/L1/L2 view
  View out(int nd);                          // output view (o,v) or (o,o,v,v)

  // workspace tensor of the given shape ('o'/'v' letters), contiguous
  View ws(const std::string& nm, const char* shape, int dt = C64);
  View ws_dims(const std::string& nm, int nd, const int* d, int dt = C64);
  // constant real vector of ones of length `len` (column sums via GEMM)
  View ones(const std::string& nm, int len);

  // C (+)= alpha * einsum(spec, A, B)
  void ein(const char* spec, double ar, double ai, const View& A, const View& B,
           const View& C, bool acc);
  void ein(const char* spec, double alpha, const View& A, const View& B, const View& C,
           bool acc) {
    ein(spec, alpha, 0.0, A, B, C, acc);
  }
  // C (+)= sum_t coef_t * A_t (* B_t); all term views have C's dims
  void add(const View& C, bool acc, const std::vector<Term>& terms);
  void copy(const View& C, const View& A, double c = 1.0) { add(C, false, {Term{c, 0.0, A, View{}}}); }
  void zero(const View& C) { add(C, false, {}); }
  void trace(int n_mu, const View& Dij, const View& L1, const View& Dai, const View& Dab);

  // antisymmetrisers applied while accumulating X into C
  void acc_pij(const View& C, const View& X, double c = 1.0);     // C += c(X - X^(ij))
  void acc_pab(const View& C, const View& X, double c = 1.0);     // C += c(X - X^(ab))
  void acc_pijab(const View& C, const View& X, double c = 1.0);   // C += c P(ij)P(ab) X

  // broadcast view: x with index string `from` seen with the indices `to`
  static View bc(const View& x, const char* from, const char* to);

  // marks ops that (transitively) read one of the varying slots
  void analyse(const std::vector<int>& varying_slots);

  // Runs the program for nb trajectories at once (before select_backend):
  // slots that depend on the per-trajectory inputs (F, amplitudes, output,
  // result) get nb copies, [nb][numel]; contractions with one shared operand
  // fold the trajectory index into M or N, the others become batched
  // products; elementwise ops gain an outer trajectory dimension.
  void batch(int nb);
  int nb = 1;
  long long bstride(int slot) const { return slots[slot].batched ? slots[slot].numel1 : 0; }
  // tile shape and split-K of a contraction from its extents
  static void plan_gemm(Op& op, bool allow_split, int tile = -1);

  // shares memory between workspace slots with disjoint lifetimes within one
  // phase (after analyse; before allocate); without it every slot is its own
  void plan_memory(size_t first = 0);
  std::vector<int> slot_buf;              // buffer (representative slot) of each slot
  std::map<int, int> pool_of;             // slot -> shared buffer index
  std::vector<int> buf_slot;              // shared buffer -> its first slot
  std::vector<size_t> pool_bytes;
  // device allocation of the non-fixed slots from index `first` on (returns
  // bytes allocated); `zero`: clear them (accumulators of adjoint programs)
  long long allocate(std::vector<void*>& bases, std::vector<void*>& owned, size_t first = 0, bool zero = false);

  // ALL: every op.  SETUP: ops that depend on the integrals only (once per
  // system).  PROLOGUE: the rest of the ops independent of the varying
  // slots (once per RK4 step).  STAGE: ops on the varying slots.  DYNAMIC:
  // every op except SETUP ones.
  enum Phase { ALL = 0, PROLOGUE = 1, STAGE = 2, SETUP = 3, DYNAMIC = 4 };
  // `timed`, when given, receives (op, start event, stop event) per launch;
  // the caller synchronises and destroys the events.
  struct Timed {
    const Op* op;
    cudaEvent_t a, b;
  };
  cudaError_t run(const std::vector<void*>& bases, cudaStream_t st, Phase ph,
                  std::vector<Timed>* timed = nullptr) const;
  // same ops, issued as a DAG over `ex`'s streams (slot hazards become
  // event edges) and joined back into `st`
  cudaError_t run_dag(const std::vector<void*>& bases, cudaStream_t st, Phase ph, DagExec& ex) const;
  cudaError_t launch_op(const Op& op, const std::vector<void*>& bases, cudaStream_t st) const;
  static bool in_phase(const Op& op, Phase ph);

  // mixed precision: which GEMMs go to the tensor-core backend
  // (before analyse/allocate) rewrites every contraction with at least
  // `min_macs` multiply-adds, K >= min_k and M, N >= min_mn into pack A, pack B and a
  // tensor-core slice product with `slices` BF16 slices per operand
  // contractions left out with K <= simt_max_k and at least simt_min_macs
  // multiply-adds run as slice products on the FP32 pipe (GB_SIMT)
  void select_backend(int prec_mode, long long min_macs, int slices, int min_k, int min_mn, int simt_max_k,
                      long long simt_min_macs);
  int err_slot = -1;  // U8 slot holding the tensor-core kernels' error flag
};

// merges contiguous dimensions of an elementwise op (program.cpp)
void coalesce(AddArgs& a);

// Reverse-mode (vector-Jacobian product) program of `f` (adjoint.cpp).
// `f` must be batched and analysed but not yet backend-selected.  The
// adjoint program shares f's slots [0, f.slots.size()) (bound to the same
// memory) and adds one adjoint slot per differentiable slot; adj_of[s] is
// the adjoint slot of forward slot s (-1: not differentiable).  Adjoints are
// carried conjugated (a = conj(dJ/dRe z + i dJ/dIm z)), so every op of the
// holomorphic equations maps to plain transposed products.  Each generated
// op inherits the varying / constant flags of the forward op it reverses.
void build_adjoint(const Program& f, Program& a, std::vector<int>& adj_of);

// FP64 contraction tile shapes (kernels.cu)
constexpr int kNumTiles = 7;
extern const int kTiles[kNumTiles][2];
int choose_tile(long long M, long long N);
bool tile_fits(int tile, long long M);  // the M tiles fit the launch grid

// kernel launchers (kernels.cu)
cudaError_t launch_gemm(const Op& op, const void* A, const void* B, void* C, cudaStream_t st);
cudaError_t launch_pack(const PackArgs& p, cudaStream_t st);
cudaError_t launch_ozaki(const TcArgs& a, const void* packA, const void* packB, cudaStream_t st);
bool simt_slices_supported(int K, int S);
cudaError_t launch_simt_slices(const Op& op, const void* A, const void* B, void* C, cudaStream_t st);
bool tc_available();
cudaError_t launch_add(const AddArgs& a, cudaStream_t st);
cudaError_t launch_reduce(const ReduceArgs& r, cudaStream_t st);
cudaError_t launch_trace(int n, int o, int n_mu, const double* mu, const void* dij,
                         const void* l1, const void* dai, const void* dab, void* res, int nb,
                         const long long* bs, long long bsres, cudaStream_t st);
void count_launch(long long k = 1);
long long launch_count();

// error reporting (capi.cpp)
void set_error(const std::string& msg);

}  // namespace tdcc
