// Programs: ordered op lists over symbolic buffer slots.  The einsum planner
// turns "mnef,mnaf->ae" on strided views into a GEMM over flattened mode
// groups (no permute copies); `analyse` splits a program into a prologue
// (ops independent of the RK4 block's varying inputs, run once per step)
// and the per-stage body.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>

#include "engine.h"
#include "gemm_tc.h"

namespace tdcc {

Program::Program(Dims d, std::string nm) : dims(d), name(std::move(nm)) {
  const long long n = d.n, o = d.o, v = d.v;
  slots.resize(kNumFixedSlots);
  slots[S_TEI] = {"tei", R64, n * n * n * n, true};
  slots[S_F] = {"F", C64, n * n, true};
  slots[S_T1] = {"t1", C64, o * v, true};
  slots[S_T2] = {"t2", C64, o * o * v * v, true};
  slots[S_L1] = {"l1", C64, o * v, true};
  slots[S_L2] = {"l2", C64, o * o * v * v, true};
  slots[S_OUT] = {"out", C64, o * o * v * v, true};
  slots[S_MU] = {"mu", R64, 3 * n * n, true};
  slots[S_RES] = {"res", C64, 3, true};
}

static int extent(const Dims& d, char c) {
  if (c == 'o') return d.o;
  if (c == 'v') return d.v;
  throw std::runtime_error(std::string("bad block letter ") + c);
}

View Program::G(const char* blk) const {
  View x;
  x.slot = S_TEI;
  x.dt = R64;
  x.nd = 4;
  const long long n = dims.n;
  const long long st[4] = {n * n * n, n * n, n, 1};
  x.off = 0;
  for (int i = 0; i < 4; ++i) {
    x.d[i] = extent(dims, blk[i]);
    x.s[i] = st[i];
    if (blk[i] == 'v') x.off += dims.o * st[i];
  }
  return x;
}

View Program::Fb(const char* blk) const {
  View x;
  x.slot = S_F;
  x.dt = C64;
  x.nd = 2;
  const long long n = dims.n;
  x.d[0] = extent(dims, blk[0]);
  x.d[1] = extent(dims, blk[1]);
  x.s[0] = n;
  x.s[1] = 1;
  x.off = (blk[0] == 'v' ? dims.o * n : 0) + (blk[1] == 'v' ? dims.o : 0);
  return x;
}

View Program::amp(int slot) const {
  View x;
  x.slot = slot;
  x.dt = C64;
  const int o = dims.o, v = dims.v;
  if (slot == S_T1 || slot == S_L1) {
    x.nd = 2;
    x.d[0] = o;
    x.d[1] = v;
    x.s[0] = v;
    x.s[1] = 1;
  } else {
    x.nd = 4;
    x.d[0] = o;
    x.d[1] = o;
    x.d[2] = v;
    x.d[3] = v;
    x.s[3] = 1;
    x.s[2] = v;
    x.s[1] = (long long)v * v;
    x.s[0] = (long long)o * v * v;
  }
  return x;
}

View Program::out(int nd) {
  View x = amp(nd == 2 ? S_T1 : S_T2);
  x.slot = S_OUT;
  slots[S_OUT].numel = x.numel();  // the per-trajectory extent (batch stride)
  return x;
}

View Program::ws_dims(const std::string& nm, int nd, const int* d, int dt) {
  View x;
  x.slot = (int)slots.size();
  x.dt = dt;
  x.nd = nd;
  long long st = 1;
  for (int i = nd - 1; i >= 0; --i) {
    x.d[i] = d[i];
    x.s[i] = st;
    st *= d[i];
  }
  slots.push_back({nm, dt, st, false});
  return x;
}

View Program::ones(const std::string& nm, int len) {
  int d[1] = {len};
  View x = ws_dims(nm, 1, d, R64);
  slots[x.slot].init.assign(len, 1.0);
  return x;
}

View Program::ws(const std::string& nm, const char* shape, int dt) {
  int d[4];
  const int nd = (int)strlen(shape);
  for (int i = 0; i < nd; ++i) d[i] = extent(dims, shape[i]);
  return ws_dims(nm, nd, d, dt);
}

View Program::bc(const View& x, const char* from, const char* to) {
  View r;
  r.slot = x.slot;
  r.off = x.off;
  r.dt = x.dt;
  r.nd = (int)strlen(to);
  for (int i = 0; i < r.nd; ++i) {
    const char* p = strchr(from, to[i]);
    if (p) {
      const int k = (int)(p - from);
      r.d[i] = x.d[k];
      r.s[i] = x.s[k];
    } else {
      r.d[i] = 1;  // caller fixes dims to match the target
      r.s[i] = 0;
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// einsum -> GEMM over mode groups
// ---------------------------------------------------------------------------
void Program::ein(const char* spec, double ar, double ai, const View& A, const View& B,
                  const View& C, bool acc) {
  std::string s(spec);
  const size_t comma = s.find(','), arrow = s.find("->");
  if (comma == std::string::npos || arrow == std::string::npos)
    throw std::runtime_error("einsum spec: " + s);
  const std::string ia = s.substr(0, comma), ib = s.substr(comma + 1, arrow - comma - 1),
                    ic = s.substr(arrow + 2);
  if ((int)ia.size() != A.nd || (int)ib.size() != B.nd || (int)ic.size() != C.nd)
    throw std::runtime_error("einsum rank mismatch: " + s);
  auto dim_of = [&](char c) -> int {
    size_t p;
    if ((p = ia.find(c)) != std::string::npos) return A.d[p];
    if ((p = ib.find(c)) != std::string::npos) return B.d[p];
    return C.d[ic.find(c)];
  };
  // consistency of extents
  for (size_t i = 0; i < ia.size(); ++i)
    if (dim_of(ia[i]) != A.d[i]) throw std::runtime_error("einsum extent mismatch: " + s);
  for (size_t i = 0; i < ib.size(); ++i)
    if (dim_of(ib[i]) != B.d[i]) throw std::runtime_error("einsum extent mismatch: " + s);
  for (size_t i = 0; i < ic.size(); ++i)
    if (dim_of(ic[i]) != C.d[i]) throw std::runtime_error("einsum extent mismatch: " + s);

  Op op;
  op.kind = OP_GEMM;
  op.tag = name + ":" + s;
  GemmArgs& g = op.g;
  memset(&g, 0, sizeof(g));
  auto push = [&](ModeGroup& grp, int dim, long long s0, long long s1) {
    if (grp.n >= kMaxModes) throw std::runtime_error("einsum: too many modes in a group: " + s);
    grp.dim[grp.n] = dim;
    grp.s0[grp.n] = s0;
    grp.s1[grp.n] = s1;
    grp.n++;
  };
  for (size_t i = 0; i < ic.size(); ++i) {
    const char c = ic[i];
    const size_t pa = ia.find(c), pb = ib.find(c);
    if (pa != std::string::npos && pb != std::string::npos)
      throw std::runtime_error("einsum: batch index unsupported: " + s);
    if (pa != std::string::npos)
      push(g.gm, C.d[i], A.s[pa], C.s[i]);
    else if (pb != std::string::npos)
      push(g.gn, C.d[i], B.s[pb], C.s[i]);
    else
      throw std::runtime_error("einsum: broadcast output index unsupported: " + s);
  }
  for (size_t i = 0; i < ia.size(); ++i) {
    const char c = ia[i];
    if (ic.find(c) != std::string::npos) continue;
    if (ia.find(c) != i) throw std::runtime_error("einsum: repeated index: " + s);
    const size_t pb = ib.find(c);
    push(g.gk, A.d[i], A.s[i], pb != std::string::npos ? B.s[pb] : 0);
  }
  for (size_t i = 0; i < ib.size(); ++i) {
    const char c = ib[i];
    if (ic.find(c) != std::string::npos || ia.find(c) != std::string::npos) continue;
    push(g.gk, B.d[i], 0, B.s[i]);
  }
  auto prod = [](const ModeGroup& grp) {
    long long p = 1;
    for (int i = 0; i < grp.n; ++i) p *= grp.dim[i];
    return p;
  };
  const long long M = prod(g.gm), N = prod(g.gn), K = prod(g.gk);
  if (M > (1LL << 31) - 1 || N > (1LL << 31) - 1 || K > (1LL << 31) - 1)
    throw std::runtime_error("einsum: dimension too large: " + s);
  g.M = (int)M;
  g.N = (int)N;
  g.K = (int)K;
  g.ar = ar;
  g.ai = ai;
  g.acc = acc ? 1 : 0;
  g.nb = 1;
  plan_gemm(op, true);
  op.sa = A.slot;
  op.sb = B.slot;
  op.sc = C.slot;
  op.oa = A.off;
  op.ob = B.off;
  op.oc = C.off;
  op.dta = A.dt;
  op.dtb = B.dt;
  op.dtc = C.dt;
  if (C.dt == R64 && (A.dt == C64 || B.dt == C64))
    throw std::runtime_error("einsum: complex product into real output: " + s);
  const int mult = (A.dt == C64 && B.dt == C64) ? 8 : (A.dt == C64 || B.dt == C64) ? 4 : 2;
  op.flops = mult * M * N * K;
  auto esz = [](int dt) { return dt == C64 ? 16LL : 8LL; };
  op.bytes = M * K * esz(A.dt) + K * N * esz(B.dt) + M * N * esz(C.dt) * (acc ? 2 : 1);
  flops_total += op.flops;
  op.reads = {A.slot, B.slot};
  if (acc) op.reads.push_back(C.slot);
  op.write = C.slot;
  // split-K accumulates with atomics: zero the target first when overwriting
  op.zeroed = acc;
  if (g.atomic && !acc) {
    zero(C);
    op.reads.push_back(C.slot);
    op.zeroed = true;
  }
  ops.push_back(op);
}

// Tile shape, then split-K so that few output tiles still fill the 152 SMs
// (only where the output is zeroed or accumulated into: splits add with
// atomics).
void Program::plan_gemm(Op& op, bool allow_split, int tile) {
  GemmArgs& g = op.g;
  const long long M = g.M, N = g.N, K = g.K, nbt = std::max(g.nb, 1);
  op.tile = tile >= 0 ? tile : choose_tile(M, N);
  const long long tiles = ((M + kTiles[op.tile][0] - 1) / kTiles[op.tile][0]) *
                          ((N + kTiles[op.tile][1] - 1) / kTiles[op.tile][1]) * nbt;
  long long splits = 1;
  if (allow_split && tiles < 2 * 152 && K >= 64) {
    splits = (2 * 152 + tiles - 1) / tiles;
    splits = std::min<long long>(splits, K / 32);
    splits = std::max<long long>(splits, 1);
  }
  long long kchunk = (K + splits - 1) / splits;
  kchunk = ((kchunk + 15) / 16) * 16;
  g.kchunk = (int)std::max<long long>(kchunk, 16);
  splits = (K + g.kchunk - 1) / g.kchunk;
  g.nsplit = (int)std::max<long long>(splits, 1);
  g.atomic = splits > 1 ? 1 : 0;
}

void Program::add(const View& C, bool acc, const std::vector<Term>& terms) {
  if ((int)terms.size() > kMaxAddTerms) throw std::runtime_error("add: too many terms");
  Op op;
  op.kind = OP_ADD;
  op.tag = name + ":add";
  AddArgs& a = op.a;
  memset(&a, 0, sizeof(a));
  if (C.nd > kAddDims) throw std::runtime_error("add: too many dimensions in " + name);
  a.nd = C.nd;
  for (int i = 0; i < C.nd; ++i) {
    a.d[i] = C.d[i];
    a.sC[i] = C.s[i];
  }
  a.total = C.numel();
  a.cc = C.dt == C64;
  a.acc = acc ? 1 : 0;
  a.nt = (int)terms.size();
  op.add_sc = C.slot;
  op.add_oc = C.off;
  op.write = C.slot;
  if (acc) op.reads.push_back(C.slot);
  for (int t = 0; t < a.nt; ++t) {
    const Term& T = terms[t];
    if (T.A.nd != C.nd) throw std::runtime_error("add: term rank mismatch in " + name);
    for (int i = 0; i < C.nd; ++i)
      if (T.A.d[i] != C.d[i] && T.A.s[i] != 0) throw std::runtime_error("add: term dims mismatch in " + name);
    AddTerm& at = a.t[t];
    at.cr = T.cr;
    at.ci = T.ci;
    at.ac = T.A.dt == C64;
    for (int i = 0; i < C.nd; ++i) at.sA[i] = T.A.s[i];
    op.add_slots[t][0] = T.A.slot;
    op.add_off[t][0] = T.A.off;
    op.reads.push_back(T.A.slot);
    if (T.B.slot >= 0) {
      if (T.B.nd != C.nd) throw std::runtime_error("add: factor rank mismatch in " + name);
      at.bc = T.B.dt == C64;
      for (int i = 0; i < C.nd; ++i) at.sB[i] = T.B.s[i];
      op.add_slots[t][1] = T.B.slot;
      op.add_off[t][1] = T.B.off;
      op.reads.push_back(T.B.slot);
    } else {
      op.add_slots[t][1] = -1;
      op.add_off[t][1] = 0;
    }
    if (C.dt == R64 && (at.ac || at.bc || T.ci != 0.0))
      throw std::runtime_error("add: complex term into real output in " + name);
  }
  {
    const long long e = a.cc ? 16 : 8;
    long long nread = a.nt + (acc ? 1 : 0);
    for (int t = 0; t < a.nt; ++t)
      if (op.add_slots[t][1] >= 0) ++nread;
    op.bytes = a.total * e * (nread + 1);
  }
  coalesce(a);
  ops.push_back(op);
}

// Drops unit dimensions and merges neighbours k, k+1 wherever every operand
// is contiguous across them (s[k] == s[k+1] * d[k+1]), so the kernel
// decodes as few indices as possible.
void coalesce(AddArgs& a) {
  int nd = 0;
  int d[kAddDims];
  long long sc[kAddDims], sa[kMaxAddTerms][kAddDims], sb[kMaxAddTerms][kAddDims];
  for (int i = 0; i < a.nd; ++i) {
    if (a.d[i] == 1) continue;
    const bool merge = nd > 0 && [&] {
      const int j = nd - 1;
      if (sc[j] != a.sC[i] * a.d[i]) return false;
      for (int t = 0; t < a.nt; ++t) {
        if (sa[t][j] != a.t[t].sA[i] * a.d[i]) return false;
        if (sb[t][j] != a.t[t].sB[i] * a.d[i]) return false;
      }
      return true;
    }();
    if (merge) {
      const int j = nd - 1;
      d[j] *= a.d[i];
      sc[j] = a.sC[i];
      for (int t = 0; t < a.nt; ++t) {
        sa[t][j] = a.t[t].sA[i];
        sb[t][j] = a.t[t].sB[i];
      }
    } else {
      d[nd] = a.d[i];
      sc[nd] = a.sC[i];
      for (int t = 0; t < a.nt; ++t) {
        sa[t][nd] = a.t[t].sA[i];
        sb[t][nd] = a.t[t].sB[i];
      }
      ++nd;
    }
  }
  if (nd == 0) {  // a single element
    d[0] = 1;
    sc[0] = 0;
    for (int t = 0; t < a.nt; ++t) sa[t][0] = sb[t][0] = 0;
    nd = 1;
  }
  a.nd = nd;
  for (int i = 0; i < kAddDims; ++i) {
    a.d[i] = i < nd ? d[i] : 1;
    a.sC[i] = i < nd ? sc[i] : 0;
    for (int t = 0; t < a.nt; ++t) {
      a.t[t].sA[i] = i < nd ? sa[t][i] : 0;
      a.t[t].sB[i] = i < nd ? sb[t][i] : 0;
    }
  }
}

void Program::trace(int n_mu, const View& Dij, const View& L1, const View& Dai, const View& Dab) {
  Op op;
  op.kind = OP_TRACE;
  op.tag = name + ":trace";
  op.tr_slots[0] = Dij.slot;
  op.tr_slots[1] = L1.slot;
  op.tr_slots[2] = Dai.slot;
  op.tr_slots[3] = Dab.slot;
  op.tr_n_mu = n_mu;
  slots[S_RES].numel = n_mu;  // res = [n_mu] per trajectory
  op.reads = {Dij.slot, L1.slot, Dai.slot, Dab.slot, S_MU};
  op.write = S_RES;
  ops.push_back(op);
}

void Program::acc_pij(const View& C, const View& X, double c) {
  add(C, true, {Term{c, 0, X, View{}}, Term{-c, 0, X.swap(0, 1), View{}}});
}
void Program::acc_pab(const View& C, const View& X, double c) {
  add(C, true, {Term{c, 0, X, View{}}, Term{-c, 0, X.swap(2, 3), View{}}});
}
void Program::acc_pijab(const View& C, const View& X, double c) {
  add(C, true,
      {Term{c, 0, X, View{}}, Term{-c, 0, X.swap(2, 3), View{}}, Term{-c, 0, X.swap(0, 1), View{}},
       Term{c, 0, X.swap(0, 1).swap(2, 3), View{}}});
}

// ---------------------------------------------------------------------------
// dependency analysis
// ---------------------------------------------------------------------------
void Program::analyse(const std::vector<int>& varying_slots) {
  std::vector<char> vs(slots.size(), 0);
  for (int s : varying_slots) vs[s] = 1;
  vs[S_OUT] = 1;
  for (auto& op : ops) op.varying = false;
  bool changed = true;
  while (changed) {
    changed = false;
    for (auto& op : ops) {
      bool v = op.varying;
      for (int r : op.reads)
        if (r >= 0 && vs[r]) v = true;
      if (op.write >= 0 && vs[op.write]) v = true;
      if (v && !op.varying) {
        op.varying = true;
        changed = true;
      }
      if (v && op.write >= 0 && !vs[op.write]) {
        vs[op.write] = 1;
        changed = true;
      }
    }
  }
  // constant ops: (transitively) independent of every caller-bound slot
  // except the integrals, and writing slots no other op writes
  std::vector<char> dyn(slots.size(), 0);
  for (int s : {S_F, S_T1, S_T2, S_L1, S_L2, S_OUT, S_MU, S_RES}) dyn[s] = 1;
  std::vector<char> opdyn(ops.size(), 0);
  changed = true;
  while (changed) {
    changed = false;
    for (size_t i = 0; i < ops.size(); ++i) {
      const Op& op = ops[i];
      bool d = opdyn[i] || op.kind == OP_TRACE;
      for (int r : op.reads)
        if (r >= 0 && dyn[r]) d = true;
      if (op.write >= 0 && dyn[op.write]) d = true;
      if (d && !opdyn[i]) {
        opdyn[i] = 1;
        changed = true;
      }
      if (d && op.write >= 0 && !dyn[op.write]) {
        dyn[op.write] = 1;
        changed = true;
      }
    }
  }
  for (size_t i = 0; i < ops.size(); ++i) ops[i].is_const = !opdyn[i];
}

// ---------------------------------------------------------------------------
// trajectory batching
// ---------------------------------------------------------------------------
static bool prepend_mode(ModeGroup& g, int dim, long long s0, long long s1) {
  if (g.n >= kMaxModes) return false;
  for (int i = g.n; i > 0; --i) {
    g.dim[i] = g.dim[i - 1];
    g.s0[i] = g.s0[i - 1];
    g.s1[i] = g.s1[i - 1];
  }
  g.dim[0] = dim;
  g.s0[0] = s0;
  g.s1[0] = s1;
  g.n++;
  return true;
}

void Program::batch(int nbt) {
  if (nbt < 1) throw std::runtime_error("batch: trajectory count must be >= 1");
  for (auto& op : ops)
    if (op.kind == OP_PACK || op.kind == OP_TCGEMM)
      throw std::runtime_error("batch: must run before the backend selection");
  nb = nbt;
  for (auto& sl : slots) sl.numel1 = sl.numel;
  if (nb == 1) return;
  // slots that depend on a per-trajectory input
  std::vector<char> bt(slots.size(), 0);
  for (int sl : {S_F, S_T1, S_T2, S_L1, S_L2, S_OUT, S_RES}) bt[sl] = 1;
  bool changed = true;
  while (changed) {
    changed = false;
    for (const auto& op : ops) {
      bool any = false;
      for (int r : op.reads)
        if (r >= 0 && bt[r]) any = true;
      if (any && op.write >= 0 && !bt[op.write]) {
        bt[op.write] = 1;
        changed = true;
      }
    }
  }
  for (size_t i = 0; i < slots.size(); ++i) {
    slots[i].batched = bt[i] != 0;
    if (bt[i]) slots[i].numel = slots[i].numel1 * nb;
  }
  for (auto& op : ops) {
    if (op.kind == OP_GEMM) {
      GemmArgs& g = op.g;
      const bool ea = bt[op.sa], eb = bt[op.sb], ec = bt[op.sc];
      if (!ec) {
        if (ea || eb) throw std::runtime_error("batch: per-trajectory input into a shared output: " + op.tag);
        continue;
      }
      const long long M1 = g.M, N1 = g.N, K = g.K;
      const long long sa = bstride(op.sa), sb = bstride(op.sb), sc = bstride(op.sc);
      const long long kMax = (1LL << 31) - 1;
      const bool fold_m = ea && !eb && g.gm.n < kMaxModes && M1 * nb <= kMax;
      const bool fold_n = !fold_m && !ea && eb && g.gn.n < kMaxModes && N1 * nb <= kMax;
      if (fold_m) {
        prepend_mode(g.gm, nb, sa, sc);  // one GEMM over all trajectories' rows
        g.M = (int)(M1 * nb);
      } else if (fold_n) {
        prepend_mode(g.gn, nb, sb, sc);
        g.N = (int)(N1 * nb);
      } else {
        g.nb = nb;
        g.bsA = sa;
        g.bsB = sb;
        g.bsC = sc;
      }
      op.flops *= nb;
      auto esz = [](int dt) { return dt == C64 ? 16LL : 8LL; };
      op.bytes = (ea ? nb : 1) * M1 * K * esz(op.dta) + (eb ? nb : 1) * K * N1 * esz(op.dtb) +
                 nb * M1 * N1 * esz(op.dtc) * (g.acc ? 2 : 1);
      plan_gemm(op, op.zeroed);
    } else if (op.kind == OP_ADD) {
      AddArgs& a = op.a;
      if (!bt[op.add_sc]) {
        for (int t = 0; t < a.nt; ++t)
          if (bt[op.add_slots[t][0]] || (op.add_slots[t][1] >= 0 && bt[op.add_slots[t][1]]))
            throw std::runtime_error("batch: per-trajectory term into a shared output: " + op.tag);
        continue;
      }
      if (a.nd >= kAddDims) throw std::runtime_error("batch: too many dimensions: " + op.tag);
      for (int i = a.nd; i > 0; --i) {
        a.d[i] = a.d[i - 1];
        a.sC[i] = a.sC[i - 1];
        for (int t = 0; t < a.nt; ++t) {
          a.t[t].sA[i] = a.t[t].sA[i - 1];
          a.t[t].sB[i] = a.t[t].sB[i - 1];
        }
      }
      a.d[0] = nb;
      a.sC[0] = bstride(op.add_sc);
      for (int t = 0; t < a.nt; ++t) {
        a.t[t].sA[0] = bstride(op.add_slots[t][0]);
        a.t[t].sB[0] = op.add_slots[t][1] >= 0 ? bstride(op.add_slots[t][1]) : 0;
      }
      a.nd++;
      a.total *= nb;
      op.bytes *= nb;
      coalesce(a);
    } else if (op.kind == OP_TRACE) {
      op.tr_nb = nb;
      for (int k = 0; k < 4; ++k) op.tr_bs[k] = bstride(op.tr_slots[k]);
      op.tr_bsres = bstride(S_RES);
    }
  }
}

// Buffer sharing: a workspace slot touched only by ops of one phase (setup,
// prologue or stage), defined before it is read, can share memory with any
// other such slot whose program-order lifetime [first op, last op] does not
// overlap.  Every way a program is executed (whole, dynamic part, prologue
// then stages) keeps program order within a phase, and the DAG executor
// orders accesses by buffer, so the shared memory is never live twice.
void Program::plan_memory(size_t first) {
  slot_buf.resize(slots.size());
  for (size_t i = 0; i < slots.size(); ++i) slot_buf[i] = (int)i;
  const size_t n = slots.size();
  std::vector<int> f(n, -1), l(n, -1), ph(n, -1);
  std::vector<char> mixed(n, 0), read_first(n, 0);
  for (size_t k = 0; k < ops.size(); ++k) {
    const Op& op = ops[k];
    const int p = op.is_const ? 0 : op.varying ? 2 : 1;
    auto touch = [&](int sl, bool is_write) {
      if (sl < 0) return;
      if (f[sl] < 0) {
        f[sl] = (int)k;
        if (!is_write) read_first[sl] = 1;
      }
      l[sl] = (int)k;
      if (ph[sl] < 0) ph[sl] = p;
      else if (ph[sl] != p) mixed[sl] = 1;
    };
    for (int r : op.reads) touch(r, false);
    if (op.write >= 0) {
      // an op that reads its own output (accumulate) reads before writing
      bool reads_self = false;
      for (int r : op.reads) reads_self |= r == op.write;
      touch(op.write, !reads_self);
    }
  }
  struct Buf {
    size_t bytes;
    int free_after;  // last op index of its current occupant
  };
  std::vector<Buf> pool;
  std::vector<int> order;
  for (size_t i = std::max<size_t>(first, kNumFixedSlots); i < n; ++i) {
    if (slots[i].fixed || !slots[i].init.empty() || (int)i == err_slot || f[i] < 0 || mixed[i] || read_first[i] ||
        ph[i] == 0)
      continue;
    order.push_back((int)i);
  }
  std::sort(order.begin(), order.end(), [&](int a, int b) { return f[a] < f[b]; });
  for (int sl : order) {
    const size_t bytes = (size_t)slots[sl].numel * (size_t)elem_bytes(slots[sl].dt);
    int best = -1;
    for (size_t q = 0; q < pool.size(); ++q)
      if (pool[q].free_after < f[sl] && pool[q].bytes >= bytes && (best < 0 || pool[q].bytes < pool[best].bytes))
        best = (int)q;
    if (best < 0)
      for (size_t q = 0; q < pool.size(); ++q)  // grow the largest free buffer
        if (pool[q].free_after < f[sl] && (best < 0 || pool[q].bytes > pool[best].bytes)) best = (int)q;
    if (best < 0) {
      pool.push_back({bytes, l[sl]});
      buf_slot.push_back(sl);
      slot_buf[sl] = sl;
      pool_of[sl] = (int)pool.size() - 1;
    } else {
      pool[best].bytes = std::max(pool[best].bytes, bytes);
      pool[best].free_after = l[sl];
      slot_buf[sl] = buf_slot[best];
      pool_of[sl] = best;
    }
  }
  pool_bytes.clear();
  for (const auto& b : pool) pool_bytes.push_back(b.bytes);
}

long long Program::allocate(std::vector<void*>& bases, std::vector<void*>& owned, size_t first, bool zero) {
  long long bytes = 0;
  if (bases.size() < slots.size()) bases.resize(slots.size(), nullptr);
  // shared buffers first (plan_memory), then every other slot
  std::vector<void*> pool_ptr(pool_bytes.size(), nullptr);
  for (size_t q = 0; q < pool_bytes.size(); ++q) {
    void* p = nullptr;
    if (cudaMalloc(&p, pool_bytes[q]) != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error("cudaMalloc failed for a shared workspace buffer in " + name);
    }
    owned.push_back(p);
    pool_ptr[q] = p;
    // all-ones bytes are NaN: a read of memory no op wrote cannot pass silently
    if (cudaMemset(p, zero ? 0 : 0xFF, pool_bytes[q]) != cudaSuccess) throw std::runtime_error("clearing workspace failed");
    bytes += (long long)pool_bytes[q];
  }
  for (size_t i = std::max<size_t>(first, kNumFixedSlots); i < slots.size(); ++i) {
    if (slots[i].fixed) continue;
    auto it = pool_of.find((int)i);
    if (it != pool_of.end()) {
      bases[i] = pool_ptr[it->second];
      continue;
    }
    const size_t b = (size_t)slots[i].numel * (size_t)elem_bytes(slots[i].dt);
    void* p = nullptr;
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error("cudaMalloc failed for workspace " + slots[i].name + " in " + name);
    }
    owned.push_back(p);
    bases[i] = p;
    if (cudaMemset(p, zero ? 0 : 0xFF, b) != cudaSuccess) throw std::runtime_error("clearing workspace " + slots[i].name + " failed");
    if (!slots[i].init.empty() &&
        cudaMemcpy(p, slots[i].init.data(), slots[i].init.size() * sizeof(double),
                   cudaMemcpyHostToDevice) != cudaSuccess)
      throw std::runtime_error("upload of constant slot " + slots[i].name + " failed");
    bytes += (long long)b;
  }
  // A pageable cudaMemcpy may return before its DMA has landed, and the
  // program's kernels run on non-blocking streams that do not order against
  // it: wait for the uploads before any kernel can read these slots.
  if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("synchronising constant-slot uploads failed");
  return bytes;
}

static inline const void* at(const std::vector<void*>& b, int slot, long long off, int dt) {
  const char* p = static_cast<const char*>(b[slot]);
  return p + off * elem_bytes(dt);
}

bool Program::in_phase(const Op& op, Phase ph) {
  switch (ph) {
    case SETUP: return op.is_const;
    case DYNAMIC: return !op.is_const;
    case PROLOGUE: return !op.varying && !op.is_const;
    case STAGE: return op.varying;
    default: return true;
  }
}

cudaError_t Program::launch_op(const Op& op, const std::vector<void*>& bases, cudaStream_t st) const {
  cudaError_t e = cudaSuccess;
  if (op.kind == OP_GEMM) {
    const void* a = at(bases, op.sa, op.oa, op.dta);
    const void* b = at(bases, op.sb, op.ob, op.dtb);
    void* c = const_cast<void*>(at(bases, op.sc, op.oc, op.dtc));
    e = op.backend == GB_SIMT ? launch_simt_slices(op, a, b, c, st) : launch_gemm(op, a, b, c, st);
  } else if (op.kind == OP_ADD) {
    AddArgs a = op.a;
    a.C = const_cast<void*>(at(bases, op.add_sc, op.add_oc, a.cc ? C64 : R64));
    for (int t = 0; t < a.nt; ++t) {
      a.t[t].A = at(bases, op.add_slots[t][0], op.add_off[t][0], a.t[t].ac ? C64 : R64);
      a.t[t].B = op.add_slots[t][1] >= 0
                     ? at(bases, op.add_slots[t][1], op.add_off[t][1], a.t[t].bc ? C64 : R64)
                     : nullptr;
    }
    e = launch_add(a, st);
  } else if (op.kind == OP_TRACE) {
    e = launch_trace(dims.n, dims.o, op.tr_n_mu, static_cast<const double*>(bases[S_MU]),
                     bases[op.tr_slots[0]], bases[op.tr_slots[1]], bases[op.tr_slots[2]],
                     bases[op.tr_slots[3]], bases[S_RES], op.tr_nb, op.tr_bs, op.tr_bsres, st);
  } else if (op.kind == OP_PACK) {
    PackArgs p = op.pk;
    p.src = at(bases, op.pk_src, op.pk_off, op.pk_dt);
    char* dst = static_cast<char*>(bases[op.pk_dst]);
    p.out = dst;
    p.exps = reinterpret_cast<int*>(dst + op.pk_exp_off);
    e = launch_pack(p, st);
  } else if (op.kind == OP_REDUCE) {
    ReduceArgs r = op.rd;
    r.out = const_cast<void*>(at(bases, op.rd_out, op.rd_oout, C64));
    r.X = at(bases, op.rd_x, op.rd_ox, C64);
    r.Y = op.rd_y >= 0 ? at(bases, op.rd_y, op.rd_oy, r.ycplx ? C64 : R64) : nullptr;
    e = launch_reduce(r, st);
  } else if (op.kind == OP_TCGEMM) {
    TcArgs a = op.tc;
    const char* pa = static_cast<const char*>(bases[op.tc_pa]);
    const char* pb = static_cast<const char*>(bases[op.tc_pb]);
    a.expA = reinterpret_cast<const int*>(pa + op.tc_expa_off);
    a.expB = reinterpret_cast<const int*>(pb + op.tc_expb_off);
    a.C = const_cast<void*>(at(bases, op.sc, op.oc, op.dtc));
    a.err = static_cast<int*>(bases[op.tc_err]);
    e = launch_ozaki(a, pa, pb, st);
  }
  if (e != cudaSuccess) set_error("kernel launch failed in " + op.tag + ": " + cudaGetErrorString(e));
  return e;
}

cudaError_t Program::run(const std::vector<void*>& bases, cudaStream_t st, Phase ph,
                         std::vector<Timed>* timed) const {
  for (const auto& op : ops) {
    if (!in_phase(op, ph)) continue;
    Timed tm{&op, nullptr, nullptr};
    if (timed) {
      cudaEventCreate(&tm.a);
      cudaEventCreate(&tm.b);
      cudaEventRecord(tm.a, st);
    }
    const cudaError_t e = launch_op(op, bases, st);
    if (timed) {
      cudaEventRecord(tm.b, st);
      timed->push_back(tm);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// DAG execution: ops of a phase become nodes; edges follow the slot hazards
// (read-after-write, write-after-write, write-after-read).  Independent ops
// go to different streams of the pool; under stream capture the event
// waits become graph edges, so the captured graph runs them concurrently.
// ---------------------------------------------------------------------------
void DagExec::init(size_t nops, int nstreams) {
  if (!ev.empty()) return;
  streams.resize(nstreams);
  for (auto& s : streams) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  ev.resize(nops);
  for (auto& e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  for (int i = 0; i < nstreams; ++i) {
    cudaEvent_t e;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    tails.push_back(e);
  }
}

void DagExec::destroy() {
  for (auto& s : streams) cudaStreamDestroy(s);
  for (auto& e : ev) cudaEventDestroy(e);
  for (auto& e : tails) cudaEventDestroy(e);
  if (fork) cudaEventDestroy(fork);
  streams.clear();
  ev.clear();
  tails.clear();
  fork = nullptr;
}

cudaError_t Program::run_dag(const std::vector<void*>& bases, cudaStream_t st, Phase ph,
                             DagExec& ex) const {
  ex.init(ops.size(), 4);
  const int ns = (int)ex.streams.size();
  // hazards are tracked per buffer: slots that share memory are ordered too
  auto buf = [&](int sl) { return (sl >= 0 && sl < (int)slot_buf.size()) ? slot_buf[sl] : sl; };
  std::vector<int> last_writer(slots.size(), -1);
  std::vector<std::vector<int>> readers(slots.size());
  std::vector<int> op_stream(ops.size(), -1);
  std::vector<int> tail(ns, -1);  // last op issued on each stream
  std::vector<char> stream_used(ns, 0);
  cudaError_t e = cudaEventRecord(ex.fork, st);
  if (e != cudaSuccess) return e;
  int rr = 0;
  for (size_t i = 0; i < ops.size(); ++i) {
    const Op& op = ops[i];
    if (!in_phase(op, ph)) continue;
    std::vector<int> deps;
    for (int r : op.reads)
      if (r >= 0 && last_writer[buf(r)] >= 0) deps.push_back(last_writer[buf(r)]);
    if (op.write >= 0) {
      if (last_writer[buf(op.write)] >= 0) deps.push_back(last_writer[buf(op.write)]);
      for (int rd : readers[buf(op.write)]) deps.push_back(rd);
    }
    std::sort(deps.begin(), deps.end());
    deps.erase(std::unique(deps.begin(), deps.end()), deps.end());
    // prefer the stream whose last op is the newest dependency
    int s = -1;
    for (int k = (int)deps.size() - 1; k >= 0 && s < 0; --k)
      for (int q = 0; q < ns; ++q)
        if (tail[q] == deps[k]) {
          s = q;
          break;
        }
    if (s < 0) {
      s = rr;
      rr = (rr + 1) % ns;
    }
    cudaStream_t cs = ex.streams[s];
    if (!stream_used[s]) {
      if ((e = cudaStreamWaitEvent(cs, ex.fork, 0)) != cudaSuccess) return e;
      stream_used[s] = 1;
    }
    for (int d : deps)
      if (op_stream[d] != s && (e = cudaStreamWaitEvent(cs, ex.ev[d], 0)) != cudaSuccess) return e;
    if ((e = launch_op(op, bases, cs)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ex.ev[i], cs)) != cudaSuccess) return e;
    op_stream[i] = s;
    tail[s] = (int)i;
    for (int r : op.reads)
      if (r >= 0) readers[buf(r)].push_back((int)i);
    if (op.write >= 0) {
      last_writer[buf(op.write)] = (int)i;
      readers[buf(op.write)].clear();
    }
  }
  // join every used stream back into the caller's stream
  for (int q = 0; q < ns; ++q) {
    if (!stream_used[q]) continue;
    if ((e = cudaEventRecord(ex.tails[q], ex.streams[q])) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, ex.tails[q], 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static long long rup(long long x, long long m) { return (x + m - 1) / m * m; }

// Merges neighbouring modes of a packing traversal whose strides (s0) make
// them one run (s0[q] == dim[q+1] * s0[q+1]): the flat index maps to the
// same offsets, with fewer index divisions in the packing kernels.
static void merge_pack_modes(ModeGroup& g) {
  ModeGroup m{};
  for (int q = 0; q < g.n; ++q) {
    if (g.dim[q] == 1) continue;
    if (m.n > 0 && m.s0[m.n - 1] == (long long)g.dim[q] * g.s0[q]) {
      m.dim[m.n - 1] *= g.dim[q];
      m.s0[m.n - 1] = g.s0[q];
    } else {
      m.dim[m.n] = g.dim[q];
      m.s0[m.n] = g.s0[q];
      ++m.n;
    }
  }
  if (m.n == 0) {  // a single element
    m.n = 1;
    m.dim[0] = 1;
    m.s0[0] = 0;
  }
  for (int q = 0; q < m.n; ++q) m.s1[q] = m.s0[q];
  g = m;
}

void Program::select_backend(int prec_mode, long long min_macs, int S, int min_k, int min_mn, int simt_max_k,
                             long long simt_min_macs) {
  if (prec_mode != 1) return;
  if (S < 1 || S > 6) throw std::runtime_error("slices must be 1..6");
  constexpr int BM = 128, BN = 64, BK = 64;  // tensor-core tile (gemm_tc.h)
  std::vector<Op> out;
  out.reserve(ops.size() * 2);
  // packed operands already produced: identical packing of an unchanged
  // source is reused (e.g. t2 with K = (e,f) feeds three contractions)
  struct PackRef {
    int slot;
    long long exp_off;
    size_t pos;  // index of the pack op in `out`
    int src;
  };
  std::map<std::string, PackRef> pack_cache;
  std::vector<long long> last_write(slots.size() + 4 * ops.size() + 16, -1);
  auto push_op = [&](const Op& o) {
    if (o.write >= 0) {
      if ((size_t)o.write >= last_write.size()) last_write.resize(o.write + 1, -1);
      last_write[o.write] = (long long)out.size();
    }
    out.push_back(o);
  };
  auto group_key = [](const ModeGroup& g, bool use_s1) {
    std::string k = std::to_string(g.n);
    for (int i = 0; i < g.n; ++i)
      k += "," + std::to_string(g.dim[i]) + ":" + std::to_string(use_s1 ? g.s1[i] : g.s0[i]);
    return k;
  };
  for (auto& op : ops) {
    if (op.kind != OP_GEMM) {
      push_op(op);
      continue;
    }
    const long long M = op.g.M, N = op.g.N, K = op.g.K;
    if (M * N * K * std::max(op.g.nb, 1) < min_macs || K < min_k || std::min(M, N) < min_mn) {
      // short contractions: slice products on the FP32 pipe (the FP64 pipe
      // is the one the elementwise ops and the update need)
      const bool types_ok = op.dtc == C64 || (op.dta != C64 && op.dtb != C64);
      if (K <= simt_max_k && simt_slices_supported((int)K, S) && types_ok &&
          M * N * K * std::max(op.g.nb, 1) >= simt_min_macs) {
        Op o = op;
        o.backend = GB_SIMT;
        o.g.nsplit = 1;
        o.g.kchunk = (int)K;
        o.g.atomic = 0;
        o.tc = TcArgs{};
        o.tc.S = S;
        int e2 = 0;
        const double fr = std::frexp(std::fabs(op.g.ar), &e2);
        o.tc.alpha_pow2 = (op.g.ai == 0.0 && op.g.ar != 0.0 && fr == 0.5) ? 1 : 0;
        o.tc.alpha_e = e2 - 1;
        o.tc.alpha_neg = op.g.ar < 0.0 ? 1 : 0;
        push_op(o);
      } else {
        push_op(op);
      }
      continue;
    }
    if (err_slot < 0) {
      int d1[1] = {256};
      View e = ws_dims("tc_err", 1, d1, U8);
      slots[e.slot].init.assign(32, 0.0);
      err_slot = e.slot;
    }
    const bool ac = op.dta == C64, bc = op.dtb == C64;
    // S <= 4: the 128-column tile (one K chunk per CTA, K split across CTAs
    // beyond it) when B has rows enough to fill it
    const long long nBrows = N * (bc ? 2 : 1);
    const bool tile128 = S <= TC_TILE128_MAX_S && nBrows >= 96;
    const long long rA = rup(M * (ac ? 2 : 1), BM), rB = rup(nBrows, tile128 ? TcTile128::BN : BN),
                    Kp = rup(K, BK);
    // batched products: an operand with a batch stride is packed per batch
    const int nbt = std::max(op.g.nb, 1);
    const int nbA = (nbt > 1 && op.g.bsA != 0) ? nbt : 1, nbB = (nbt > 1 && op.g.bsB != 0) ? nbt : 1;
    auto packed_slot = [&](const std::string& nm, long long rows, long long& exp_off) {
      exp_off = rup((long long)S * rows * Kp * 2, 256);
      int d1[1] = {(int)0};
      const long long bytes = exp_off + rup(rows * 4, 256);
      if (bytes > (1LL << 31) - 1) {
        // store as R64 elements to keep the extent in an int
        d1[0] = (int)((bytes + 7) / 8);
        return ws_dims(nm, 1, d1, R64).slot;
      }
      d1[0] = (int)bytes;
      return ws_dims(nm, 1, d1, U8).slot;
    };
    Op pa, pb, t;
    pa.varying = pb.varying = t.varying = op.varying;  // phases of reverse-mode programs
    pa.is_const = pb.is_const = t.is_const = op.is_const;
    pa.kind = pb.kind = OP_PACK;
    pa.tag = op.tag + ":packA";
    pb.tag = op.tag + ":packB";
    // A: rows = M modes (strides g.gm.s0), K modes strides g.gk.s0
    pa.pk = PackArgs{};
    pa.pk.cplx = ac;
    pa.pk.gr = op.g.gm;
    pa.pk.gk = op.g.gk;
    pa.pk.rows = (int)M;
    pa.pk.K = (int)K;
    pa.pk.rows_pad = (int)rA;
    pa.pk.K_pad = (int)Kp;
    pa.pk.S = S;
    pa.pk.nb = nbA;
    pa.pk.bs = op.g.bsA;
    pa.pk_src = op.sa;
    pa.pk_off = op.oa;
    pa.pk_dt = op.dta;
    pa.reads = {op.sa};
    pa.write = pa.pk_dst;
    pa.bytes = nbA * (M * K * elem_bytes(op.dta) + (long long)S * rA * Kp * 2);
    // B: rows = N modes (strides g.gn.s0), K modes strides g.gk.s1
    pb.pk = PackArgs{};
    pb.pk.cplx = bc;
    pb.pk.gr = op.g.gn;
    pb.pk.gk = op.g.gk;
    for (int i = 0; i < kMaxModes; ++i) pb.pk.gk.s0[i] = op.g.gk.s1[i];
    pb.pk.rows = (int)N;
    pb.pk.K = (int)K;
    pb.pk.rows_pad = (int)rB;
    pb.pk.K_pad = (int)Kp;
    pb.pk.S = S;
    pb.pk.nb = nbB;
    pb.pk.bs = op.g.bsB;
    pb.pk_src = op.sb;
    pb.pk_off = op.ob;
    pb.pk_dt = op.dtb;
    pb.reads = {op.sb};
    pb.bytes = nbB * (N * K * elem_bytes(op.dtb) + (long long)S * rB * Kp * 2);
    merge_pack_modes(pa.pk.gr);
    merge_pack_modes(pa.pk.gk);
    merge_pack_modes(pb.pk.gr);
    merge_pack_modes(pb.pk.gk);
    // resolve packed slots (reuse an identical, still valid packing)
    bool emit_a = true, emit_b = true;
    auto resolve = [&](Op& pk, const ModeGroup& gr, const ModeGroup& gk, bool k_s1, long long rows,
                       const std::string& nm, bool& emit) {
      const std::string key = std::to_string(pk.pk_src) + "@" + std::to_string(pk.pk_off) + "#" +
                              std::to_string(pk.pk_dt) + "|" + group_key(gr, false) + "|" +
                              group_key(gk, k_s1) + "|" + std::to_string(rows) + "x" + std::to_string(Kp) +
                              "s" + std::to_string(S) + "b" + std::to_string(pk.pk.nb) + ":" +
                              std::to_string(pk.pk.bs) + (op.varying ? "v" : "p") + (op.is_const ? "c" : "");
      auto it = pack_cache.find(key);
      if (it != pack_cache.end() && last_write[it->second.src] < (long long)it->second.pos) {
        pk.pk_dst = it->second.slot;
        pk.pk_exp_off = it->second.exp_off;
        emit = false;
        return;
      }
      pk.pk_dst = packed_slot(nm, rows * pk.pk.nb, pk.pk_exp_off);
      pk.write = pk.pk_dst;
      emit = true;
      pack_cache[key] = PackRef{pk.pk_dst, pk.pk_exp_off, (size_t)-1, pk.pk_src};
    };
    resolve(pa, op.g.gm, op.g.gk, false, rA, op.tag + ":packA", emit_a);
    resolve(pb, op.g.gn, op.g.gk, true, rB, op.tag + ":packB", emit_b);
    // slice product
    t.kind = OP_TCGEMM;
    t.tag = op.tag;
    t.backend = GB_TC;
    t.flops = op.flops;
    t.sc = op.sc;
    t.oc = op.oc;
    t.dtc = op.dtc;
    t.tc_pa = pa.pk_dst;
    t.tc_pb = pb.pk_dst;
    t.tc_err = err_slot;
    t.tc_expa_off = pa.pk_exp_off;
    t.tc_expb_off = pb.pk_exp_off;
    TcArgs& a = t.tc;
    a = TcArgs{};
    a.M = (int)M;
    a.N = (int)N;
    a.rowsA_pad = (int)rA;
    a.rowsB_pad = (int)rB;
    a.nb = nbt;
    a.bat_a = nbA > 1;
    a.bat_b = nbB > 1;
    a.bsC = op.g.bsC;
    a.kblocks = (int)(Kp / BK);
    a.S = S;
    int cols = 32;
    while (cols < (S + 2) * BN) cols *= 2;  // S level accumulators + int64 partial sums
    if (cols > 512) throw std::runtime_error("tensor-core tile needs more than 512 TMEM columns");
    a.tmem_cols = cols;
    a.ac = ac;
    a.bc = bc;
    a.cc = op.dtc == C64;
    a.gmC = op.g.gm;
    a.gnC = op.g.gn;
    for (int i = 0; i < kMaxModes; ++i) {
      a.gmC.s0[i] = op.g.gm.s1[i];
      a.gnC.s0[i] = op.g.gn.s1[i];
    }
    a.ar = op.g.ar;
    a.ai = op.g.ai;
    {
      // real power-of-two coefficients (the equations' +-1, +-1/2, +-1/4 ...)
      // are applied exactly in the exponent of the epilogue's conversion
      int e2 = 0;
      const double fr = std::frexp(std::fabs(op.g.ar), &e2);
      a.alpha_pow2 = (op.g.ai == 0.0 && op.g.ar != 0.0 && fr == 0.5) ? 1 : 0;
      a.alpha_e = e2 - 1;
      a.alpha_neg = op.g.ar < 0.0 ? 1 : 0;
    }
    a.acc = op.g.acc;
    // split K so that few output tiles still occupy the SMs: one CTA per SM,
    // cost = waves x (K blocks per CTA + fixed pipeline/epilogue overhead);
    // the 128-column tile takes at most one exact K chunk per CTA
    // S <= 4 and at most two K blocks: the persistent 64-column form, whose
    // TMEM drain runs under the next tile's loads and MMAs (measured at o=10,
    // v=38 with 24 trajectories: 10-35 % faster than the 128-column tile for
    // one or two K blocks, 30-50 % slower for six or more, where the
    // 128-column tile's MMA rate and operand reuse count)
    const bool persist = S <= TC_TILE128_MAX_S && a.kblocks <= 2;
    const long long ctas = (rB / (tile128 && !persist ? TcTile128::BN : BN)) * (rA / BM) * nbt;
    const long long min_sp = (tile128 || persist) ? (a.kblocks + tc_chunk_kblocks(S) - 1) / tc_chunk_kblocks(S) : 1;
    long long splits = min_sp;
    {
      double best = 1e300;
      const long long maxs = std::max<long long>(min_sp, std::min<long long>(a.kblocks, 64));
      for (long long sp = min_sp; sp <= maxs; ++sp) {
        const long long waves = (ctas * sp + 151) / 152;
        const long long per = (a.kblocks + sp - 1) / sp;
        const double cost = (double)waves * (double)(per * S + 6);
        if (cost < best - 1e-9) {
          best = cost;
          splits = sp;
        }
      }
    }
    a.kb_per_split = (int)((a.kblocks + splits - 1) / splits);
    splits = (a.kblocks + a.kb_per_split - 1) / a.kb_per_split;
    a.nsplit = (int)splits;
    a.atomic = splits > 1 ? 1 : 0;
    t.zeroed = a.acc || a.atomic;  // split K is allowed (a zero op precedes when not accumulating)
    // short K: the narrow variant (two CTAs per SM overlap their latencies)
    a.variant = persist ? 3 : tile128 ? 2 : (a.kb_per_split == 1 && S <= 5) ? 1 : 0;
    t.bytes = (long long)S * (nbA * rA + nbB * rB) * Kp * 2 + nbt * M * N * elem_bytes(op.dtc);
    t.reads = {pa.pk_dst, pb.pk_dst};
    if (a.acc || a.atomic) t.reads.push_back(op.sc);
    t.write = op.sc;
    for (Op* pk : {&pa, &pb}) {
      if (!((pk == &pa) ? emit_a : emit_b)) continue;
      for (auto& kv : pack_cache)
        if (kv.second.slot == pk->pk_dst) kv.second.pos = out.size();
      push_op(*pk);
    }
    if (a.atomic && !a.acc) {
      // zero the output first: its modes are the M and N groups (strides s1)
      Op z;
      z.varying = op.varying;
      z.is_const = op.is_const;
      z.kind = OP_ADD;
      z.tag = op.tag + ":zero";
      AddArgs& za = z.a;
      memset(&za, 0, sizeof(za));
      // output modes: batch, then the M and N groups (strides s1), sorted by
      // decreasing stride so that the coalescing can merge them
      std::vector<std::pair<long long, int>> md;
      if (nbt > 1) md.push_back({op.g.bsC, nbt});
      for (int i = 0; i < op.g.gm.n; ++i) md.push_back({op.g.gm.s1[i], op.g.gm.dim[i]});
      for (int i = 0; i < op.g.gn.n; ++i) md.push_back({op.g.gn.s1[i], op.g.gn.dim[i]});
      std::stable_sort(md.begin(), md.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
      std::vector<std::pair<long long, int>> mm;
      for (const auto& x : md) {
        if (!mm.empty() && mm.back().first == x.first * x.second) {
          mm.back().first = x.first;
          mm.back().second *= x.second;
        } else if (x.second > 1) {
          mm.push_back(x);
        }
      }
      if ((int)mm.size() > kAddDims) throw std::runtime_error("tensor-core output with too many modes: " + op.tag);
      za.nd = std::max<int>(1, (int)mm.size());
      for (int i = 0; i < kAddDims; ++i) {
        za.d[i] = i < (int)mm.size() ? mm[i].second : 1;
        za.sC[i] = i < (int)mm.size() ? mm[i].first : 0;
      }
      za.total = M * N * nbt;
      za.cc = op.dtc == C64;
      za.acc = 0;
      za.nt = 0;
      z.add_sc = op.sc;
      z.add_oc = op.oc;
      z.write = op.sc;
      z.bytes = nbt * M * N * elem_bytes(op.dtc);
      push_op(z);
    }
    push_op(t);
  }
  ops.swap(out);
}

}  // namespace tdcc
