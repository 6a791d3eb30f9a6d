// Reverse-mode programs: the vector-Jacobian product of an equation program,
// generated from its op list (the op list is the program; its adjoint is the
// op list read backwards, each op replaced by its transposed products).
//
// Conventions.  The equations are holomorphic in the amplitudes and the
// dressed Fock matrix (polynomials, no conjugation), and the objective J is
// real.  With g = dJ/dRe z + i dJ/dIm z, a holomorphic map w = f(z) gives
// g_z = J_f^H g_w; the conjugate a = conj(g) therefore obeys a_z = J_f^T a_w,
// so every op reverses into plain transposed products with the forward
// coefficients (no conjugations anywhere).  A real parameter theta entering
// through z contributes dJ/dtheta = Re(sum a * dz/dtheta).
//
//   C (=|+=) alpha A B        ->  aA += alpha aC B^T ;  aB += alpha A^T aC ;
//                                 aC = 0 if C was overwritten
//   C (=|+=) sum_t c_t A_t B_t ->  aA_t += c_t aC B_t (a reduction where A_t is
//                                 broadcast) ; same for B_t ; aC = 0 if overwritten
//   res_k = sum mu_k rho      ->  a_rho += sum_k a_res_k mu_k ; a_res = 0
#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "engine.h"

namespace tdcc {

namespace {

long long group_size(const ModeGroup& g) {
  long long p = 1;
  for (int i = 0; i < g.n; ++i) p *= g.dim[i];
  return p;
}

// zero `slot` (+ offset) over an index space given as (dim, stride) pairs
Op zero_op(int slot, long long off, int dt, std::vector<std::pair<long long, int>> md, const std::string& tag) {
  // decreasing stride, then merge contiguous neighbours
  std::stable_sort(md.begin(), md.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
  std::vector<std::pair<long long, int>> mm;
  for (const auto& x : md) {
    if (x.second <= 1) continue;
    if (!mm.empty() && mm.back().first == x.first * x.second) {
      mm.back().first = x.first;
      mm.back().second *= x.second;
    } else {
      mm.push_back(x);
    }
  }
  if ((int)mm.size() > kAddDims) throw std::runtime_error("adjoint: zero over too many dimensions: " + tag);
  Op z;
  z.kind = OP_ADD;
  z.tag = tag;
  memset(&z.a, 0, sizeof(z.a));
  long long total = 1;
  z.a.nd = std::max<int>(1, (int)mm.size());
  for (int i = 0; i < kAddDims; ++i) {
    z.a.d[i] = i < (int)mm.size() ? mm[i].second : 1;
    z.a.sC[i] = i < (int)mm.size() ? mm[i].first : 0;
    if (i < (int)mm.size()) total *= mm[i].second;
  }
  z.a.total = total;
  z.a.cc = dt == C64;
  z.a.acc = 0;
  z.a.nt = 0;
  z.add_sc = slot;
  z.add_oc = off;
  z.write = slot;
  z.bytes = total * elem_bytes(dt);
  return z;
}

}  // namespace

void build_adjoint(const Program& f, Program& a, std::vector<int>& adj_of) {
  for (const auto& op : f.ops)
    if (op.kind == OP_PACK || op.kind == OP_TCGEMM || op.kind == OP_REDUCE)
      throw std::runtime_error("adjoint: build it from the FP64 op list (before the backend selection)");
  a.dims = f.dims;
  a.name = f.name + "_adj";
  a.nb = f.nb;
  a.slots = f.slots;
  a.ops.clear();
  a.flops_total = 0;
  a.err_slot = -1;
  const int nf = (int)f.slots.size();
  // differentiable slots: the inputs and everything computed from them
  std::vector<char> d(nf, 0);
  for (int s : {S_F, S_T1, S_T2, S_L1, S_L2}) d[s] = 1;
  bool changed = true;
  while (changed) {
    changed = false;
    for (const auto& op : f.ops) {
      bool any = false;
      for (int r : op.reads)
        if (r >= 0 && r < nf && d[r]) any = true;
      if (any && op.write >= 0 && !d[op.write]) {
        d[op.write] = 1;
        changed = true;
      }
    }
  }
  adj_of.assign(nf, -1);
  for (int s = 0; s < nf; ++s) {
    if (!d[s]) continue;
    if (f.slots[s].dt != C64) throw std::runtime_error("adjoint: real differentiable slot " + f.slots[s].name);
    SlotInfo si = f.slots[s];
    si.name = "adj:" + si.name;
    si.init.clear();
    adj_of[s] = (int)a.slots.size();
    a.slots.push_back(si);
  }
  auto adj = [&](int s) { return (s >= 0 && s < nf) ? adj_of[s] : -1; };
  auto push = [&](Op o, const Op& from) {
    o.varying = from.varying;
    o.is_const = from.is_const;
    a.flops_total += o.flops;
    a.ops.push_back(std::move(o));
  };

  for (int i = (int)f.ops.size() - 1; i >= 0; --i) {
    const Op& op = f.ops[i];
    if (op.is_const || op.write < 0 || adj(op.write) < 0) continue;
    if (op.kind == OP_GEMM) {
      const GemmArgs& g = op.g;
      const int aC = adj(op.sc);
      const long long nbt = std::max(g.nb, 1);
      auto esz = [](int dt) { return dt == C64 ? 16LL : 8LL; };
      // aA[gm, gk] += alpha sum_gn aC[gm, gn] B[gk, gn]
      if (adj(op.sa) >= 0) {
        Op o;
        o.kind = OP_GEMM;
        o.tag = op.tag + ":adjA";
        memset(&o.g, 0, sizeof(o.g));
        GemmArgs& h = o.g;
        h.gm = g.gm;  // s0: aC strides (= C's), s1: aA strides (= A's)
        for (int k = 0; k < g.gm.n; ++k) std::swap(h.gm.s0[k], h.gm.s1[k]);
        h.gn = g.gk;  // s0: B strides, s1: aA strides
        for (int k = 0; k < g.gk.n; ++k) {
          h.gn.s0[k] = g.gk.s1[k];
          h.gn.s1[k] = g.gk.s0[k];
        }
        h.gk = g.gn;  // s0: aC strides, s1: B strides
        for (int k = 0; k < g.gn.n; ++k) {
          h.gk.s0[k] = g.gn.s1[k];
          h.gk.s1[k] = g.gn.s0[k];
        }
        h.M = (int)group_size(h.gm);
        h.N = (int)group_size(h.gn);
        h.K = (int)group_size(h.gk);
        h.ar = g.ar;
        h.ai = g.ai;
        h.acc = 1;
        h.nb = g.nb;
        h.bsA = g.bsC;
        h.bsB = g.bsB;
        h.bsC = g.bsA;
        o.sa = aC;
        o.oa = op.oc;
        o.dta = C64;
        o.sb = op.sb;
        o.ob = op.ob;
        o.dtb = op.dtb;
        o.sc = adj(op.sa);
        o.oc = op.oa;
        o.dtc = C64;
        o.zeroed = true;
        Program::plan_gemm(o, true);
        const int mult = op.dtb == C64 ? 8 : 4;
        o.flops = mult * (long long)h.M * h.N * h.K * nbt;
        o.bytes = nbt * ((long long)h.M * h.K * 16 + (long long)h.K * h.N * esz(op.dtb) + 2LL * h.M * h.N * 16);
        o.reads = {o.sa, o.sb, o.sc};
        o.write = o.sc;
        push(std::move(o), op);
      }
      // aB[gk, gn] += alpha sum_gm A[gm, gk] aC[gm, gn]
      if (adj(op.sb) >= 0) {
        Op o;
        o.kind = OP_GEMM;
        o.tag = op.tag + ":adjB";
        memset(&o.g, 0, sizeof(o.g));
        GemmArgs& h = o.g;
        h.gm = g.gk;  // s0: A strides, s1: aB strides
        h.gn = g.gn;  // s0: aC strides, s1: aB strides
        for (int k = 0; k < g.gn.n; ++k) {
          h.gn.s0[k] = g.gn.s1[k];
          h.gn.s1[k] = g.gn.s0[k];
        }
        h.gk = g.gm;  // s0: A strides, s1: aC strides
        h.M = (int)group_size(h.gm);
        h.N = (int)group_size(h.gn);
        h.K = (int)group_size(h.gk);
        h.ar = g.ar;
        h.ai = g.ai;
        h.acc = 1;
        h.nb = g.nb;
        h.bsA = g.bsA;
        h.bsB = g.bsC;
        h.bsC = g.bsB;
        o.sa = op.sa;
        o.oa = op.oa;
        o.dta = op.dta;
        o.sb = aC;
        o.ob = op.oc;
        o.dtb = C64;
        o.sc = adj(op.sb);
        o.oc = op.ob;
        o.dtc = C64;
        o.zeroed = true;
        Program::plan_gemm(o, true);
        const int mult = op.dta == C64 ? 8 : 4;
        o.flops = mult * (long long)h.M * h.N * h.K * nbt;
        o.bytes = nbt * ((long long)h.M * h.K * esz(op.dta) + (long long)h.K * h.N * 16 + 2LL * h.M * h.N * 16);
        o.reads = {o.sa, o.sb, o.sc};
        o.write = o.sc;
        push(std::move(o), op);
      }
      if (!g.acc) {
        std::vector<std::pair<long long, int>> md;
        if (nbt > 1) md.push_back({g.bsC, (int)nbt});
        for (int k = 0; k < g.gm.n; ++k) md.push_back({g.gm.s1[k], g.gm.dim[k]});
        for (int k = 0; k < g.gn.n; ++k) md.push_back({g.gn.s1[k], g.gn.dim[k]});
        push(zero_op(aC, op.oc, C64, md, op.tag + ":adj0"), op);
      }
    } else if (op.kind == OP_ADD) {
      const AddArgs& x = op.a;
      const int aC = adj(op.add_sc);
      for (int t = 0; t < x.nt; ++t)
        for (int which = 0; which < 2; ++which) {
          const int slotX = op.add_slots[t][which];
          if (slotX < 0 || adj(slotX) < 0) continue;
          if (slotX == op.add_sc) throw std::runtime_error("adjoint: in-place elementwise op in " + op.tag);
          const long long* sX = which == 0 ? x.t[t].sA : x.t[t].sB;
          const int slotY = op.add_slots[t][1 - which];
          const long long* sY = which == 0 ? x.t[t].sB : x.t[t].sA;
          const long long offX = op.add_off[t][which], offY = op.add_off[t][1 - which];
          const int ycplx = which == 0 ? x.t[t].bc : x.t[t].ac;
          bool reduce = false;
          for (int k = 0; k < x.nd; ++k)
            if (x.d[k] > 1 && sX[k] == 0) reduce = true;
          if (!reduce) {
            Op o;
            o.kind = OP_ADD;
            o.tag = op.tag + ":adj";
            memset(&o.a, 0, sizeof(o.a));
            AddArgs& y = o.a;
            y.nd = x.nd;
            for (int k = 0; k < x.nd; ++k) {
              y.d[k] = x.d[k];
              y.sC[k] = sX[k];
              y.t[0].sA[k] = x.sC[k];
              y.t[0].sB[k] = slotY >= 0 ? sY[k] : 0;
            }
            y.total = x.total;
            y.cc = 1;
            y.acc = 1;
            y.nt = 1;
            y.t[0].ac = 1;
            y.t[0].bc = ycplx;
            y.t[0].cr = x.t[t].cr;
            y.t[0].ci = x.t[t].ci;
            o.add_sc = adj(slotX);
            o.add_oc = offX;
            o.add_slots[0][0] = aC;
            o.add_off[0][0] = op.add_oc;
            o.add_slots[0][1] = slotY;
            o.add_off[0][1] = slotY >= 0 ? offY : 0;
            o.reads = {aC, o.add_sc};
            if (slotY >= 0) o.reads.push_back(slotY);
            o.write = o.add_sc;
            o.bytes = x.total * 16 * (slotY >= 0 ? 4 : 3);
            coalesce(y);
            push(std::move(o), op);
          } else {
            Op o;
            o.kind = OP_REDUCE;
            o.tag = op.tag + ":adjR";
            ReduceArgs& r = o.rd;
            memset(&r, 0, sizeof(r));
            long long no = 1, nr = 1;
            for (int k = 0; k < x.nd; ++k) {
              if (x.d[k] == 1) continue;
              if (sX[k] != 0) {
                if (r.no >= kRedDims) throw std::runtime_error("adjoint: reduce dims: " + op.tag);
                r.dout[r.no] = x.d[k];
                r.so_out[r.no] = sX[k];
                r.so_x[r.no] = x.sC[k];
                r.so_y[r.no] = slotY >= 0 ? sY[k] : 0;
                no *= x.d[k];
                r.no++;
              } else {
                if (r.nr >= kRedDims) throw std::runtime_error("adjoint: reduce dims: " + op.tag);
                r.dred[r.nr] = x.d[k];
                r.sr_x[r.nr] = x.sC[k];
                r.sr_y[r.nr] = slotY >= 0 ? sY[k] : 0;
                nr *= x.d[k];
                r.nr++;
              }
            }
            r.nout = no;
            r.nred = nr;
            r.ycplx = ycplx;
            r.cr = x.t[t].cr;
            r.ci = x.t[t].ci;
            r.acc = 1;
            o.rd_out = adj(slotX);
            o.rd_oout = offX;
            o.rd_x = aC;
            o.rd_ox = op.add_oc;
            o.rd_y = slotY;
            o.rd_oy = slotY >= 0 ? offY : 0;
            o.reads = {aC, o.rd_out};
            if (slotY >= 0) o.reads.push_back(slotY);
            o.write = o.rd_out;
            o.flops = 8 * no * nr;
            o.bytes = no * nr * 16 * (slotY >= 0 ? 2 : 1) + no * 32;
            push(std::move(o), op);
          }
        }
      if (!x.acc) {
        std::vector<std::pair<long long, int>> md;
        for (int k = 0; k < x.nd; ++k) md.push_back({x.sC[k], x.d[k]});
        push(zero_op(aC, op.add_oc, C64, md, op.tag + ":adj0"), op);
      }
    } else if (op.kind == OP_TRACE) {
      // a_block[p, q] += a_res[k] * mu_k[p, q] for the four density blocks
      const int aR = adj(S_RES);
      const int o_ = f.dims.o, v = f.dims.v, n = f.dims.n;
      const int rows[4] = {o_, o_, v, v}, cols[4] = {o_, v, o_, v};
      const long long moff[4] = {0, (long long)o_, (long long)o_ * n, (long long)o_ * n + o_};
      for (int b = 0; b < 4; ++b) {
        const int sl = op.tr_slots[b];
        if (adj(sl) < 0) continue;
        for (int k = 0; k < op.tr_n_mu; ++k) {
          Op o;
          o.kind = OP_ADD;
          o.tag = op.tag + ":adj";
          memset(&o.a, 0, sizeof(o.a));
          AddArgs& y = o.a;
          const int nbt = std::max(op.tr_nb, 1);
          y.nd = 3;
          y.d[0] = nbt;
          y.d[1] = rows[b];
          y.d[2] = cols[b];
          y.sC[0] = nbt > 1 ? op.tr_bs[b] : 0;
          y.sC[1] = cols[b];
          y.sC[2] = 1;
          y.t[0].sA[0] = nbt > 1 ? op.tr_bsres : 0;  // a_res[k] broadcast over the block
          y.t[0].sB[1] = n;                          // mu_k block (shared by trajectories)
          y.t[0].sB[2] = 1;
          y.total = (long long)nbt * rows[b] * cols[b];
          y.cc = 1;
          y.acc = 1;
          y.nt = 1;
          y.t[0].ac = 1;
          y.t[0].bc = 0;
          y.t[0].cr = 1.0;
          y.t[0].ci = 0.0;
          o.add_sc = adj(sl);
          o.add_oc = 0;
          o.add_slots[0][0] = aR;
          o.add_off[0][0] = k;
          o.add_slots[0][1] = S_MU;
          o.add_off[0][1] = (long long)k * n * n + moff[b];
          o.reads = {aR, S_MU, o.add_sc};
          o.write = o.add_sc;
          o.bytes = y.total * 40;
          coalesce(y);
          push(std::move(o), op);
        }
      }
      std::vector<std::pair<long long, int>> md = {{1, op.tr_n_mu}};
      if (op.tr_nb > 1) md.push_back({op.tr_bsres, op.tr_nb});
      push(zero_op(aR, 0, C64, md, op.tag + ":adj0"), op);
    } else {
      throw std::runtime_error("adjoint: unsupported op in " + op.tag);
    }
  }
}

}  // namespace tdcc
