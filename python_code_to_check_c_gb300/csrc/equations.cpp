// The CCSD / CC2 right-hand sides as engine programs.
//
// Each builder emits the reference's terms (same index patterns, prefactors
// and antisymmetrisers; file:line on every builder) for one RK4 block.  Terms
// that depend only on that block's frozen inputs are accumulated into their
// own workspace slots, so Program::analyse() lifts them out of the four RK4
// stages (the reference recomputes them 4x per step).  Where a term is
// re-associated (same algebra, different contraction order) the comment
// gives the identity used.
#include <stdexcept>

#include "engine.h"

namespace tdcc {

namespace {

using P = Program;

Term T(double c, const View& a) { return Term{c, 0.0, a, View{}}; }
Term T2f(double c, const View& a, const View& b) { return Term{c, 0.0, a, b}; }

// tt[i,j,a,b] = t1[i,a] t1[j,b]
View make_tt(P& p, const View& t1, const char* nm) {
  View tt = p.ws(nm, "oovv");
  p.add(tt, false, {T2f(1.0, P::bc(t1, "ia", "ijab"), P::bc(t1, "jb", "ijab"))});
  return tt;
}

// tau1[m,n,a,b] = t1[m,a] t1[n,b] - t1[n,a] t1[m,b]   (CCSD_Helper.py:292)
View make_tau1(P& p, const View& t1, const char* nm) {
  View x = p.ws(nm, "oovv");
  p.add(x, false,
        {T2f(1.0, P::bc(t1, "ia", "ijab"), P::bc(t1, "jb", "ijab")),
         T2f(-1.0, P::bc(t1, "ib", "ijab"), P::bc(t1, "ja", "ijab"))});
  return x;
}

// Xg[m,e] = sum_nf <mn||ef> t1[n,f]  (so Fme = F_ov + Xg, CCSD_Helper.py:163-170)
View make_xg(P& p, const View& t1) {
  View xg = p.ws("Xg", "ov");
  p.ein("mnef,nf->me", 1.0, p.G("oovv"), t1, xg, false);
  return xg;
}

// Fme = F_ov + Xg (varies with the field through F)
View make_fme(P& p, const View& xg) {
  View fme = p.ws("Fme", "ov");
  p.add(fme, false, {T(1.0, p.Fb("ov")), T(1.0, xg)});
  return fme;
}

// ----- hoisted pieces of the CCSD/CC2 T2 equations that depend on t1 only --
// Wabef_2 (CCSD_Helper.py:240-252) and the t1-only terms of T2eq_rhs
// (term1, the Wmnij_2/Wabef_2 tau ladders, the t1 t1 ring, term7, term8;
// CCSD_Helper.py:284-306) into C2.
struct T2Const {
  View C2, tau1, tt;
};

// Particle-particle ladder with a Wabef built from the integrals and t1,
//   c * sum_ef Wx_abef X_ijef,
//   Wx = <ab||ef> + P(ab)[-<am||ef> t1_mb] + w <mn||ef> tau1_mnab,
// without forming the v^4 tensor Wx (same algebra, re-associated):
//   c <ab||ef> X_ijef  -  c P(ab) sum_m t1_mb U_ijam  +  c w sum_mn tau1_mnab Z_mnij
// with U_ijam = <am||ef> X_ijef (o^3 v^3) and Z_mnij = <mn||ef> X_ijef (o^4 v^2).
// The vvvv ladder runs on the integrals themselves, whose packed operand is
// a per-system constant.  Z is returned for reuse (Wmnij).
View ladder(P& p, const View& t1, const View& tau1, const View& X, double c, double w,
            const View& out, const char* tag) {
  p.ein("abef,ijef->ijab", c, p.G("vvvv"), X, out, true);
  View u = p.ws(std::string(tag) + "_U", "oovo");  // [i,j,a,m]
  p.ein("amef,ijef->ijam", 1.0, p.G("vovv"), X, u, false);
  View y = p.ws(std::string(tag) + "_Ut1", "oovv");
  p.ein("ijam,mb->ijab", -1.0, u, t1, y, false);
  p.acc_pab(out, y, c);
  View z = p.ws(std::string(tag) + "_Z", "oooo");
  p.ein("mnef,ijef->mnij", 1.0, p.G("oovv"), X, z, false);
  p.ein("mnij,mnab->ijab", c * w, z, tau1, out, true);
  return z;
}

T2Const build_t2_const(P& p, const View& t1) {
  T2Const r;
  r.tt = make_tt(p, t1, "tt");
  r.tau1 = make_tau1(p, t1, "tau1");
  // Wmnij_2 = <mn||ij> + P(ij)[<mn||ie> t1_je] + P(ij)[1/4 <mn||ef> tt_ijef]
  View wmnij2 = p.ws("Wmnij_2", "oooo");
  View y = p.ws("Wmnij_2_y", "oooo");
  p.ein("mnie,je->mnij", 1.0, p.G("ooov"), t1, y, false);
  p.ein("mnef,ijef->mnij", 0.25, p.G("oovv"), r.tt, y, true);
  p.add(wmnij2, false, {T(1.0, p.G("oooo")), T(1.0, y), T(-1.0, y.swap(2, 3))});
  // C2 = <ij||ab> + 1/2 Wmnij_2 tau1 + 1/2 Wabef_2 tau1 + ...
  // (Wabef_2 = <ab||ef> + P(ab)[-<am||ef> t1_mb] + 1/4 <mn||ef> tau1_mnab,
  //  CCSD_Helper.py:240-252, applied through `ladder`)
  r.C2 = p.ws("C2", "oovv");
  p.copy(r.C2, p.G("oovv"));
  p.ein("mnij,mnab->ijab", 0.5, wmnij2, r.tau1, r.C2, true);
  ladder(p, t1, r.tau1, r.tau1, 0.5, 0.25, r.C2, "L2t1");
  // ring with t1 t1: -P(ij)P(ab) sum_me <mb||ej> t1_ie t1_ma
  View rt = p.ws("ring_t1_a", "ovoo");  // [m,b,i,j]
  p.ein("mbej,ie->mbij", 1.0, p.G("ovvo"), t1, rt, false);
  View rc = p.ws("ring_t1", "oovv");
  p.ein("mbij,ma->ijab", -1.0, rt, t1, rc, false);
  p.acc_pijab(r.C2, rc);
  // term7: P(ij) <ab||ej> t1_ie ; term8: -P(ab) <mb||ij> t1_ma
  View t7 = p.ws("t2_term7", "oovv");
  p.ein("abej,ie->ijab", 1.0, p.G("vvvo"), t1, t7, false);
  p.acc_pij(r.C2, t7);
  View t8 = p.ws("t2_term8", "oovv");
  p.ein("mbij,ma->ijab", -1.0, p.G("ovoo"), t1, t8, false);
  p.acc_pab(r.C2, t8);
  return r;
}

}  // namespace

// ---------------------------------------------------------------------------
// T1 residual, CCSD and CC2 (CCSD_Helper.py:136-196).  Block T1: t1 and F vary.
// ---------------------------------------------------------------------------
void build_t1(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), out = p.out(2);
  // t2-only pieces (hoisted)
  View fae_c = p.ws("Fae_c", "vv");
  p.ein("mnef,mnaf->ae", -0.5, p.G("oovv"), t2, fae_c, false);
  View fmi_c = p.ws("Fmi_c", "oo");
  p.ein("mnef,inef->mi", 0.5, p.G("oovv"), t2, fmi_c, false);
  View c1 = p.ws("T1_c", "ov");
  p.ein("nmei,mnae->ia", -0.5, p.G("oovo"), t2, c1, false);
  p.ein("maef,imef->ia", -0.5, p.G("ovvv"), t2, c1, true);
  // Fme = F_ov + sum_nf <mn||ef> t1_nf
  View xg = make_xg(p, t1);
  View fme = make_fme(p, xg);
  // Fae = F_vv - 1/2 Fme^T t1 + <ma||fe> t1_mf - 1/2 <mn||ef> t2_mnaf
  //   (the t1 t1 part of tau: -1/2 sum_mnf <mn||ef> t1_ma t1_nf = -1/2 sum_m Xg_me t1_ma)
  View fae = p.ws("Fae", "vv");
  p.add(fae, false, {T(1.0, p.Fb("vv")), T(1.0, fae_c)});
  p.ein("me,ma->ae", -0.5, fme, t1, fae, true);
  p.ein("mafe,mf->ae", 1.0, p.G("ovvv"), t1, fae, true);
  // Fmi = F_oo + 1/2 Fme t1^T + <mn||ie> t1_ne + 1/2 <mn||ef> t2_inef
  View fmi = p.ws("Fmi", "oo");
  p.add(fmi, false, {T(1.0, p.Fb("oo")), T(1.0, fmi_c)});
  p.ein("me,ie->mi", 0.5, fme, t1, fmi, true);
  p.ein("mnie,ne->mi", 1.0, p.G("ooov"), t1, fmi, true);
  // T1 = f_ov + Fae t1 - Fmi t1 + Fme t2 - <na||if> t1_nf + (t2 terms)
  p.add(out, false, {T(1.0, p.Fb("ov")), T(1.0, c1)});
  p.ein("ae,ie->ia", 1.0, fae, t1, out, true);
  p.ein("mi,ma->ia", -1.0, fmi, t1, out, true);
  p.ein("me,imae->ia", 1.0, fme, t2, out, true);
  p.ein("naif,nf->ia", -1.0, p.G("ovov"), t1, out, true);
}

// ---------------------------------------------------------------------------
// CCSD T2 residual (CCSD_Helper.py:199-309).  Block T2: t2 and F vary.
// ---------------------------------------------------------------------------
void build_t2_ccsd(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), out = p.out(4);
  T2Const k = build_t2_const(p, t1);
  View xg = make_xg(p, t1);
  // Wmnij without its t2 term (CCSD_Helper.py:199-210):
  //   Wmnij_c = <mn||ij> + P(ij)[<mn||ie> t1_je] + 1/2 <mn||ef> tau1_ijef
  View wmn_c = p.ws("Wmnij_c", "oooo");
  View y = p.ws("Wmnij_c_y", "oooo");
  p.ein("mnie,je->mnij", 1.0, p.G("ooov"), t1, y, false);
  p.add(wmn_c, false, {T(1.0, p.G("oooo")), T(1.0, y), T(-1.0, y.swap(2, 3))});
  p.ein("mnef,ijef->mnij", 0.5, p.G("oovv"), k.tau1, wmn_c, true);
  // Wmbej without its t2 term (CCSD_Helper.py:255-265)
  View wmbej_c = p.ws("Wmbej_c", "ovvo");
  p.copy(wmbej_c, p.G("ovvo"));
  p.ein("mnej,nb->mbej", -1.0, p.G("oovo"), t1, wmbej_c, true);
  p.ein("mnef,jnfb->mbej", -1.0, p.G("oovv"), k.tt, wmbej_c, true);
  p.ein("mbef,jf->mbej", 1.0, p.G("ovvv"), t1, wmbej_c, true);
  // t1-only parts of Fae / Fmi (CCSD_Helper.py:136-160)
  View fae_c = p.ws("Fae_c", "vv");
  p.ein("mafe,mf->ae", 1.0, p.G("ovvv"), t1, fae_c, false);
  p.ein("me,ma->ae", -0.5, xg, t1, fae_c, true);
  View fmi_c = p.ws("Fmi_c", "oo");
  p.ein("mnie,ne->mi", 1.0, p.G("ooov"), t1, fmi_c, false);
  p.ein("me,ie->mi", 0.5, xg, t1, fmi_c, true);

  // ---- per stage (t2, F) ----
  View fme = make_fme(p, xg);
  // Fae = F_vv + Fae_c - 1/2 F_ov^T t1 - 1/2 <mn||ef> t2_mnaf
  View fae = p.ws("Fae", "vv");
  p.add(fae, false, {T(1.0, p.Fb("vv")), T(1.0, fae_c)});
  p.ein("me,ma->ae", -0.5, p.Fb("ov"), t1, fae, true);
  p.ein("mnef,mnaf->ae", -0.5, p.G("oovv"), t2, fae, true);
  // term2: P(ab) sum_e (Fae - 1/2 Fme t1)_be t2_ijae
  p.ein("me,mb->be", -0.5, fme, t1, fae, true);
  View x2 = p.ws("t2_term2", "oovv");
  p.ein("be,ijae->ijab", 1.0, fae, t2, x2, false);
  // Fmi = F_oo + Fmi_c + 1/2 F_ov t1^T + 1/2 <mn||ef> t2_inef
  View fmi = p.ws("Fmi", "oo");
  p.add(fmi, false, {T(1.0, p.Fb("oo")), T(1.0, fmi_c)});
  p.ein("me,ie->mi", 0.5, p.Fb("ov"), t1, fmi, true);
  p.ein("mnef,inef->mi", 0.5, p.G("oovv"), t2, fmi, true);
  // term3: -P(ij) sum_m (Fmi + 1/2 Fme t1)_mj t2_imab
  p.ein("me,je->mj", 0.5, fme, t1, fmi, true);
  View x3 = p.ws("t2_term3", "oovv");
  p.ein("mj,imab->ijab", -1.0, fmi, t2, x3, false);
  // ring: Wmbej = Wmbej_c - 1/2 <mn||ef> t2_jnfb ; P(ij)P(ab) Wmbej t2_imae
  View wmbej = p.ws("Wmbej", "ovvo");
  p.copy(wmbej, wmbej_c);
  p.ein("mnef,jnfb->mbej", -0.5, p.G("oovv"), t2, wmbej, true);
  View ring = p.ws("t2_ring", "oovv");
  p.ein("mbej,imae->ijab", 1.0, wmbej, t2, ring, false);
  // assemble
  p.copy(out, k.C2);
  p.acc_pab(out, x2);
  p.acc_pij(out, x3);
  // particle-particle ladder 1/2 Wabef t2 (CCSD_Helper.py:227-238, 294) with
  //   Wabef = <ab||ef> + P(ab)[-<am||ef> t1_mb] + 1/2 <mn||ef> tau1_mnab
  //           + 1/4 <mn||ef> t2_mnab;
  // the last piece gives 1/8 sum_mn Z_mnij t2_mnab, Z_mnij = <mn||ef> t2_ijef,
  // which joins term44: 1/2 Wmnij t2 with Wmnij = Wmnij_c + Z/4, so
  //   term44 + that = 1/2 (Wmnij_c + Z/2) t2.
  View z = ladder(p, t1, k.tau1, t2, 0.5, 0.5, out, "L2t2");
  View wtot = p.ws("Wmnij_tot", "oooo");
  p.add(wtot, false, {T(1.0, wmn_c), T(0.5, z)});
  p.ein("mnij,mnab->ijab", 0.5, wtot, t2, out, true);
  p.acc_pijab(out, ring);
}

// ---------------------------------------------------------------------------
// CC2 T2 residual (CC2_Helper.py:12-47).  Block T2: t2 and F vary.
// ---------------------------------------------------------------------------
void build_t2_cc2(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), out = p.out(4);
  T2Const k = build_t2_const(p, t1);
  View x2 = p.ws("t2_term2", "oovv");
  p.ein("be,ijae->ijab", 1.0, p.Fb("vv"), t2, x2, false);
  View x3 = p.ws("t2_term3", "oovv");
  p.ein("mj,imab->ijab", -1.0, p.Fb("oo"), t2, x3, false);
  p.copy(out, k.C2);
  p.acc_pab(out, x2);
  p.acc_pij(out, x3);
}

// ---------------------------------------------------------------------------
// Lambda Hbar pieces that depend on t1, t2 only (CCSD_Helper.py:447-550,
// 586-607).  Shared by the CCSD Lambda builders.
// ---------------------------------------------------------------------------
namespace {
struct LamConst {
  View xg, tt, tauq, fea_c, fim_c, wieam, wmnij, wfiea, wmina;
};

// LSWabef (CCSD_Helper.py:598-607) is never formed: its two uses are
// re-associated where they occur (lsw_ladder, and term3 of LRWefam).
LamConst build_lam_const(P& p, const View& t1, const View& t2) {
  LamConst r;
  r.xg = make_xg(p, t1);
  r.tt = make_tt(p, t1, "tt");
  // tau_h = 1/2 t2 + tt  (LRFea / LRFim)
  View tauh = p.ws("tau_h", "oovv");
  p.add(tauh, false, {T(0.5, t2), T(1.0, r.tt)});
  // LRFea without F: <em||af> t1_mf - <mn||af> tau_h_mnef  (CCSD_Helper.py:447-459)
  r.fea_c = p.ws("LRFea_c", "vv");
  p.ein("emaf,mf->ea", 1.0, p.G("vovv"), t1, r.fea_c, false);
  p.ein("mnaf,mnef->ea", -1.0, p.G("oovv"), tauh, r.fea_c, true);
  // LRFim without F: <in||mf> t1_nf + <in||ef> tau_h_mnef  (CCSD_Helper.py:462-472)
  r.fim_c = p.ws("LRFim_c", "oo");
  p.ein("inmf,nf->im", 1.0, p.G("ooov"), t1, r.fim_c, false);
  p.ein("inef,mnef->im", 1.0, p.G("oovv"), tauh, r.fim_c, true);
  // LSWieam (CCSD_Helper.py:475-485)
  View tau_f = p.ws("tau_full", "oovv");
  p.add(tau_f, false, {T(1.0, t2), T(1.0, r.tt)});
  r.wieam = p.ws("LSWieam", "ovvo");
  p.copy(r.wieam, p.G("ovvo"));
  p.ein("eifa,mf->ieam", 1.0, p.G("vovv"), t1, r.wieam, true);
  p.ein("nima,ne->ieam", -1.0, p.G("ooov"), t1, r.wieam, true);
  p.ein("ijab,mjbe->ieam", -1.0, p.G("oovv"), tau_f, r.wieam, true);
  // tau_q = 1/4 t2 + 1/2 tt  (LSWmnij, LSWabef, LRWefam, LRWibjm)
  r.tauq = p.ws("tau_q", "oovv");
  p.add(r.tauq, false, {T(0.25, t2), T(0.5, r.tt)});
  // LSWmnij (CCSD_Helper.py:586-595)
  r.wmnij = p.ws("LSWmnij", "oooo");
  p.copy(r.wmnij, p.G("oooo"), 0.5);
  p.ein("ijme,ne->ijmn", 1.0, p.G("ooov"), t1, r.wmnij, true);
  p.ein("ijfe,mnfe->ijmn", 1.0, p.G("oovv"), r.tauq, r.wmnij, true);
  // LWfiea, LWmina (CCSD_Helper.py:533-550)
  r.wfiea = p.ws("LWfiea", "vovv");
  p.copy(r.wfiea, p.G("vovv"));
  p.ein("jiea,jf->fiea", -1.0, p.G("oovv"), t1, r.wfiea, true);
  r.wmina = p.ws("LWmina", "ooov");
  p.copy(r.wmina, p.G("ooov"));
  p.ein("mifa,nf->mina", 1.0, p.G("oovv"), t1, r.wmina, true);
  return r;
}

// LRFea / LRFim with the field: F_vv - F_ov^T t1 + c ; F_oo + F_ov t1^T + c
View make_lrfea(P& p, const View& t1, const View& fea_c) {
  View f = p.ws("LRFea", "vv");
  p.add(f, false, {T(1.0, p.Fb("vv")), T(1.0, fea_c)});
  p.ein("ma,me->ea", -1.0, p.Fb("ov"), t1, f, true);
  return f;
}
View make_lrfim(P& p, const View& t1, const View& fim_c) {
  View f = p.ws("LRFim", "oo");
  p.add(f, false, {T(1.0, p.Fb("oo")), T(1.0, fim_c)});
  p.ein("ie,me->im", 1.0, p.Fb("ov"), t1, f, true);
  return f;
}
}  // namespace

// ---------------------------------------------------------------------------
// CCSD Lambda1 residual (CCSD_Helper.py:488-581).  Block L1: l1 and F vary.
// ---------------------------------------------------------------------------
void build_l1_ccsd(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), l1 = p.amp(S_L1), l2 = p.amp(S_L2);
  const View out = p.out(2);
  LamConst k = build_lam_const(p, t1, t2);
  const View tauq = k.tauq;
  // LRWefam without its Fme term (CCSD_Helper.py:488-505)
  View wefam = p.ws("LRWefam_c", "vvvo");
  p.copy(wefam, p.G("vvvo"), 0.5);
  // term3  sum_b LSWabef_efab t1_mb  with LSWabef = 1/2 <ef||ab>
  //   - <em||ab> t1_mf + <nm||ab> tau_q_nmef  (CCSD_Helper.py:598-607), re-associated:
  //   1/2 <ef||ab> t1_mb  -  sum_x t1_xf Q_exam  +  sum_nk tau_q_nkef R_nkam,
  //   Q_exam = <ex||ab> t1_mb,  R_nkam = <nk||ab> t1_mb
  p.ein("efab,mb->efam", 0.5, p.G("vvvv"), t1, wefam, true);
  View q3 = p.ws("LRWefam_Q", "vovo");
  p.ein("exab,mb->exam", 1.0, p.G("vovv"), t1, q3, false);
  p.ein("exam,xf->efam", -1.0, q3, t1, wefam, true);
  View r3 = p.ws("LRWefam_R", "oovo");
  p.ein("nkab,mb->nkam", 1.0, p.G("oovv"), t1, r3, false);
  p.ein("nkef,nkam->efam", 1.0, tauq, r3, wefam, true);
  View jfam = p.ws("LRWefam_jfam", "ovvo");
  p.copy(jfam, p.G("ovvo"), -1.0);
  p.ein("jnab,nmfb->jfam", 1.0, p.G("oovv"), t2, jfam, true);
  p.ein("jfam,je->efam", 1.0, jfam, t1, wefam, true);
  p.ein("jnam,jnef->efam", 1.0, p.G("oovo"), tauq, wefam, true);
  p.ein("jfab,jmeb->efam", -1.0, p.G("ovvv"), t2, wefam, true);
  // LRWibjm without its Fme term (CCSD_Helper.py:508-524)
  View wibjm = p.ws("LRWibjm_c", "ovoo");
  p.copy(wibjm, p.G("ovoo"), -0.5);
  p.ein("injm,nb->ibjm", 1.0, k.wmnij, t1, wibjm, true);
  View ibem = p.ws("LRWibjm_ibem", "ovvo");
  p.copy(ibem, p.G("ovvo"), -1.0);
  p.ein("inef,nmfb->ibem", -1.0, p.G("oovv"), t2, ibem, true);
  p.ein("ibem,je->ibjm", 1.0, ibem, t1, wibjm, true);
  p.ein("ibef,jmef->ibjm", -1.0, p.G("ovvv"), tauq, wibjm, true);
  p.ein("inem,jneb->ibjm", 1.0, p.G("oovo"), t2, wibjm, true);
  // G intermediates (CCSD_Helper.py:526-530)
  View gfe = p.ws("Gfe", "vv");
  p.ein("mnfb,mneb->fe", -0.5, l2, t2, gfe, false);
  View gmn = p.ws("Gmn", "oo");
  p.ein("njed,mjed->nm", 0.5, l2, t2, gmn, false);
  // Fme terms of LRWefam / LRWibjm contracted with l2, re-associated:
  //   sum_efm (1/2 sum_n Fme_na t2_mnef) l2_imef = 1/2 sum_n Fme_na H_ni,
  //     H_ni = sum_mef t2_mnef l2_imef
  //   sum_bjm (1/2 sum_e Fme_ie t2_jmbe) l2_jmab = 1/2 sum_e Fme_ie K_ea,
  //     K_ea = sum_jmb t2_jmbe l2_jmab
  View hni = p.ws("H_ni", "oo");
  p.ein("mnef,imef->ni", 1.0, t2, l2, hni, false);
  View kea = p.ws("K_ea", "vv");
  p.ein("jmbe,jmab->ea", 1.0, t2, l2, kea, false);
  // l1-independent part of the residual
  View cl1 = p.ws("L1_c", "ov");
  p.copy(cl1, k.xg);
  p.ein("efam,imef->ia", 1.0, wefam, l2, cl1, true);
  p.ein("ibjm,jmab->ia", 1.0, wibjm, l2, cl1, true);
  p.ein("fe,fiea->ia", -1.0, gfe, k.wfiea, cl1, true);
  p.ein("nm,mina->ia", -1.0, gmn, k.wmina, cl1, true);

  // ---- per stage (l1, F) ----
  View fme = make_fme(p, k.xg);
  View fea = make_lrfea(p, t1, k.fea_c);
  View fim = make_lrfim(p, t1, k.fim_c);
  p.add(out, false, {T(1.0, p.Fb("ov")), T(1.0, cl1)});
  p.ein("ea,ie->ia", 1.0, fea, l1, out, true);
  p.ein("im,ma->ia", -1.0, fim, l1, out, true);
  p.ein("ieam,me->ia", 1.0, k.wieam, l1, out, true);
  p.ein("na,ni->ia", 0.5, fme, hni, out, true);
  p.ein("ie,ea->ia", 0.5, fme, kea, out, true);
}

// ---------------------------------------------------------------------------
// CCSD Lambda2 residual (CCSD_Helper.py:610-648).  Block L2: l2 and F vary.
// ---------------------------------------------------------------------------
void build_l2_ccsd(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), l1 = p.amp(S_L1), l2 = p.amp(S_L2);
  const View out = p.out(4);
  LamConst k = build_lam_const(p, t1, t2);
  // l2-independent part: <ij||ab> + P(ij) Wejab l1 - P(ab) Wijmb l1
  //   + P(ij)P(ab) Xg_jb l1_ia  (the t1 part of Fme (x) l1)
  View cl2 = p.ws("L2_c", "oovv");
  p.copy(cl2, p.G("oovv"));
  View x6 = p.ws("l2_term6", "oovv");
  p.ein("ejab,ie->ijab", 1.0, k.wfiea, l1, x6, false);
  p.acc_pij(cl2, x6);
  View x7 = p.ws("l2_term7", "oovv");
  p.ein("ijmb,ma->ijab", -1.0, k.wmina, l1, x7, false);
  p.acc_pab(cl2, x7);
  View xo = p.ws("l2_xg_l1", "oovv");
  p.add(xo, false, {T2f(1.0, P::bc(k.xg, "jb", "ijab"), P::bc(l1, "ia", "ijab"))});
  p.acc_pijab(cl2, xo);

  // ---- per stage (l2, F) ----
  View fea = make_lrfea(p, t1, k.fea_c);
  View fim = make_lrfim(p, t1, k.fim_c);
  View gbe = p.ws("Gfe", "vv");
  p.ein("mnfb,mneb->fe", -0.5, l2, t2, gbe, false);
  View gmj = p.ws("Gmn", "oo");
  p.ein("njed,mjed->nm", 0.5, l2, t2, gmj, false);
  View x2 = p.ws("l2_term2", "oovv");
  p.ein("eb,ijae->ijab", 1.0, fea, l2, x2, false);
  p.ein("ijfb,af->ijab", 1.0, p.G("oovv"), gbe, x2, true);  // term10 shares P(ab)
  View x3 = p.ws("l2_term3", "oovv");
  p.ein("jm,imab->ijab", -1.0, fim, l2, x3, false);
  p.ein("mjab,im->ijab", -1.0, p.G("oovv"), gmj, x3, true);  // term11 shares P(ij)
  // term89: P(ij)P(ab) [Wjebm l2_imae + F_ov,jb l1_ia]
  View x89 = p.ws("l2_ring", "oovv");
  p.ein("jebm,imae->ijab", 1.0, k.wieam, l2, x89, false);
  p.add(x89, true, {T2f(1.0, P::bc(p.Fb("ov"), "jb", "ijab"), P::bc(l1, "ia", "ijab"))});
  p.copy(out, cl2);
  p.acc_pab(out, x2);
  p.acc_pij(out, x3);
  p.ein("ijmn,mnab->ijab", 1.0, k.wmnij, l2, out, true);
  // particle-particle ladder sum_ef LSWabef_efab l2_ijef (term5) with
  //   LSWabef = 1/2 <ef||ab> - <em||ab> t1_mf + <nm||ab> tau_q_nmef,
  // re-associated so the v^4 tensor is never formed:
  //   1/2 <ef||ab> l2_ijef - <em||ab> Y_ijem + <nm||ab> Zq_nmij,
  //   Y_ijem = t1_mf l2_ijef,  Zq_nmij = tau_q_nmef l2_ijef
  p.ein("efab,ijef->ijab", 0.5, p.G("vvvv"), l2, out, true);
  View yl = p.ws("l2_Y", "oovo");
  p.ein("mf,ijef->ijem", 1.0, t1, l2, yl, false);
  p.ein("emab,ijem->ijab", -1.0, p.G("vovv"), yl, out, true);
  View zq = p.ws("l2_Zq", "oooo");
  p.ein("nmef,ijef->nmij", 1.0, k.tauq, l2, zq, false);
  p.ein("nmab,nmij->ijab", 1.0, p.G("oovv"), zq, out, true);
  p.acc_pijab(out, x89);
}

// ---------------------------------------------------------------------------
// CC2 Lambda1 residual (CC2_Helper.py:50-125).  Block L1: l1 and F vary.
// ---------------------------------------------------------------------------
void build_l1_cc2(P& p) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), l1 = p.amp(S_L1), l2 = p.amp(S_L2);
  const View out = p.out(2);
  View xg = make_xg(p, t1);
  View tt = make_tt(p, t1, "tt");
  View tau = make_tau1(p, t1, "tau1");
  // LRFea / LRFim without F (same pieces as CCSD)
  View tauh = p.ws("tau_h", "oovv");
  p.add(tauh, false, {T(0.5, t2), T(1.0, tt)});
  View fea_c = p.ws("LRFea_c", "vv");
  p.ein("emaf,mf->ea", 1.0, p.G("vovv"), t1, fea_c, false);
  p.ein("mnaf,mnef->ea", -1.0, p.G("oovv"), tauh, fea_c, true);
  View fim_c = p.ws("LRFim_c", "oo");
  p.ein("inmf,nf->im", 1.0, p.G("ooov"), t1, fim_c, false);
  p.ein("inef,mnef->im", 1.0, p.G("oovv"), tauh, fim_c, true);
  // Wmbej (t1 only, CC2_Helper.py:73-77)
  View wmbej = p.ws("Wmbej_cc2", "ovvo");
  p.copy(wmbej, p.G("ovvo"));
  p.ein("mbef,jf->mbej", 1.0, p.G("ovvv"), t1, wmbej, true);
  p.ein("mnej,nb->mbej", -1.0, p.G("oovo"), t1, wmbej, true);
  p.ein("mnef,jnfb->mbej", -1.0, p.G("oovv"), tt, wmbej, true);
  // Wmnij, Wmbij (CC2_Helper.py:89-104)
  View wmnij = p.ws("Wmnij_cc2", "oooo");
  p.copy(wmnij, p.G("oooo"));
  p.ein("mnie,je->mnij", 1.0, p.G("ooov"), t1, wmnij, true);
  p.ein("mnje,ie->mnij", -1.0, p.G("ooov"), t1, wmnij, true);
  p.ein("ijef,mnfe->ijmn", -0.5, p.G("oovv"), tau, wmnij, true);
  View wmbij = p.ws("Wmbij_cc2", "ovoo");
  p.copy(wmbij, p.G("ovoo"));
  p.ein("nb,mnij->mbij", -1.0, t1, wmnij, wmbij, true);
  p.ein("mbef,ijef->mbij", 0.5, p.G("ovvv"), tau, wmbij, true);
  p.ein("mbei,je->mbij", -1.0, p.G("ovvo"), t1, wmbij, true);
  p.ein("mbej,ie->mbij", 1.0, p.G("ovvo"), t1, wmbij, true);
  // Zmbej, Wabei (CC2_Helper.py:107-122)
  View zmbej = p.ws("Zmbej_cc2", "ovvo");
  p.copy(zmbej, p.G("ovvo"));
  p.ein("mbef,jf->mbej", 1.0, p.G("ovvv"), t1, zmbej, true);
  p.ein("mnej,nb->mbej", -0.5, p.G("oovo"), t1, zmbej, true);
  p.ein("mnef,jnfb->mbej", -0.5, p.G("oovv"), tt, zmbej, true);
  View wabei = p.ws("Wabei_cc2", "vvvo");
  p.copy(wabei, p.G("vvvo"));
  p.ein("abef,if->abei", 1.0, p.G("vvvv"), t1, wabei, true);
  p.ein("maei,mb->abei", 1.0, zmbej, t1, wabei, true);
  p.ein("mbei,ma->abei", -1.0, zmbej, t1, wabei, true);
  // l1-independent part: Xg - 1/2 Wmbij l2 + 1/2 Wabei l2
  View cl1 = p.ws("L1_c", "ov");
  p.copy(cl1, xg);
  p.ein("iemn,mnae->ia", -0.5, wmbij, l2, cl1, true);
  p.ein("efam,imef->ia", 0.5, wabei, l2, cl1, true);

  // ---- per stage (l1, F) ----
  View fea = make_lrfea(p, t1, fea_c);
  View fim = make_lrfim(p, t1, fim_c);
  View gbj = p.ws("Gbj", "vo");
  p.ein("me,mjbe->bj", -1.0, l1, t2, gbj, false);
  p.add(out, false, {T(1.0, p.Fb("ov")), T(1.0, cl1)});
  p.ein("ea,ie->ia", 1.0, fea, l1, out, true);
  p.ein("im,ma->ia", -1.0, fim, l1, out, true);
  p.ein("ijab,bj->ia", 1.0, p.G("oovv"), gbj, out, true);
  p.ein("ieam,me->ia", 1.0, wmbej, l1, out, true);
}

// ---------------------------------------------------------------------------
// CC2 Lambda2 residual (CC2_Helper.py:128-175).  Block L2: l2 and F vary.
// ---------------------------------------------------------------------------
void build_l2_cc2(P& p, const View& ones_v) {
  const View t1 = p.amp(S_T1), l1 = p.amp(S_L1), l2 = p.amp(S_L2);
  const View out = p.out(4);
  View xg = make_xg(p, t1);
  View wmina = p.ws("LWmina", "ooov");
  p.copy(wmina, p.G("ooov"));
  p.ein("mifa,nf->mina", 1.0, p.G("oovv"), t1, wmina, true);
  View weifa = p.ws("LWfiea", "vovv");
  p.copy(weifa, p.G("vovv"));
  p.ein("jiea,jf->fiea", -1.0, p.G("oovv"), t1, weifa, true);
  // l2-independent part
  View cl2 = p.ws("L2_c", "oovv");
  p.copy(cl2, p.G("oovv"));
  p.ein("ijmb,ma->ijab", -1.0, wmina, l1, cl2, true);
  p.ein("ijmb,ma->ijba", 1.0, wmina, l1, cl2, true);
  p.ein("ejab,ie->ijab", 1.0, weifa, l1, cl2, true);
  p.ein("ejab,ie->jiab", -1.0, weifa, l1, cl2, true);

  // ---- per stage (l2, F) ----
  // 'ijab,eb->ijab' sums e over F_vv alone: s_b = sum_e F_eb (CC2_Helper.py:139-140)
  View s = p.ws("Fvv_colsum", "v");
  p.ein("eb,e->b", 1.0, p.Fb("vv"), ones_v, s, false);
  View fme = make_fme(p, xg);
  p.add(out, false,
        {T(1.0, cl2), T2f(1.0, l2, P::bc(s, "b", "ijab")),
         T2f(-1.0, l2.swap(2, 3), P::bc(s, "a", "ijab"))});
  p.ein("imab,jm->ijab", -1.0, l2, p.Fb("oo"), out, true);
  p.ein("imab,jm->jiab", 1.0, l2, p.Fb("oo"), out, true);
  // P(ij)P(ab) l1_ia Fme_jb (CC2_Helper.py:168-171)
  View x = p.ws("l2_l1fme", "oovv");
  p.add(x, false, {T2f(1.0, P::bc(l1, "ia", "ijab"), P::bc(fme, "jb", "ijab"))});
  p.acc_pijab(out, x);
}

// ---------------------------------------------------------------------------
// Correlated density and dipole trace (CCSD_Helper.py:984-1006, 1066-1092)
// ---------------------------------------------------------------------------
void build_density(P& p, int n_mu) {
  const View t1 = p.amp(S_T1), t2 = p.amp(S_T2), l1 = p.amp(S_L1), l2 = p.amp(S_L2);
  View dij = p.ws("Dij", "oo");
  p.ein("je,ie->ij", -1.0, l1, t1, dij, false);
  p.ein("jmea,imea->ij", -0.5, l2, t2, dij, true);
  View dab = p.ws("Dab", "vv");
  p.ein("nb,na->ab", 1.0, l1, t1, dab, false);
  p.ein("mneb,mnea->ab", 0.5, l2, t2, dab, true);
  View dai = p.ws("Dai", "vo");
  p.copy(dai, t1.swap(0, 1));
  p.ein("me,miea->ai", 1.0, l1, t2, dai, true);
  View x1 = p.ws("Dai_x1", "vv");  // [a,e] = sum_m l1_me t1_ma
  p.ein("me,ma->ae", 1.0, l1, t1, x1, false);
  p.ein("ae,ie->ai", -1.0, x1, t1, dai, true);
  View x2 = p.ws("Dai_x2", "vv");  // [e,a] = sum_mnf l2_mnef t2_mnaf
  p.ein("mnef,mnaf->ea", 1.0, l2, t2, x2, false);
  p.ein("ea,ie->ai", -0.5, x2, t1, dai, true);
  View x3 = p.ws("Dai_x3", "oo");  // [m,i] = sum_nef l2_mnef t2_inef
  p.ein("mnef,inef->mi", 1.0, l2, t2, x3, false);
  p.ein("mi,ma->ai", -0.5, x3, t1, dai, true);
  p.trace(n_mu, dij, l1, dai, dab);
}

}  // namespace tdcc
