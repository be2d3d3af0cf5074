// deb_adjoint.cuh -- discrete adjoint (reverse mode) of the Rodas5 solve of
// one k-mode on its recorded step sequence: d L / d theta for a cotangent of
// the 20 output fields at every output time.  Host/device code like
// deb_core.cuh: the CUDA kernel runs it with one warp per (seed, mode) item,
// the test suite compiles it for the host.
//
// What is differentiated.  The reference differentiates its solve with
// jax.jacfwd (perturbations.py:765, DirectAdjoint; compute_matter_power in
// the notebooks).  diffrax's PID controller stops gradients through the step
// factor, so every step time is tau_start(theta) times a frozen number, and
// steps clipped to an output follow tau_out(theta).  That map -- tau_start,
// ICs, the accepted Rodas5 steps (ode_integrators_stiff.py:718-834) on the
// scaled recorded times, SaveAt linear interpolation and the output fields
// (perturbations.py:374-523) -- is what this file transposes.
//
// The step adjoint.  A Rodas5 step solves W k_s = f(t_s, u_s) + sum_q C_sq/h
// k_q + h d_s f_t with W = I/(gamma h) - J(t0, y0); the reverse sweep over
// the eight stages needs
//   * W^-T: the structured factors of the forward step reused transposed
//     (chain multipliers shifted by one element, the 8x8 core inverse
//     transposed, Woodbury with the roles of the rank-2 columns and rows
//     swapped);
//   * J(t_s, u_s)^T r at every stage point (transposed hierarchy couplings,
//     the lead rows through an inverse of their table, the metric functionals
//     h' and eta' as rank-1 terms);
//   * derivatives of r^T f(t, Y) in a, t and theta at fixed r, Y, and, for
//     the J(y0) inside W, second derivatives in a.
// The RHS is linear in every state variable but a (f = [g(a); A(a, t) y~]),
// so r^T f(t, Y) = Phi(zeta; B(r, Y)): B is a short bilinear form of r and Y
// (about 60 numbers, one O(n) pass) and Phi a scalar function of the
// coefficients zeta = (a, t, table values at a).  d/da and d/dt come from
// jets (forward-mode numbers, second order where needed); d/dtheta_p from
// evaluating Phi with the theta_p +- eps_p tables, one table set per lane.
// The theta-dependence of tau_start, the ICs and tau_out is taken by central
// differences of those scalar maps over the same table sets.
#pragma once

#include "deb_core.cuh"

namespace deb {

constexpr int NFIELD = 20;   // output fields per output time

// ------------------------------------------------------------------ jets
// Jet<double>: value and one derivative; Jet<Jet<double>>: two directions
// and their mixed second derivative.
template <class T>
struct Jet {
  T v, d;
  HD Jet() : v(0.0), d(0.0) {}
  HD Jet(double c) : v(c), d(0.0) {}
  HD Jet(const T& a, const T& b) : v(a), d(b) {}
};
template <class T> HD Jet<T> operator+(const Jet<T>& a, const Jet<T>& b) { return Jet<T>(a.v + b.v, a.d + b.d); }
template <class T> HD Jet<T> operator-(const Jet<T>& a, const Jet<T>& b) { return Jet<T>(a.v - b.v, a.d - b.d); }
template <class T> HD Jet<T> operator-(const Jet<T>& a) { return Jet<T>(-a.v, -a.d); }
template <class T> HD Jet<T> operator*(const Jet<T>& a, const Jet<T>& b) { return Jet<T>(a.v * b.v, a.d * b.v + a.v * b.d); }
template <class T> HD Jet<T> operator+(const Jet<T>& a, double b) { return Jet<T>(a.v + b, a.d); }
template <class T> HD Jet<T> operator+(double a, const Jet<T>& b) { return Jet<T>(a + b.v, b.d); }
template <class T> HD Jet<T> operator-(const Jet<T>& a, double b) { return Jet<T>(a.v - b, a.d); }
template <class T> HD Jet<T> operator-(double a, const Jet<T>& b) { return Jet<T>(a - b.v, -b.d); }
template <class T> HD Jet<T> operator*(const Jet<T>& a, double b) { return Jet<T>(a.v * b, a.d * b); }
template <class T> HD Jet<T> operator*(double a, const Jet<T>& b) { return Jet<T>(a * b.v, a * b.d); }
HD double jexp(double x) { return exp(x); }
HD double jlog(double x) { return log(x); }
HD double jrcp(double x) { return rcp(x); }
HD double jrsqrt(double x) { return rsqrt_(x); }
template <class T> HD Jet<T> jexp(const Jet<T>& a) { const T e = jexp(a.v); return Jet<T>(e, e * a.d); }
template <class T> HD Jet<T> jlog(const Jet<T>& a) { return Jet<T>(jlog(a.v), a.d * jrcp(a.v)); }
template <class T> HD Jet<T> jrcp(const Jet<T>& a) { const T r = jrcp(a.v); return Jet<T>(r, -(r * r) * a.d); }
template <class T> HD Jet<T> jrsqrt(const Jet<T>& a) {
  const T r = jrsqrt(a.v);
  return Jet<T>(r, (-0.5) * (r * r * r) * a.d);
}
template <class S> HD S jsqrt(const S& x) { return x * jrsqrt(x); }   // x > 0
template <class T> HD double val(const Jet<T>& x) { return val(x.v); }
HD double dpart(double x) { return x; }
HD double dpart(const Jet<double>& x) { return x.d; }
// derivative of a Jet<double>, mixed second derivative of a Jet<Jet<double>>
HD double d1(const Jet<double>& x) { return x.d; }
HD double d12(const Jet<Jet<double>>& x) { return x.d.d; }

// natural spline value on a given interval (the index from spl_locate)
template <class S> HD S spl_eval_at(const Spl& s, int i, const S& x) {
  const double* cf = s.c + 4 * i;
  const S u = x - LDG(s.x + i);
  return LDG(cf) + u * (LDG(cf + 1) + u * (LDG(cf + 2) + u * LDG(cf + 3)));
}
template <class S> HD S spl_eval_j(const Spl& s, const S& x) { return spl_eval_at(s, spl_locate(s, val(x)), x); }

// ------------------------------------------------------------------ coefficients of the RHS at (a, t)
// Everything of f(t, Y) for rows >= 1 that is not a state element: the
// lead-row scalars, the coefficients of the metric functionals
//   h'   = sum_m ch_m Yh_m + xh S_1/v,   Yh = Y[2, 3, 5, 7, ir, n-2]
//   eta' = sum_m ce_m Ye_m + xe fnu,     Ye = Y[4, 6, 8, ir+1, n-1]
//   P1   = sum_m cp_m Yp_m + xp (S_1/v + S_v),  Yp = Y[3, 5, 7, ir, n-2, n-1]
// (P1 = dgrho + 3 dgpres; S_1/v = sum_q w_q Y_0q / v_q, S_v = sum_q w_q Y_0q v_q,
// fnu = sum_q w_q Y_1q, v_q = 1 / sqrt(1 + (mu / q)^2), mu = a m_nu), the
// photon opacity, 1/tau and mu - mu0.
template <class S>
struct Coef {
  S sg[NSIG];
  S ch[6], ce[5], cp[6], xh, xe, xp;
  S opac, itau, dmu;
};

// Coefficients at (a, t) for the cosmology (c, m).  The three splines are
// evaluated at log a of this blob; mu0 is the expansion point of the
// per-momentum sums (the nominal mu of the bilinear form).
template <class S>
HD Coef<S> coef(const Cosmo& c, const ModeConst& m, const Dims& D, const S& a, const S& t, double mu0) {
  Coef<S> C;
  const S ia = jrcp(a), ia2 = ia * ia, a2 = a * a, la = jlog(a);
  const S cs2a = spl_eval_j(c.sp[SP_CS2A_LOGA], la), xe = spl_eval_j(c.sp[SP_XE_LOGA], la);
  const S rhonu = jexp(spl_eval_j(c.sp[SP_LRHONU_LOGA], la));
  const S rhoQ = jexp(m.pQ * la + 3.0 * (a - 1.0) * m.wa);
  const S grho = m.gOm * ia + (m.grr + m.grM * rhonu) * ia2 + m.gODE * rhoQ * a2 + m.gOk;
  const S g3 = grho * (1.0 / 3.0);
  const S iaH = jrsqrt(g3), aH = g3 * iaH;
  const S wQ = m.w0 + m.wa * (1.0 - a);
  const S wQp = (-m.wa) * aH * a;
  const S ca2 = wQ - wQp * (1.0 / 3.0) * jrcp((1.0 + wQ) + 1e-6) * iaH;
  const S opac = xe * m.akthom * ia2;
  const S pb43 = m.pb43c * ia;
  const S cs2 = cs2a * ia;
  const S rQ = m.gODE * rhoQ * a2;
  const S w1 = 1.0 + wQ;
  const S itau = jrcp(t);
  const double k = m.k, k2 = m.k2;
  C.sg[SG_ONE] = S(1.0); C.sg[SG_K] = S(k); C.sg[SG_K2] = S(k2); C.sg[SG_OP] = opac; C.sg[SG_AH] = aH; C.sg[SG_A] = a;
  C.sg[SG_AHA] = aH * a; C.sg[SG_KCS] = k2 * cs2; C.sg[SG_PBO] = pb43 * opac;
  C.sg[SG_ITG] = (-(D.lg + 1.0)) * itau; C.sg[SG_ITP] = (-(D.lgp + 1.0)) * itau; C.sg[SG_ITR] = (-(D.lr + 1.0)) * itau;
  C.sg[SG_W1] = w1; C.sg[SG_DE1] = 3.0 * (m.cs2Q - wQ) * aH;
  C.sg[SG_DE2] = 9.0 * w1 * (m.cs2Q - ca2) * aH * aH * m.ik2; C.sg[SG_DE3] = (1.0 - 3.0 * m.cs2Q) * aH;
  C.sg[SG_DE4] = m.cs2Q * jrcp(w1) * k2;
  const double h2 = 0.5 * m.ik2;
  C.ch[0] = 2.0 * k2 * iaH; C.ch[1] = m.gOc * ia * iaH; C.ch[2] = m.gOb * ia * iaH; C.ch[3] = m.grhog * ia2 * iaH;
  C.ch[4] = m.grN * ia2 * iaH; C.ch[5] = rQ * iaH;
  C.ce[0] = m.gOc * ia * h2; C.ce[1] = m.gOb * ia * h2; C.ce[2] = m.g43g * ia2 * h2; C.ce[3] = m.g43N * ia2 * h2;
  C.ce[4] = w1 * rQ * h2;
  C.cp[0] = m.gOc * ia; C.cp[1] = m.gOb * ia; C.cp[2] = 2.0 * m.grhog * ia2; C.cp[3] = 2.0 * m.grN * ia2;
  C.cp[4] = (1.0 + 3.0 * m.cs2Q) * rQ; C.cp[5] = 9.0 * (m.cs2Q - ca2) * aH * w1 * rQ * m.ik2;
  C.xh = m.grM * ia2 * iaH; C.xe = m.grMk * ia2 * h2; C.xp = m.grM * ia2;
  C.opac = opac; C.itau = itau; C.dmu = a * m.amnu - mu0;
  return C;
}

// ------------------------------------------------------------------ the bilinear form B(r, Y)
enum { B_SIG = 0, B_OP = NSIG, B_FREE, B_V, B_IT = B_V + 3, B_H1, B_H1T = B_H1 + 6, B_HW = B_H1T + 3, B_HWT = B_HW + 6,
       B_E = B_HWT + 3, B_EF = B_E + 5, B_P, B_P1V = B_P + 6, B_PV = B_P1V + 3, NB = B_PV + 3 };

// second-order expansion of a per-momentum sum in mu - mu0
template <class S> HD S tay(const S& dmu, const double* T) { return T[0] + dmu * (T[1] + dmu * (0.5 * T[2])); }

// r^T f(t, Y) from the bilinear form and the coefficients (exact at the
// nominal point, second order in mu - mu0 for a perturbed m_nu).
template <class S>
HD S phi(const Coef<S>& C, const double* B, double k) {
  S r = C.sg[0] * B[B_SIG];
  for (int i = 1; i < NSIG; ++i) r = r + C.sg[i] * B[B_SIG + i];
  S h1 = C.xh * tay(C.dmu, B + B_H1T), hw = C.xh * tay(C.dmu, B + B_HWT);
  S e = C.xe * B[B_EF];
  S p = C.xp * (tay(C.dmu, B + B_P1V) + tay(C.dmu, B + B_PV));
  for (int j = 0; j < 6; ++j) {
    h1 = h1 + C.ch[j] * B[B_H1 + j];
    hw = hw + C.ch[j] * B[B_HW + j];
    p = p + C.cp[j] * B[B_P + j];
  }
  for (int j = 0; j < 5; ++j) e = e + C.ce[j] * B[B_E + j];
  r = r + h1 + C.sg[SG_W1] * hw + e + C.sg[SG_A] * p + C.opac * B[B_OP] + B[B_FREE] + k * tay(C.dmu, B + B_V) +
      C.itau * B[B_IT];
  return r;
}

// ------------------------------------------------------------------ lead-row inverse tables
// The lead rows' table (DEB_LEAD_ROWS) inverted, built once on the host:
// by scalar sigma (for B) and by source element (for the transposed
// product).  Terms with kap = 0 are padding and dropped.  The derived-value
// terms (h', eta', alpha, P1 as sources) are few and listed separately.
constexpr int LINV_MAXE = 16, LINV_NSLOT = 40, LINV_NDER = 16;
enum { DK_HP1 = 0, DK_HPW, DK_E, DK_ALPHA, DK_P1 };
struct LeadInv {
  int nsig[NSIG];
  short sig_ent[NSIG][LINV_MAXE];   // r * NLT + t
  int nslot;
  int slot_base[LINV_NSLOT], slot_off[LINV_NSLOT], slot_n[LINV_NSLOT];
  short slot_ent[LINV_NSLOT][LINV_MAXE];
  int nder;
  short der_ent[LINV_NDER];         // r * NLT + t
  short der_kind[LINV_NDER];        // DK_*
  int ok;
};

inline void build_lead_inv(LeadInv& L) {
  std::memset(&L, 0, sizeof(L));
  L.ok = 1;
  for (int r = 0; r < NLEAD; ++r)
    for (int t = 0; t < NLT; ++t) {
      const LeadTerm& e = h_lead_rows[r][t];
      if (e.kap == 0.0) continue;
      const short code = (short)(r * NLT + t);
      if (e.base == IB_DV && e.off != DV_ONE) {
        int kind = -1;
        if (e.off == DV_HP && e.sig == SG_ONE) kind = DK_HP1;
        else if (e.off == DV_HP && e.sig == SG_W1) kind = DK_HPW;
        else if (e.off == DV_ETAP && e.sig == SG_ONE) kind = DK_E;
        else if (e.off == DV_ALPHA && e.sig == SG_K2) kind = DK_ALPHA;
        else if (e.off == DV_P1 && e.sig == SG_A) kind = DK_P1;
        if (kind < 0 || L.nder >= LINV_NDER) { L.ok = 0; continue; }
        L.der_ent[L.nder] = code;
        L.der_kind[L.nder] = (short)kind;
        ++L.nder;
        continue;
      }
      if (L.nsig[e.sig] >= LINV_MAXE) { L.ok = 0; continue; }
      L.sig_ent[e.sig][L.nsig[e.sig]++] = code;
      if (e.base == IB_DV) continue;   // the constant source of row 0
      int s = 0;
      while (s < L.nslot && !(L.slot_base[s] == e.base && L.slot_off[s] == e.off)) ++s;
      if (s == L.nslot) {
        if (L.nslot >= LINV_NSLOT) { L.ok = 0; continue; }
        L.slot_base[s] = e.base; L.slot_off[s] = e.off; L.slot_n[s] = 0; ++L.nslot;
      }
      if (L.slot_n[s] >= LINV_MAXE) { L.ok = 0; continue; }
      L.slot_ent[s][L.slot_n[s]++] = code;
    }
}

#ifdef __CUDACC__
__constant__ LeadInv c_linv;
#endif
inline const LeadInv& host_linv() {
  static LeadInv L;
  static bool done = false;
  if (!done) { build_lead_inv(L); done = true; }
  return L;
}
HD const LeadInv& linv() {
#ifdef __CUDA_ARCH__
  return c_linv;
#else
  return host_linv();
#endif
}

// ------------------------------------------------------------------ vectors
// element j of a vector at p[j * s]
struct VecRef {
  double* p;
  int s;
  HD double& operator[](int j) const { return p[(long)j * s]; }
};

// Adjoint workspace of one item: the forward slot, NAV adjoint vectors, the
// segment states and a scratch block (shared memory on the GPU).
enum { A_LAM = 0, A_RB, A_UB, A_YH, A_YE, A_RHO, A_TMP, A_YOUT, A_YO2, A_KB0, NAV = A_KB0 + 8 };
enum { SC_B = 0, SC_BW = SC_B + NB, SC_BR = SC_BW + NB, SC_CF = SC_BR + NB,   // Coef<double> at a stage point
       SC_CJ = SC_CF + 48, SC_RES = SC_CJ + 96, SC_RES2 = SC_RES + 32, SC_TH = SC_RES2 + 32, SC_SCAL = SC_TH + 16,
       SC_TO = SC_SCAL + 16, SC_FT = SC_TO + 64, SC_OC = SC_FT + 72, SC_LEN = SC_OC + 16 };
enum { SS_TB0 = 0, SS_DTB, SS_DBAR, SS_STS, SS_TBN, SS_CFB, SS_A0 };

// The adjoint vectors read most often in a step -- r (every pass of the
// transposed solve, the forms, J^T), Y_h and Y_e (each solve's Woodbury
// term), ubar and the stage point -- can live in shared memory (AWS::shv,
// NSHV vectors of n) when the launch has room; the others stay in global.
constexpr int NSHV = 5;
HD int shared_slot(int i) {
  return i == A_RB ? 0 : i == A_YH ? 1 : i == A_YE ? 2 : i == A_UB ? 3 : i == A_TMP ? 4 : -1;
}

template <int G>
struct AWS {
  WS<G> w;
  double* av;      // adjoint vectors, element stride WS<G>::S
  double* seg;     // segment states [seg_cap][n], element stride WS<G>::S
  int seg_cap;
  double* sc;      // scratch, SC_LEN doubles
  int n;
  double* shv = nullptr;   // NSHV shared vectors (contiguous), or null
  HD VecRef vec(int i) const {
    const int sl = shv ? shared_slot(i) : -1;
    if (sl >= 0) return VecRef{shv + (long)sl * n, 1};
    return VecRef{av + (long)i * n * WS<G>::S, WS<G>::S};
  }
  HD VecRef fv(int i) const { return VecRef{&w.v(i, 0), WS<G>::S}; }
  HD VecRef segv(int j) const { return VecRef{seg + (long)j * n * WS<G>::S, WS<G>::S}; }
};
static_assert(sizeof(Coef<double>) <= 48 * sizeof(double), "scratch slot for Coef<double>");
static_assert(sizeof(Coef<Jet<double>>) <= 96 * sizeof(double), "scratch slot for Coef<Jet<double>>");

// ------------------------------------------------------------------ B(r, Y)
// B accumulates (add = true) or is written.  with_row0: include row 0's
// a-only term (a' = aH a); pairs whose Y is a direction (a stage vector)
// leave it out.  mu0: expansion point of the per-momentum sums.
template <int G>
HD void bform(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w,
              VecRef x, VecRef Y, double mu0, bool with_row0, double* B, bool add) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp,
            lr = D.lr, lnu = D.lnu;
  const double k = m.k;
  // per-lane partial sums of the O(n) and O(nq) reductions
  double p_op = 0.0, p_free = 0.0, p_v0 = 0.0, p_v1 = 0.0, p_v2 = 0.0, p_it = 0.0, p_hn = 0.0, p_en = 0.0;
  double p_t0 = 0.0, p_t1 = 0.0, p_t2 = 0.0, p_s0 = 0.0, p_s1 = 0.0, p_s2 = 0.0, p_fn = 0.0;
  {
    const int nt = lg - 3, np = lgp - 3, nr = lr - 3;
    for (int e = gp.lane; e < nt + np + nr; e += G) {
      const bool ph = e < nt + np;
      const int l = 3 + (e < nt ? e : (ph ? e - nt : e - nt - np));
      const int j = (e < nt ? 7 : (ph ? igp : ir)) + l;
      const double xj = x[j];
      p_free += xj * (k * (T.lo[l] * Y[j - 1] - T.up[l] * Y[j + 1]));
      if (ph) p_op -= xj * Y[j];
    }
  }
  for (int i = gp.lane; i < nq; i += G) {
    const double q = LDG(c.q + i), wq = LDG(c.w + i), dlf = w.m(M_Q + Q_DLF * nq + i);
    const double xx = mu0 / q, v = rsqrt_(1.0 + xx * xx), v3 = v * v * v, iq2 = 1.0 / (q * q);
    auto X = [&](int l) { return x[iq0 + l * nq + i]; };
    auto YY = [&](int l) { return Y[iq0 + l * nq + i]; };
    double vt = -X(0) * YY(1) + X(1) * (YY(0) - 2.0 * YY(2)) * (1.0 / 3.0) + X(2) * (2.0 * YY(1) - 3.0 * YY(3)) * 0.2;
    for (int l = 3; l < lnu; ++l) vt += X(l) * (T.lo[l] * YY(l - 1) - T.up[l] * YY(l + 1));
    vt += X(lnu) * YY(lnu - 1);
    // v and 1/v and their first two derivatives in mu
    const double dv = -xx * v3 / q, ddv = (-v3 + 3.0 * xx * xx * v3 * v * v) * iq2;
    const double iv = 1.0 / v, div = xx * v / q, ddiv = v3 * iq2;
    p_v0 += vt * v; p_v1 += vt * dv; p_v2 += vt * ddv;
    p_it -= (lnu + 1.0) * X(lnu) * YY(lnu);
    p_hn += dlf * (X(0) * (1.0 / 6.0) - X(2) * (1.0 / 15.0));
    p_en -= 0.4 * dlf * X(2);
    const double wy = wq * YY(0);
    p_t0 += wy * iv; p_t1 += wy * div; p_t2 += wy * ddiv;
    p_s0 += wy * v; p_s1 += wy * dv; p_s2 += wy * ddv;
    p_fn += wq * YY(1);
  }
  gp.sum3(p_op, p_free, p_v0);
  gp.sum3(p_v1, p_v2, p_it);
  gp.sum3(p_hn, p_en, p_t0);
  gp.sum3(p_t1, p_t2, p_s0);
  gp.sum3(p_s1, p_s2, p_fn);
  // lead rows with a state source (or row 0's constant), by scalar sigma
  const LeadInv& L = linv();
  for (int i = gp.lane; i < NSIG; i += G) {
    double s = 0.0;
    for (int e = 0; e < L.nsig[i]; ++e) {
      const int code = L.sig_ent[i][e], r = code / NLT, t = code - r * NLT;
      if (r == 0 && !with_row0) continue;
      const LeadTerm& lt = lead_term(r, t);
      const double xr = x[lead_index(D, lead_tgt(r, 0), lead_tgt(r, 1))];
      const double src = lt.base == IB_DV ? 1.0 : Y[lead_index(D, lt.base, lt.off)];
      s += lt.kap * xr * src;
    }
    B[B_SIG + i] = add ? B[B_SIG + i] + s : s;
  }
  // weights of the derived values, alpha = (h' + 6 eta') / (2 k^2) folded in
  double xk[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int e = 0; e < L.nder; ++e) {
    const int code = L.der_ent[e], r = code / NLT, t = code - r * NLT;
    xk[L.der_kind[e]] += lead_term(r, t).kap * x[lead_index(D, lead_tgt(r, 0), lead_tgt(r, 1))];
  }
  const double xh1 = xk[DK_HP1] + 0.5 * xk[DK_ALPHA] + p_hn, xhw = xk[DK_HPW];
  const double xe = xk[DK_E] + 3.0 * xk[DK_ALPHA] + p_en, xp = xk[DK_P1];
  if (gp.lead()) {
    const double yh[6] = {Y[2], Y[3], Y[5], Y[7], Y[ir], Y[n - 2]};
    const double ye[5] = {Y[4], Y[6], Y[8], Y[ir + 1], Y[n - 1]};
    const double yp[6] = {Y[3], Y[5], Y[7], Y[ir], Y[n - 2], Y[n - 1]};
    const double t1v[3] = {p_t0, p_t1, p_t2}, tv[3] = {p_s0, p_s1, p_s2};
    double v[NB - B_OP];
    v[B_OP - B_OP] = p_op; v[B_FREE - B_OP] = p_free;
    v[B_V - B_OP] = p_v0; v[B_V + 1 - B_OP] = p_v1; v[B_V + 2 - B_OP] = p_v2; v[B_IT - B_OP] = p_it;
    for (int j = 0; j < 6; ++j) { v[B_H1 + j - B_OP] = xh1 * yh[j]; v[B_HW + j - B_OP] = xhw * yh[j]; v[B_P + j - B_OP] = xp * yp[j]; }
    for (int j = 0; j < 3; ++j) {
      v[B_H1T + j - B_OP] = xh1 * t1v[j]; v[B_HWT + j - B_OP] = xhw * t1v[j];
      v[B_P1V + j - B_OP] = xp * t1v[j]; v[B_PV + j - B_OP] = xp * tv[j];
    }
    for (int j = 0; j < 5; ++j) v[B_E + j - B_OP] = xe * ye[j];
    v[B_EF - B_OP] = xe * p_fn;
    for (int j = 0; j < NB - B_OP; ++j) B[B_OP + j] = add ? B[B_OP + j] + v[j] : v[j];
  }
  gp.sync();
}

// ------------------------------------------------------------------ J^T x
// z[j] += (J(t, Y)^T x)[j] for j >= 1 (the rows' dependence on state
// elements; the column of a is d phi / d a), with the coefficients C at
// (a, t).  S = Jet<double> adds the a-derivative of J^T x instead (the
// dependence of the W-matrix's J(y0) on a).  Three passes, each writing
// distinct elements: hierarchy couplings (gathered), lead-row sources
// (by the inverse table; needs lmax >= 5 so that no two sources alias),
// and the metric functionals.
template <class S, int G>
HD void apply_jt(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w,
                 const Coef<S>& C, const S& a, VecRef x, VecRef z) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp,
            lr = D.lr, lnu = D.lnu;
  const double k = m.k;
  // (1) photon T, photon P and massless nu chains: rows 3 .. lmax-1 couple
  // to their neighbours; damping on the photon rows
  {
    const int cT = lg + 1, cP = lgp + 1, cR = lr + 1;
    for (int e = gp.lane; e < cT + cP + cR; e += G) {
      const int which = e < cT ? 0 : (e < cT + cP ? 1 : 2);
      const int l = which == 0 ? e : (which == 1 ? e - cT : e - cT - cP);
      const int lmax = which == 0 ? lg : (which == 1 ? lgp : lr);
      const int j = (which == 0 ? 7 : (which == 1 ? igp : ir)) + l;
      S s = S(0.0);
      if (l + 1 >= 3 && l + 1 <= lmax - 1) s = s + (k * T.lo[l + 1]) * x[j + 1];
      if (l - 1 >= 3 && l - 1 <= lmax - 1) s = s - (k * T.up[l - 1]) * x[j - 1];
      if (which < 2 && l >= 3 && l <= lmax - 1) s = s - C.opac * x[j];
      z[j] += dpart(s);
    }
  }
  // massive neutrinos (every row explicit), element (l, q): a lane per
  // momentum bin walks its multipoles with X(l-1), X(l), X(l+1) in registers
  // (k v_q once per bin; lanes of one l read consecutive q)
  for (int q = gp.lane; q < nq; q += G) {
    const S aq = a * w.m(M_Q + Q_AMQ * nq + q);
    const S kv = k * jrsqrt(1.0 + aq * aq);
    auto X = [&](int ll) { return x[iq0 + ll * nq + q]; };
    double xm = 0.0, x0 = X(0), xp = lnu >= 1 ? X(1) : 0.0;
    for (int l = 0; l <= lnu; ++l) {
      const double xn = l + 2 <= lnu ? X(l + 2) : 0.0;
      S s = S(0.0);
      if (l >= 1) {   // row l-1, its coupling to l + ... = D(l-1)
        const int lp = l - 1;
        const double dc = lp == 0 ? -1.0 : (lp == 1 ? -2.0 / 3.0 : (lp == 2 ? -0.6 : -T.up[lp]));
        s = s + (dc * xm) * kv;
      }
      if (l + 1 <= lnu) {   // row l+1, its coupling to l - ...
        const int lp = l + 1;
        const double uc = lp == 1 ? 1.0 / 3.0 : (lp == 2 ? 0.4 : (lp == lnu ? 1.0 : T.lo[lp]));
        s = s + (uc * xp) * kv;
      }
      if (l == lnu) s = s - ((lnu + 1.0) * x0) * C.itau;
      z[iq0 + l * nq + q] += dpart(s);
      xm = x0;
      x0 = xp;
      xp = xn;
    }
  }
  gp.sync();
  // (2) lead rows with state sources
  const LeadInv& L = linv();
  for (int sl = gp.lane; sl < L.nslot; sl += G) {
    S s = S(0.0);
    for (int e = 0; e < L.slot_n[sl]; ++e) {
      const int code = L.slot_ent[sl][e], r = code / NLT, t = code - r * NLT;
      const LeadTerm& lt = lead_term(r, t);
      s = s + C.sg[lt.sig] * (lt.kap * x[lead_index(D, lead_tgt(r, 0), lead_tgt(r, 1))]);
    }
    z[lead_index(D, L.slot_base[sl], L.slot_off[sl])] += dpart(s);
  }
  gp.sync();
  // (3) metric functionals: their weights from the rows that read them
  double xk[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int e = 0; e < L.nder; ++e) {
    const int code = L.der_ent[e], r = code / NLT, t = code - r * NLT;
    xk[L.der_kind[e]] += lead_term(r, t).kap * x[lead_index(D, lead_tgt(r, 0), lead_tgt(r, 1))];
  }
  double hn = 0.0, en = 0.0;
  for (int i = gp.lane; i < nq; i += G) {
    const double dlf = w.m(M_Q + Q_DLF * nq + i);
    hn += dlf * (x[iq0 + i] * (1.0 / 6.0) - x[iq0 + 2 * nq + i] * (1.0 / 15.0));
    en -= 0.4 * dlf * x[iq0 + 2 * nq + i];
  }
  gp.sum2(hn, en);
  const S wh = (xk[DK_HP1] + 0.5 * xk[DK_ALPHA] + hn) + C.sg[SG_W1] * xk[DK_HPW];
  const S we = S(xk[DK_E] + 3.0 * xk[DK_ALPHA] + en);
  const S wp = C.sg[SG_A] * xk[DK_P1];
  if (gp.lead()) {
    z[2] += dpart(wh * C.ch[0]);
    z[3] += dpart(wh * C.ch[1] + wp * C.cp[0]);
    z[5] += dpart(wh * C.ch[2] + wp * C.cp[1]);
    z[7] += dpart(wh * C.ch[3] + wp * C.cp[2]);
    z[ir] += dpart(wh * C.ch[4] + wp * C.cp[3]);
    z[n - 2] += dpart(wh * C.ch[5] + wp * C.cp[4]);
    z[4] += dpart(we * C.ce[0]);
    z[6] += dpart(we * C.ce[1]);
    z[8] += dpart(we * C.ce[2]);
    z[ir + 1] += dpart(we * C.ce[3]);
    z[n - 1] += dpart(we * C.ce[4] + wp * C.cp[5]);
  }
  for (int i = gp.lane; i < nq; i += G) {
    const double wq = LDG(c.w + i);
    const S aq = a * w.m(M_Q + Q_AMQ * nq + i);
    const S v = jrsqrt(1.0 + aq * aq), iv = jrcp(v);
    z[iq0 + i] += dpart(wh * C.xh * wq * iv + wp * C.xp * wq * (iv + v));
    z[iq1 + i] += dpart(we * C.xe * wq);
  }
  gp.sync();
}

// ------------------------------------------------------------------ W^T solve
// z = M^-T r on indices >= 2 in place (M = I/(gamma h) - B factored by
// factor_M).  The transposed chain uses the same pivots: its sweep
// multipliers are LO of the next element and its back-substitution
// multipliers UP of the previous one.
template <int G>
HD void solve_Mt(const Grp<G>& gp, const Dims& D, const WS<G>& w, VecRef r) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  auto LO = [&](int i) { return w.v(V_LO, i); };
  auto UP = [&](int i) { return w.v(V_UP, i); };
  auto PI = [&](int i) { return w.v(V_PI, i); };
  if (gp.lead()) {
    const double id = w.m(M_SCAL + S_ID);
    r[2] = r[2] * id;
    const double z3 = r[3] * id;
    r[3] = z3;
    r[4] = (r[4] - z3) * w.m(M_SCAL + S_IDAH);
    // DE block stored as P^T L U of the forward matrix: M^T = U^T L^T P
    const double i00 = w.m(M_DE + 0), a01 = w.m(M_DE + 1), l10 = w.m(M_DE + 2), i11 = w.m(M_DE + 3);
    const double v0 = r[n - 2] * i00;
    const double v1 = (r[n - 1] - a01 * v0) * i11;
    double w0 = v0 - l10 * v1, w1 = v1;
    if (w.m(M_DE + 4) != 0.0) { const double t = w0; w0 = w1; w1 = t; }
    r[n - 2] = w0; r[n - 1] = w1;
  }
  for (int ch = gp.lane; ch < nq + 3; ch += G) {
    const bool tail = ch > nq;
    const int start = ch == 0 ? ir : (!tail ? iq0 + ch - 1 : (ch == nq + 1 ? 10 : igp + 3));
    const int stride = (ch == 0 || tail) ? 1 : nq;
    const int cnt = ch == 0 ? lr + 1 : (!tail ? lnu + 1 : (ch == nq + 1 ? lg - 2 : lgp - 2));
    // groups of eight elements load ahead of their dependent FMAs, so a
    // sweep pays the memory latency once per group, not once per element
    int i = start + (cnt - 1) * stride;
    double rn = r[i];
    int j = cnt - 2;
    for (; j >= 7; j -= 8) {
      double rv[8], lv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) { rv[q] = r[i - (q + 1) * stride]; lv[q] = LO(i - q * stride); }
#pragma unroll
      for (int q = 0; q < 8; ++q) { rn = rv[q] - lv[q] * rn; r[i - (q + 1) * stride] = rn; }
      i -= 8 * stride;
    }
    for (; j >= 0; --j) {
      const int ip = i;
      i -= stride;
      rn = r[i] - LO(ip) * rn;
      r[i] = rn;
    }
    if (!tail) {
      double zz = rn * PI(start);
      r[start] = zz;
      int jb = 1;
      for (; jb + 7 < cnt; jb += 8) {
        double sv[8], uv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int ii = i + (q + 1) * stride;
          sv[q] = r[ii] * PI(ii);
          uv[q] = UP(ii - stride);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) { zz = sv[q] - uv[q] * zz; r[i + (q + 1) * stride] = zz; }
        i += 8 * stride;
      }
      for (; jb < cnt; ++jb) {
        i += stride;
        zz = r[i] * PI(i) - UP(i - stride) * zz;
        r[i] = zz;
      }
    } else {
      r[start - 1] -= LO(start) * rn;
    }
  }
  gp.sync();
  {
    const int cidx[8] = {5, 6, 7, 8, 9, igp, igp + 1, igp + 2};
    double rc[8];
    for (int j = 0; j < 8; ++j) rc[j] = r[cidx[j]];
    gp.sync();
    for (int row = gp.lane; row < 8; row += G) {
      double zz = 0.0;
      for (int j = 0; j < 8; ++j) zz += w.m(M_CINV8 + row * 8 + j) * rc[j];
      r[cidx[row]] = zz;
    }
  }
  gp.sync();
  for (int t = gp.lane; t < 2; t += G) {
    const int start = t == 0 ? 10 : igp + 3;
    const int cnt = t == 0 ? lg - 2 : lgp - 2;
    double zz = r[start] * PI(start) - UP(start - 1) * r[start - 1];
    r[start] = zz;
    int j = 1;
    for (; j + 7 < cnt; j += 8) {
      double sv[8], uv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = start + j + q;
        sv[q] = r[i] * PI(i);
        uv[q] = UP(i - 1);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) { zz = sv[q] - uv[q] * zz; r[start + j + q] = zz; }
    }
    for (; j < cnt; ++j) {
      const int i = start + j;
      zz = r[i] * PI(i) - UP(i - 1) * zz;
      r[i] = zz;
    }
  }
  gp.sync();
}

// the rank-1 columns u_h, u_e of J (rows of h' and eta') as (index, u_h, u_e)
template <int G, class F>
HD void visit_u_lanes(const Grp<G>& gp, const Dims& D, const WS<G>& w, double wQ, F f) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, ir = D.ir;
  for (int e = gp.lane; e < 8 + 2 * nq; e += G) {
    if (e < 8) {
      switch (e) {
        case 0: f(3, -0.5, 0.0); break;
        case 1: f(5, -0.5, 0.0); break;
        case 2: f(7, -2.0 / 3.0, 0.0); break;
        case 3: f(9, 4.0 / 15.0, 1.6); break;
        case 4: f(ir, -2.0 / 3.0, 0.0); break;
        case 5: f(ir + 2, 4.0 / 15.0, 1.6); break;
        case 6: f(n - 2, -0.5 * (1.0 + wQ), 0.0); break;
        default: f(2, 0.0, 1.0); break;
      }
    } else {
      const int i = (e - 8) >> 1;
      const double dlf = w.m(M_Q + Q_DLF * nq + i);
      if (((e - 8) & 1) == 0) f(iq0 + i, dlf / 6.0, 0.0);
      else f(iq0 + 2 * nq + i, -dlf / 15.0, -0.4 * dlf);
    }
  }
}

// Y_h = M^-T g_h and Y_e = M^-T g_e (the functionals as vectors), once per step
template <int G>
HD void prep_wt(const Grp<G>& gp, const Dims& D, const WS<G>& w, VecRef yh, VecRef ye) {
  const int n = D.n, nq = D.nq;
  for (int j = gp.lane; j < n; j += G) { yh[j] = 0.0; ye[j] = 0.0; }
  gp.sync();
  // the eta' list's last entry is a zero pad that names the same element
  // as the one before it: it is left out, not written over the coefficient
  for (int t = gp.lane; t < nq + 6; t += G) {
    yh[gather_index(D, GL_H, t)] = w.m(gl_off(nq, GL_H) + t);
    if (t < nq + 5) ye[gather_index(D, GL_E, t)] = w.m(gl_off(nq, GL_E) + t);
  }
  gp.sync();
  solve_Mt<G>(gp, D, w, yh);
  solve_Mt<G>(gp, D, w, ye);
}

// b <- W^-T b for the W factored by the forward step (its factors in w),
// with Y_h, Y_e from prep_wt; wQ at (t0, y0).
template <int G>
HD void solve_Wt(const Grp<G>& gp, const Dims& D, const WS<G>& w, VecRef b, VecRef yh, VecRef ye, double wQ) {
  const int n = D.n, nq = D.nq;
  const double z1 = b[1] * w.m(M_SCAL + S_ID);
  gp.sync();
  for (int t = gp.lane; t < nq + 6; t += G) b[gather_index(D, GL_R1, t)] += w.m(gl_off(nq, GL_R1) + t) * z1;
  gp.sync();
  solve_Mt<G>(gp, D, w, b);
  double sh = 0.0, se = 0.0;
  visit_u_lanes<G>(gp, D, w, wQ, [&](int i, double uh, double ue) { sh += uh * b[i]; se += ue * b[i]; });
  gp.sum2(sh, se);
  const double th = w.m(M_CINV + 0) * sh + w.m(M_CINV + 2) * se;
  const double te = w.m(M_CINV + 1) * sh + w.m(M_CINV + 3) * se;
  for (int j = 2 + gp.lane; j < n; j += G) b[j] += yh[j] * th + ye[j] * te;
  gp.sync();
  double s0 = 0.0;
  for (int j = 1 + gp.lane; j < n; j += G) s0 += w.v(V_JC0, j) * (j == 1 ? z1 : b[j]);
  s0 = gp.sum(s0);
  if (gp.lead()) { b[1] = z1; b[0] = (b[0] + s0) * w.m(M_SCAL + S_W00I); }
  gp.sync();
}

// ------------------------------------------------------------------ output fields as a function of a
// convert_to_output_variables (perturbations.py:374-523) with the state
// entered as 13 scalars s = (eta, dc, tc, db, tb, dg, tg, dr, tr, dq, tq,
// drhonu, fnu), drhonu = sum_q w_q Y_0q / v_q, fnu = sum_q w_q Y_1q: linear
// in s for fixed a, written for any scalar type of a.
template <class S>
HD void outputs_s(const Cosmo& c, const ModeConst& m, const S& a, const double* s, S* r) {
  const double k = m.k, k2 = m.k2;
  const double eta = s[0], dc = s[1], tc = s[2], db = s[3], tb = s[4], dg = s[5], tg = s[6], dr = s[7], tr = s[8];
  const double dq = s[9], tq = s[10], drhonu = s[11], fnu = s[12];
  const S la = jlog(a), ia = jrcp(a), a2 = a * a, ia2 = ia * ia;
  const S rhonu = jexp(spl_eval_j(c.sp[SP_LRHONU_LOGA], la));
  const S pnu = jexp(spl_eval_j(c.sp[SP_LPNU_LOGA], la));
  const S irn = jrcp(rhonu);
  const S dnu = drhonu * irn, tnu = (k * fnu) * jrcp(rhonu + pnu);
  const S wQ = m.w0 + m.wa * (1.0 - a);
  const S rhoQ = jexp(m.pQ * la + 3.0 * (a - 1.0) * m.wa);
  const S rptQ = (1.0 + wQ) * rhoQ * (m.grhom * m.ODE * tq) * a2;
  const S grho = (m.grhom * m.Om) * ia + (m.grhog + m.grhor * (m.Neff + m.Nmnu * rhonu)) * ia2 +
                 (m.grhom * m.ODE) * rhoQ * a2 + m.grhom * m.Ok;
  const S g3 = grho * (1.0 / 3.0);
  const S iaH = jrsqrt(g3);
  const double cdb = m.grhom * (m.Oc * dc + m.Ob * db), ctb = m.grhom * (m.Oc * tc + m.Ob * tb);
  const S dgrho = cdb * ia + (m.grhog * dg + m.grhor * (m.Neff * dr + m.Nmnu * drhonu)) * ia2 +
                  (m.grhom * m.ODE * dq) * rhoQ * a2;
  const S dgtheta = ctb * ia + ((4.0 / 3.0) * (m.grhog * tg + m.Neff * m.grhor * tr)) * ia2 +
                    (m.Nmnu * m.grhor * k * fnu) * ia2 + rptQ;
  const S hp = (2.0 * k2 * eta + dgrho) * iaH;
  const S etap = dgtheta * (0.5 * m.ik2);
  const S alpha = (hp + 6.0 * etap) * (0.5 * m.ik2);
  const S den = (m.grhom * m.Om) * ia + (m.grhor * m.Nmnu) * rhonu * ia2;
  const S iden = jrcp(den);
  const S dm = (cdb * ia + (m.grhor * m.Nmnu * drhonu) * ia2) * iden;
  const S tm = (ctb * ia + (m.Nmnu * m.grhor * k * fnu) * ia2) * iden * (1.0 / 3.0) + alpha * k2;
  const double iOm = 1.0 / (m.grhom * m.Om);
  const S dbc = S(cdb * iOm);
  const S tbc = (ctb * iOm) * (1.0 / 3.0) * a2 + alpha * k2;
  r[0] = S(eta); r[1] = etap; r[2] = hp; r[3] = alpha; r[4] = dm; r[5] = tm * iaH; r[6] = dbc; r[7] = tbc * iaH;
  r[8] = S(dc); r[9] = tc * iaH; r[10] = S(db); r[11] = tb * iaH; r[12] = S(dg); r[13] = tg * iaH; r[14] = S(dr);
  r[15] = tr * iaH; r[16] = dnu; r[17] = tnu * iaH; r[18] = S(dq); r[19] = tq * iaH;
}

template <class S>
HD S gdot20(const double* g, const S* r) {
  S s = r[0] * g[0];
  for (int i = 1; i < 20; ++i) s = s + r[i] * g[i];
  return s;
}

// ------------------------------------------------------------------ per-item context
struct AdjItem {
  const double* blob0;   // nominal table blob
  const double* blobs;   // 2 npar perturbed blobs: set 2p = theta_p + eps_p, 2p + 1 = theta_p - eps_p
  int blob_len, npar;
  const double* eps;     // [npar]
  const double* tau0;    // [nout] nominal output times
  const double* taus;    // [2 npar][nout]
  const double* rec;     // recorded start time and step ends (deb_forward_record)
  int nrec;
  const double* ck;      // checkpoints [slot][n]
  int ck_stride;
  const double* gy;      // [nout][20] cotangent
  double k;
};

// table set e of an evaluation list: -1 = nominal, else perturbed set e
HD bool item_cosmo(const AdjItem& it, int set, Cosmo& c) {
  const double* b = set < 0 ? it.blob0 : it.blobs + (long)set * it.blob_len;
  return load_cosmo(b, it.blob_len, c);
}

// Evaluation slots of one derivative pass: 0 = d/da (nominal), 1 = d/dt
// (nominal), 2 + s = value on perturbed table set s.  Each writes res[slot];
// with a second form B2, res2[slot] gets the pass on B2 (d/da on every set
// for B2 when second = true, with slot 0 giving d2/da2).
template <int G>
HD void phi_pass(const Grp<G>& gp, const AdjItem& it, const Dims& D, const double* B, const double* B2,
                 double a, double t, double mu0, double* res, double* res2, Coef<double>* cf_out,
                 Coef<Jet<double>>* cj_out) {
  const int nev = 2 + 2 * it.npar;
  // the nominal coefficients asked for (cf_out / cj_out) on a lane of their
  // own, slot nev, beside the slots instead of after slot 0's jets
  const bool extra = cf_out || cj_out;
  for (int e = gp.lane; e < nev + (extra ? 1 : 0); e += G) {
    Cosmo c;
    ModeConst m;
    const int set = (e < 2 || e == nev) ? -1 : e - 2;
    if (!item_cosmo(it, set, c)) {
      if (e < nev) { res[e] = 0.0; if (res2) res2[e] = 0.0; }
      continue;
    }
    mode_const(c, it.k, m);
    if (e == nev) {
      if (cj_out) *cj_out = coef<Jet<double>>(c, m, D, Jet<double>(a, 1.0), Jet<double>(t), mu0);
      else *cf_out = coef<double>(c, m, D, a, t, mu0);
      continue;
    }
    if (e == 0) {
      if (B2) {
        // a-jet of a-jet: d phi(B) / da and d2 phi(B2) / da2
        typedef Jet<Jet<double>> J2;
        const J2 aj(Jet<double>(a, 1.0), Jet<double>(1.0, 0.0));
        const Coef<J2> C = coef<J2>(c, m, D, aj, J2(t), mu0);
        res[e] = phi<J2>(C, B, m.k).v.d;
        res2[e] = d12(phi<J2>(C, B2, m.k));
      } else {
        const Coef<Jet<double>> C = coef<Jet<double>>(c, m, D, Jet<double>(a, 1.0), Jet<double>(t), mu0);
        res[e] = phi<Jet<double>>(C, B, m.k).d;
      }
    } else if (e == 1) {
      const Coef<Jet<double>> C = coef<Jet<double>>(c, m, D, Jet<double>(a), Jet<double>(t, 1.0), mu0);
      res[e] = phi<Jet<double>>(C, B, m.k).d;
      if (B2) res2[e] = phi<Jet<double>>(C, B2, m.k).d;
    } else {
      if (B2) {
        const Coef<Jet<double>> C = coef<Jet<double>>(c, m, D, Jet<double>(a, 1.0), Jet<double>(t), mu0);
        res[e] = phi<Jet<double>>(C, B, m.k).v;
        res2[e] = phi<Jet<double>>(C, B2, m.k).d;
      } else {
        const Coef<double> C = coef<double>(c, m, D, a, t, mu0);
        res[e] = phi<double>(C, B, m.k);
      }
    }
  }
  gp.sync();
}

// ------------------------------------------------------------------ the stage vectors of one step backwards
// Stage s before its W^-T solve: rb = kbar_s and, for s >= 1, tmp = u_s as
// stage_prep formed it (u_s = y0 + sum_q a_sq k_q for s <= 5, u_6 = u_5 +
// k_5, u_7 = u_6 + k_6) -- one pass, every load of an element issued before
// its arithmetic (register arrays indexed by unrolled constants).
template <int G>
HD void adj_stage_pre(const Grp<G>& gp, const AWS<G>& A, const Rodas& R, int n, int s) {
  const VecRef rb = A.vec(A_RB), tmp = A.vec(A_TMP), kbs = A.vec(A_KB0 + s), y0 = A.fv(V_Y);
  const int sb = s <= 5 ? s : 5;
  double a[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) a[q] = q < sb ? R.a[sb][q] : 0.0;
  for (int j = gp.lane; j < n; j += G) {
    double k[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) k[q] = q < s ? A.fv(V_K0 + q)[j] : 0.0;
    const double kb = kbs[j], y = y0[j];
    rb[j] = kb;
    if (s >= 1) {
      double uu = y;
#pragma unroll
      for (int q = 0; q < 5; ++q)
        if (q < sb) uu += a[q] * k[q];
      if (s >= 6) uu = uu + k[5];
      if (s >= 7) uu = uu + k[6];
      tmp[j] = uu;
    }
  }
  gp.sync();
}

// Stage s after J^T r_s went into ubar (s >= 1) or dL/dy0 (s = 0), in one
// pass: kbar_q += C_sq / dt r_s (q < s) with the dt-derivative partial sums
// pc = r_s . sum_q C_sq k_q and pk = r_s . k_s; rho += k_s[0] r_s; and the
// stage point's cotangent: u_6 = u_5 + k_5 and u_7 = u_6 + k_6 pass ubar on
// (kbar_{s-1} += ubar), u_s = y0 + sum_q a_sq k_q (1 <= s <= 5) sends it to
// dL/dy0 and kbar_q and clears it.  pc, pk are this lane's partial sums.
template <int G>
HD void adj_stage_post(const Grp<G>& gp, const AWS<G>& A, const Rodas& R, int n, int s, double idt, double ks0,
                       double& pc_out, double& pk_out) {
  const VecRef rb = A.vec(A_RB), ub = A.vec(A_UB), lam = A.vec(A_LAM), rho = A.vec(A_RHO), ks = A.fv(V_K0 + s);
  double cs[7], ci[7], aa[5];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    cs[q] = q < s ? R.C[s][q] : 0.0;
    ci[q] = q < s ? R.C[s][q] * idt : 0.0;
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) aa[q] = (s <= 5 && q < s) ? R.a[s][q] : 0.0;
  double pc = 0.0, pk = 0.0;
  for (int j = gp.lane; j < n; j += G) {
    double k[7], kb[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      k[q] = q < s ? A.fv(V_K0 + q)[j] : 0.0;
      kb[q] = q < s ? A.vec(A_KB0 + q)[j] : 0.0;
    }
    const double rj = rb[j], kj = ks[j], rh = rho[j], uj = s >= 1 ? ub[j] : 0.0;
    double ck = 0.0;
#pragma unroll
    for (int q = 0; q < 7; ++q)
      if (q < s) {
        ck += cs[q] * k[q];
        kb[q] += ci[q] * rj;
      }
    pc += rj * ck;
    pk += rj * kj;
    rho[j] = rh + ks0 * rj;
    if (s >= 6) {
#pragma unroll
      for (int q = 5; q < 7; ++q)
        if (q == s - 1) kb[q] += uj;
    } else if (s >= 1) {
      lam[j] += uj;
#pragma unroll
      for (int q = 0; q < 5; ++q)
        if (q < s) kb[q] += aa[q] * uj;
      ub[j] = 0.0;
    }
#pragma unroll
    for (int q = 0; q < 7; ++q)
      if (q < s) A.vec(A_KB0 + q)[j] = kb[q];
  }
  pc_out = pc;
  pk_out = pk;
}

// ------------------------------------------------------------------ one step backwards
// On entry the forward step from (t0, y0 = V_Y) over dt has been recomputed
// into w (stages, factors, y1 in vector vu) with g0 its background at y0, and
// A_LAM holds dL/dy1.  On exit A_LAM holds dL/dy0, theta-gradient terms are
// added to sc[SC_TH + p], and tb0 / dtb receive dL/dt0 and dL/ddt.
template <int G>
HD void step_adjoint(const Grp<G>& gp, const AdjItem& it, const Cosmo& c, const ModeConst& m, const Dims& D,
                     const Tab& T, const Rodas& R, const AWS<G>& A, int vu, double t0, double dt,
                     const Bg<double>& g0, double& tb0, double& dtb) {
  const WS<G>& w = A.w;
  const int n = D.n, nq = D.nq, iq0 = D.iq0, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  double* sc = A.sc;
  const VecRef lam = A.vec(A_LAM), rb = A.vec(A_RB), ub = A.vec(A_UB), yh = A.vec(A_YH), ye = A.vec(A_YE),
               rho = A.vec(A_RHO), tmp = A.vec(A_TMP);
  auto KB = [&](int s) { return A.vec(A_KB0 + s); };
  auto K = [&](int s) { return A.fv(V_K0 + s); };
  const VecRef y0 = A.fv(V_Y);
  const double a0 = y0[0], mu0 = a0 * m.amnu;
  const double d = w.m(M_SCAL + S_D);
  const double idt = 1.0 / dt;
  prep_wt<G>(gp, D, w, yh, ye);
  for (int j = gp.lane; j < n; j += G) {
    const double l = lam[j];
    KB(7)[j] = l;
    ub[j] = l;
    lam[j] = 0.0;
    rho[j] = 0.0;
    for (int s = 0; s < 7; ++s) KB(s)[j] = 0.0;
  }
  for (int i = gp.lane; i < NB; i += G) sc[SC_BW + i] = 0.0;
  for (int i = gp.lane; i < 3 + nq; i += G) sc[SC_FT + i] = 0.0;
  gp.sync();
  double dbar = 0.0, tb = 0.0, db = 0.0;
  // truncation rows of d f / d tau and their coefficient (lmax + 1) / t0^2
  auto trunc_row = [&](int e, int& row, double& cf) {
    const double it2 = 1.0 / (t0 * t0);
    if (e == 0) { row = 7 + lg; cf = (lg + 1.0) * it2; }
    else if (e == 1) { row = igp + lgp; cf = (lgp + 1.0) * it2; }
    else if (e == 2) { row = ir + lr; cf = (lr + 1.0) * it2; }
    else { row = iq0 + lnu * nq + (e - 3); cf = (lnu + 1.0) * it2; }
  };
  for (int s = 7; s >= 0; --s) {
    // r = W^-T kbar_s; stage point u_s (as stage_prep forms it) and time
    adj_stage_pre<G>(gp, A, R, n, s);
    solve_Wt<G>(gp, D, w, rb, yh, ye, g0.wQ);
    const double ts = t0 + R.c[s] * dt;
    const VecRef u = s >= 1 ? tmp : y0;
    const double as = u[0];
    // derivatives of r^T f(t_s, u_s)
    bform<G>(gp, c, m, D, T, w, rb, u, as * m.amnu, true, sc + SC_B, false);
    phi_pass<G>(gp, it, D, sc + SC_B, nullptr, as, ts, as * m.amnu, sc + SC_RES, nullptr,
                reinterpret_cast<Coef<double>*>(sc + SC_CF), nullptr);
    if (gp.lead())
      for (int p = 0; p < it.npar; ++p)
        sc[SC_TH + p] += (sc[SC_RES + 2 + 2 * p] - sc[SC_RES + 3 + 2 * p]) / (2.0 * LDG(it.eps + p));
    const double tbs = sc[SC_RES + 1];
    tb += tbs;
    db += R.c[s] * tbs;
    // J(t_s, u_s)^T r into ubar (stages >= 1) or into dL/dy0 (stage 0)
    const VecRef tgt = s >= 1 ? ub : lam;
    const Coef<double> Cs = *reinterpret_cast<const Coef<double>*>(sc + SC_CF);
    apply_jt<double, G>(gp, c, m, D, T, w, Cs, as, rb, tgt);
    if (gp.lead()) tgt[0] += sc[SC_RES + 0];
    gp.sync();
    // sum_q C_sq / dt k_q: kbar_q += C_sq / dt r, and its dt-derivative; the
    // pair (r_s, k_s) of the J(y0) inside W: rho += k_s[0] r_s; the stage
    // point's cotangent
    const double ks0 = K(s)[0];
    double pc, pk;
    adj_stage_post<G>(gp, A, R, n, s, idt, ks0, pc, pk);
    gp.sum2(pc, pk);
    db -= pc * idt * idt;
    dbar -= pk;
    // dt d_s f_t(t0, y0)
    if (s <= 4) {
      double pf = 0.0;
      for (int e = gp.lane; e < 3 + nq; e += G) {
        int row; double cf;
        trunc_row(e, row, cf);
        sc[SC_FT + e] += dt * R.d[s] * rb[row];
        pf += rb[row] * cf * y0[row];
      }
      pf = gp.sum(pf);
      db += R.d[s] * pf;
    }
    // the J(y0) inside W: pairs (r_s, k_s)
    bform<G>(gp, c, m, D, T, w, rb, K(s), mu0, false, sc + SC_BW, true);
    gp.sync();
  }
  // W = I/(gamma dt) - J(t0, y0): dL/dW = -sum_s r_s k_s^T
  // pass on B_W = sum_s B(r_s, k_s) (value and first derivatives) and on
  // B(rho, y0) (derivatives of d phi / da)
  bform<G>(gp, c, m, D, T, w, rho, y0, mu0, true, sc + SC_BR, false);
  phi_pass<G>(gp, it, D, sc + SC_BW, sc + SC_BR, a0, t0, mu0, sc + SC_RES, sc + SC_RES2, nullptr,
              reinterpret_cast<Coef<Jet<double>>*>(sc + SC_CJ));
  if (gp.lead()) {
    for (int p = 0; p < it.npar; ++p) {
      const double i2e = 1.0 / (2.0 * LDG(it.eps + p));
      // d/dtheta of [d phi / da (rho, y0)] and of phi~(sum_s B(r_s, k_s))
      sc[SC_TH + p] += (sc[SC_RES2 + 2 + 2 * p] - sc[SC_RES2 + 3 + 2 * p]) * i2e +
                       (sc[SC_RES + 2 + 2 * p] - sc[SC_RES + 3 + 2 * p]) * i2e;
    }
  }
  // res[0] = d phi~(B_W) / da, res2[0] = d2 phi(rho, y0) / da2, res[1] = d phi~(B_W) / dt
  const double da0 = sc[SC_RES + 0] + sc[SC_RES2 + 0];
  tb += sc[SC_RES + 1];
  {
    const Coef<Jet<double>> Cj = *reinterpret_cast<const Coef<Jet<double>>*>(sc + SC_CJ);
    apply_jt<Jet<double>, G>(gp, c, m, D, T, w, Cj, Jet<double>(a0, 1.0), rho, lam);
  }
  if (gp.lead()) lam[0] += da0;
  db += dbar * (-d * idt);
  // d f / d tau terms: f_t[row] = (lmax + 1) y0[row] / t0^2
  double pt = 0.0;
  for (int e = gp.lane; e < 3 + nq; e += G) {
    int row; double cf;
    trunc_row(e, row, cf);
    const double fb = sc[SC_FT + e];
    lam[row] += cf * fb;
    pt -= 2.0 * cf / t0 * y0[row] * fb;
  }
  pt = gp.sum(pt);
  tb += pt;
  gp.sync();
  (void)vu; (void)lr;
  tb0 = tb;
  dtb = db;
}

// ------------------------------------------------------------------ one item: the whole solve backwards
// Boundary j of the recorded step sequence (0 .. nrec): tau_start, the
// recorded step ends (a negative entry names the output time the step was
// clipped to), and the last output time T1 for the final step -- the replay
// semantics of deb_replay at the nominal tables.
HD double adj_time(const AdjItem& it, double T1, int j) {
  if (j == 0) return LDG(it.rec);
  if (j >= it.nrec) return T1;
  const double v = LDG(it.rec + j);
  const double t = v < 0.0 ? LDG(it.tau0 + (int)(-v) - 1) : v;
  return t >= T1 ? T1 : t;
}

// Output fields' cotangent at output o inside step (tj, tj1] with weight
// cf: dL/dy_out is added to lam with cf and to yo2 with (1 - cf); returns
// dL/dcf.  Output-conversion theta terms go to sc[SC_TH].
template <int G>
HD double output_adjoint(const Grp<G>& gp, const AdjItem& it, const Cosmo& c0, const ModeConst& m0, const Dims& D,
                         const AWS<G>& A, int o, double cf, VecRef y0, VecRef y1) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, ir = D.ir;
  double* sc = A.sc;
  const double* g = it.gy + (long)o * NFIELD;
  const VecRef lam = A.vec(A_LAM), yo2 = A.vec(A_YO2), yo = A.vec(A_YOUT);
  for (int j = gp.lane; j < n; j += G) yo[j] = y0[j] + cf * (y1[j] - y0[j]);
  gp.sync();
  const double a = yo[0];
  double drho = 0.0, fnu = 0.0, ddrho = 0.0;
  for (int i = gp.lane; i < nq; i += G) {
    const double wq = LDG(c0.w + i), amq = m0.amnu / LDG(c0.q + i), aq = a * amq;
    const double v = rsqrt_(1.0 + aq * aq);
    drho += wq * yo[iq0 + i] / v;
    fnu += wq * yo[iq1 + i];
    ddrho += wq * yo[iq0 + i] * a * amq * amq * v;
  }
  gp.sum3(drho, fnu, ddrho);
  const double sv[13] = {yo[2], yo[3], yo[4], yo[5], yo[6], yo[7], yo[8], yo[ir], yo[ir + 1], yo[n - 2], yo[n - 1],
                         drho, fnu};
  // 0..12: coefficient of s_e (unit s, nominal tables); 13: d/da at fixed s;
  // 14 + b: value on perturbed set b (its own m_nu in drhonu)
  const int nev = 14 + 2 * it.npar;
  double* res = sc + SC_RES;
  for (int e = gp.lane; e < nev; e += G) {
    if (e < 14) {
      double r[20];
      if (e < 13) {
        double su[13];
        for (int q = 0; q < 13; ++q) su[q] = q == e ? 1.0 : 0.0;
        outputs_s<double>(c0, m0, a, su, r);
        res[e] = gdot20(g, r);
      } else {
        Jet<double> rj[20];
        outputs_s<Jet<double>>(c0, m0, Jet<double>(a, 1.0), sv, rj);
        res[e] = gdot20(g, rj).d;
      }
    } else {
      Cosmo cb;
      ModeConst mb;
      if (!item_cosmo(it, e - 14, cb)) { res[e] = 0.0; continue; }
      mode_const(cb, it.k, mb);
      double sb[13];
      for (int q = 0; q < 13; ++q) sb[q] = sv[q];
      double dr = 0.0;
      for (int i = 0; i < nq; ++i) {
        const double aq = a * mb.amnu / LDG(cb.q + i);
        dr += LDG(cb.w + i) * yo[iq0 + i] * sqrt(1.0 + aq * aq);
      }
      sb[11] = dr;
      double r[20];
      outputs_s<double>(cb, mb, a, sb, r);
      res[e] = gdot20(g, r);
    }
  }
  gp.sync();
  if (gp.lead())
    for (int p = 0; p < it.npar; ++p) sc[SC_TH + p] += (res[14 + 2 * p] - res[15 + 2 * p]) / (2.0 * LDG(it.eps + p));
  // dL/dy_out (sparse) into lam and yo2, and its product with y1 - y0
  const int fixed[11] = {2, 3, 4, 5, 6, 7, 8, ir, ir + 1, n - 2, n - 1};
  double dcf = 0.0;
  for (int e = gp.lane; e < 12 + 2 * nq; e += G) {
    int j;
    double v;
    if (e < 11) { j = fixed[e]; v = res[e]; }
    else if (e == 11) { j = 0; v = res[13] + res[11] * ddrho; }
    else {
      const int i = (e - 12) >> 1;
      const double wq = LDG(c0.w + i);
      if (((e - 12) & 1) == 0) {
        const double aq = a * m0.amnu / LDG(c0.q + i);
        j = iq0 + i; v = res[11] * wq * sqrt(1.0 + aq * aq);
      } else {
        j = iq1 + i; v = res[12] * wq;
      }
    }
    lam[j] += cf * v;
    yo2[j] += (1.0 - cf) * v;
    dcf += v * (y1[j] - y0[j]);
  }
  dcf = gp.sum(dcf);
  gp.sync();
  return dcf;
}

// Adjoint of one item.  gth[p] receives dL/dtheta_p for the npar
// parameters of the perturbed table sets.  Returns a deb mode status.
template <int G>
HD int adjoint_item(const Grp<G>& gp, const AdjItem& it, const Dims& D, const Tab& T, const Rodas& R, int nout,
                    const AWS<G>& A, double* gth) {
  const int n = D.n;
  const WS<G>& w = A.w;
  double* sc = A.sc;
  Cosmo c0;
  ModeConst m0;
  if (it.nrec < 1 || !load_cosmo(it.blob0, it.blob_len, c0) || c0.nq != D.nq) return ST_BAD_INPUT;
  mode_const(c0, it.k, m0);
  const int N = it.nrec, S = it.ck_stride;
  if (S < 1 || S > A.seg_cap) return ST_BAD_INPUT;
  double T1 = LDG(it.tau0);
  int omax = 0;
  for (int o = 1; o < nout; ++o) { const double t = LDG(it.tau0 + o); if (t > T1) { T1 = t; omax = o; } }
  const double ts0 = LDG(it.rec);
  Ctl ctl;
  ctl.dense = 0; ctl.nout = nout; ctl.replay = 1; ctl.record = 0; ctl.step_ts = 0; ctl.return_full = 0;
  // momentum-bin constants of the nominal tables into MISC
  initial_conditions<G>(gp, c0, m0, D, ts0, w, V_Y);
  const VecRef lam = A.vec(A_LAM), yo2 = A.vec(A_YO2);
  for (int j = gp.lane; j < n; j += G) lam[j] = 0.0;
  for (int i = gp.lane; i < 16; i += G) sc[SC_TH + i] = 0.0;
  for (int i = gp.lane; i < nout; i += G) sc[SC_TO + i] = 0.0;
  if (gp.lead()) { sc[SC_SCAL + SS_STS] = 0.0; sc[SC_SCAL + SS_TBN] = 0.0; }
  gp.sync();
  // a boundary's time adjoint into tau_start (scaled times), an output time or T1
  auto boundary = [&](int j, double tbar) {
    if (!gp.lead()) return;
    if (j == 0) { sc[SC_SCAL + SS_STS] += tbar; return; }
    if (j >= N) { sc[SC_TO + omax] += tbar; return; }
    const double v = LDG(it.rec + j);
    if (v < 0.0) { sc[SC_TO + (int)(-v) - 1] += tbar; return; }
    if (v >= T1) { sc[SC_TO + omax] += tbar; return; }
    sc[SC_SCAL + SS_STS] += tbar * v / ts0;
  };
  Run r;
  r.vy = V_Y; r.vu = V_U;
  const int nseg = (N + S - 1) / S;
  for (int sg = nseg - 1; sg >= 0; --sg) {
    const int c = sg * S, e = (c + S < N) ? c + S : N;
    // states of the segment from its checkpoint
    {
      const VecRef s0 = A.segv(0);
      for (int j = gp.lane; j < n; j += G) s0[j] = LDG(it.ck + (long)sg * n + j);
      gp.sync();
    }
    for (int j = c; j + 1 < e; ++j) {
      const VecRef sj = A.segv(j - c), sj1 = A.segv(j - c + 1), yv = A.fv(V_Y), uv = A.fv(V_U);
      for (int q = gp.lane; q < n; q += G) yv[q] = sj[q];
      gp.sync();
      r.t0 = adj_time(it, T1, j); r.t1 = adj_time(it, T1, j + 1);
      bool bad;
      step_attempt<G>(gp, c0, m0, D, T, R, ctl, w, r, bad);
      for (int q = gp.lane; q < n; q += G) sj1[q] = uv[q];
      gp.sync();
    }
    for (int j = e - 1; j >= c; --j) {
      const VecRef sj = A.segv(j - c), yv = A.fv(V_Y), uv = A.fv(V_U);
      for (int q = gp.lane; q < n; q += G) { yv[q] = sj[q]; yo2[q] = 0.0; }
      gp.sync();
      const double tj = adj_time(it, T1, j), tj1 = adj_time(it, T1, j + 1);
      r.t0 = tj; r.t1 = tj1;
      bool bad;
      Bg<double> g0;
      step_attempt<G>(gp, c0, m0, D, T, R, ctl, w, r, bad, &g0);
      const double dtj = tj1 - tj;
      double tb_left = 0.0, tb_right = sc[SC_SCAL + SS_TBN];
      // outputs inside (tj, tj1]
      for (int o = 0; o < nout; ++o) {
        const double to = LDG(it.tau0 + o);
        if (!(to > tj && to <= tj1)) continue;
        bool any = false;
        for (int f = 0; f < NFIELD; ++f) any = any || LDG(it.gy + (long)o * NFIELD + f) != 0.0;
        if (!any) continue;
        const double cf = (to - tj) / dtj;
        const double dcf = output_adjoint<G>(gp, it, c0, m0, D, A, o, cf, yv, uv);
        if (gp.lead()) sc[SC_TO + o] += dcf / dtj;
        tb_left += dcf * (to - tj1) / (dtj * dtj);
        tb_right -= dcf * (to - tj) / (dtj * dtj);
      }
      double tb0, dtb;
      step_adjoint<G>(gp, it, c0, m0, D, T, R, A, V_U, tj, dtj, g0, tb0, dtb);
      boundary(j + 1, tb_right + dtb);
      tb_left += tb0 - dtb;
      for (int q = gp.lane; q < n; q += G) lam[q] += yo2[q];
      gp.sync();
      if (gp.lead()) sc[SC_SCAL + SS_TBN] = tb_left;
      gp.sync();
    }
  }
  boundary(0, sc[SC_SCAL + SS_TBN]);
  gp.sync();
  // tau_start, the ICs and the output times of each perturbed set
  const VecRef ic = A.fv(V_U);
  for (int b = 0; b < 2 * it.npar; ++b) {
    Cosmo cb;
    ModeConst mb;
    if (!item_cosmo(it, b, cb) || cb.nq != D.nq) return ST_BAD_INPUT;
    mode_const(cb, it.k, mb);
    const double tsb = mode_start(cb, mb, ctl, it.taus + (long)b * nout);
    initial_conditions<G>(gp, cb, mb, D, tsb, w, V_U);
    double dot = 0.0;
    for (int j = gp.lane; j < n; j += G) dot += lam[j] * ic[j];
    dot = gp.sum(dot);
    if (gp.lead()) { sc[SC_RES + b] = dot; sc[SC_RES2 + b] = tsb; }
    gp.sync();
  }
  if (gp.lead()) {
    for (int p = 0; p < it.npar; ++p) {
      const double i2e = 1.0 / (2.0 * LDG(it.eps + p));
      double g = sc[SC_TH + p];
      g += (sc[SC_RES + 2 * p] - sc[SC_RES + 2 * p + 1]) * i2e;
      g += sc[SC_SCAL + SS_STS] * (sc[SC_RES2 + 2 * p] - sc[SC_RES2 + 2 * p + 1]) * i2e;
      for (int o = 0; o < nout; ++o)
        g += sc[SC_TO + o] * (LDG(it.taus + (long)(2 * p) * nout + o) - LDG(it.taus + (long)(2 * p + 1) * nout + o)) * i2e;
      gth[p] = g;
    }
  }
  gp.sync();
  return isfinite_(lam[0]) ? ST_OK : ST_NONFINITE;
}

}  // namespace deb
