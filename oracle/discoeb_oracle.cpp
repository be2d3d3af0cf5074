// discoeb_oracle.cpp -- CPU oracle for the DISCO-EB perturbation hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU path is
// compared against (and the timed CPU baseline); nothing in the shipped
// library links, loads or calls it.
//
// It restates, in plain FP64 C++, the reference algorithm of
// ``discoeb.perturbations.evolve_perturbations``:
//   * natural cubic spline evaluation   src/discoeb/spline_interpolation.py:130-153
//   * conformal Hubble rate             src/discoeb/background.py:100-122
//   * massive-nu momentum sums          src/discoeb/perturbations.py:22-50
//   * synchronous-gauge RHS             src/discoeb/perturbations.py:84-371
//   * output conversion (20 fields)     src/discoeb/perturbations.py:374-523
//   * adiabatic initial conditions      src/discoeb/perturbations.py:526-627
//   * start time (2x 7-step bisection)  src/discoeb/perturbations.py:630-681, util.py:365-396
//   * per-mode driver                   src/discoeb/perturbations.py:728-781, 926-997
//   * Rodas5 (transformed) step         src/discoeb/ode_integrators_stiff.py:622-834
//   * PID controller, error norm        perturbations.py:701-724,759-760 (diffrax PIDController)
//   * SaveAt(ts) linear interpolation   ode_integrators_stiff.py:698-700,833
// Like the reference it builds the DENSE Jacobian by forward-mode
// differentiation (dual numbers, one direction per column: jax.jacfwd) and
// factors W = I/(gamma h) - J by LU with partial pivoting (lu_factor).
//
// Tables arrive in the flat FP64 cosmology blob documented in
// include/discoeb_gb300.h (the same bytes the GPU receives).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- dual numbers
struct Dual {
  double v, d;
  Dual() : v(0), d(0) {}
  Dual(double x) : v(x), d(0) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
inline Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
inline Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
inline Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
inline Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
inline Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
inline Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
inline Dual operator/(double a, Dual b) { return Dual(a / b.v, -a * b.d / (b.v * b.v)); }
inline Dual exp(Dual a) { double e = std::exp(a.v); return Dual(e, e * a.d); }
inline Dual log(Dual a) { return Dual(std::log(a.v), a.d / a.v); }
inline Dual sqrt(Dual a) { double s = std::sqrt(a.v); return Dual(s, 0.5 * a.d / s); }
inline Dual pow(Dual a, double p) { double r = std::pow(a.v, p); return Dual(r, p * std::pow(a.v, p - 1.0) * a.d); }
inline double val(double x) { return x; }
inline double val(Dual x) { return x.v; }
using std::exp; using std::log; using std::sqrt; using std::pow;

// ---------------------------------------------------------------- table blob
enum { H_OMEGAM = 0, H_OMEGAB, H_OMEGADE, H_OMEGAK, H_GRHOM, H_GRHOG, H_GRHOR, H_NEFF, H_NMNU,
       H_AMNU, H_W0, H_WA, H_CS2DE, H_YHE, H_H0, H_TAUMIN, H_AS, H_NS, H_KP, H_NQ,
       H_NSPL0 = 20, H_BLOBLEN = 27, H_MAGIC = 28, HDR_LEN = 32 };
enum { SP_XE_LOGA = 0, SP_CS2A_LOGA, SP_LRHONU_LOGA, SP_LPNU_LOGA, SP_A_TAU, SP_TAU_A, SP_XE_TAU, NSPL };

struct Spline { const double *x, *y, *S; int n; };

struct Cosmo {
  double Om, Ob, ODE, Ok, grhom, grhog, grhor, Neff, Nmnu, amnu, w0, wa, cs2Q, YHe, H0, taumin, As, ns, kp;
  int nq;
  Spline sp[NSPL];
  const double *q, *w;
};

bool load_cosmo(const double* b, Cosmo& c) {
  if (b[H_MAGIC] != 20231103.0) return false;
  c.Om = b[H_OMEGAM]; c.Ob = b[H_OMEGAB]; c.ODE = b[H_OMEGADE]; c.Ok = b[H_OMEGAK];
  c.grhom = b[H_GRHOM]; c.grhog = b[H_GRHOG]; c.grhor = b[H_GRHOR]; c.Neff = b[H_NEFF];
  c.Nmnu = b[H_NMNU]; c.amnu = b[H_AMNU]; c.w0 = b[H_W0]; c.wa = b[H_WA]; c.cs2Q = b[H_CS2DE];
  c.YHe = b[H_YHE]; c.H0 = b[H_H0]; c.taumin = b[H_TAUMIN]; c.As = b[H_AS]; c.ns = b[H_NS]; c.kp = b[H_KP];
  c.nq = (int)b[H_NQ];
  const double* p = b + HDR_LEN;
  for (int s = 0; s < NSPL; ++s) {
    int n = (int)b[H_NSPL0 + s];
    c.sp[s].n = n; c.sp[s].x = p; c.sp[s].y = p + n; c.sp[s].S = p + 2 * n; p += 3 * n;
  }
  c.q = p; c.w = p + c.nq;
  return true;
}

// left searchsorted, clipped to [0, n-2]  (spline_interpolation.py:143)
inline int locate(const Spline& s, double x) {
  int lo = 0, hi = s.n;            // first index with s.x[i] >= x
  while (lo < hi) { int mid = (lo + hi) >> 1; if (s.x[mid] < x) lo = mid + 1; else hi = mid; }
  int i = lo - 1;
  if (i < 0) i = 0;
  if (i > s.n - 2) i = s.n - 2;
  return i;
}

template <class T> T spline_eval(const Spline& s, T x) {
  int i = locate(s, val(x));
  double h = s.x[i + 1] - s.x[i];
  T t = (x - s.x[i]) / h;
  T A = 1.0 - t, B = t;
  return A * s.y[i] + B * s.y[i + 1] + ((A * A * A - A) * s.S[i] + (B * B * B - B) * s.S[i + 1]) * (h * h) / 6.0;
}

template <class T> T rho_Q(const Cosmo& c, T a) {
  return pow(a, -3.0 * (1.0 + c.w0 + c.wa)) * exp(3.0 * (a - 1.0) * c.wa);
}

// conformal Hubble rate, background.py:100-122
template <class T> T aprimeoa(const Cosmo& c, T a) {
  T rhonu = exp(spline_eval(c.sp[SP_LRHONU_LOGA], log(a)));
  T grho = c.grhom * c.Om / a + (c.grhog + c.grhor * (c.Neff + c.Nmnu * rhonu)) / (a * a)
         + c.grhom * c.ODE * rho_Q(c, a) * (a * a) + c.grhom * c.Ok;
  return sqrt(grho / 3.0);
}

struct Dims {
  int lg, lgp, lr, lnu, nq, n;
  int idxgp, idxr, iq0;
};

Dims make_dims(int lg, int lgp, int lr, int lnu, int nq) {
  Dims d; d.lg = lg; d.lgp = lgp; d.lr = lr; d.lnu = lnu; d.nq = nq;
  d.n = 7 + (lg + 1) + (lgp + 1) + (lr + 1) + nq * (lnu + 1) + 2;
  d.idxgp = 8 + lg; d.idxr = 9 + lg + lgp; d.iq0 = 10 + lg + lgp + lr;
  return d;
}

// ---------------------------------------------------------------- RHS
// model_synchronous, perturbations.py:84-371.  T is double or Dual.
template <class T>
void rhs(const Cosmo& c, const Dims& D, double k, T tau, const T* y, T* f) {
  const int nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, iq2 = iq1 + nq, iq3 = iq2 + nq, iq4 = iq3 + nq;
  const int n = D.n;
  const double Oc = c.Om - c.Ob;
  const double k2 = k * k;
  T a = y[0];
  T loga = log(a);
  T eta = y[2], dc = y[3], tc = y[4], db = y[5], tb = y[6];
  T dg = y[7], tg = y[8], sg = y[9] / 2.0;
  const int ir = D.idxr;
  T dr = y[ir], tr = y[ir + 1], sr = y[ir + 2] / 2.0;
  T dq = y[n - 2], tq = y[n - 1];
  T cs2 = spline_eval(c.sp[SP_CS2A_LOGA], loga) / a;
  T xe = spline_eval(c.sp[SP_XE_LOGA], loga);
  T photbar = c.grhog / (c.grhom * c.Ob * a);
  T pb43 = 4.0 / 3.0 * photbar;
  T wQ = c.w0 + c.wa * (1.0 - a);
  T rhoQ = rho_Q(c, a);
  T a2 = a * a;
  T rptQ = (1.0 + wQ) * rhoQ * c.grhom * c.ODE * tq * a2;
  T aH = aprimeoa(c, a);
  T wQp = -c.wa * aH * a;
  T ca2 = wQ - wQp / 3.0 / ((1.0 + wQ) + 1e-6) / aH;
  const double akthom = 2.3038921003709498e-9 * (1.0 - c.YHe) * c.Ob * c.H0 * c.H0;
  T opac = xe * akthom / a2;
  f[0] = aH * a;
  // nu_perturb, perturbations.py:22-50
  T drhonu = 0.0, dpnu = 0.0, fnu = 0.0, shearnu = 0.0;
  std::vector<T> v(nq);
  for (int i = 0; i < nq; ++i) {
    T aq = a * c.amnu / c.q[i];
    v[i] = 1.0 / sqrt(1.0 + aq * aq);
  }
  for (int i = 0; i < nq; ++i) drhonu = drhonu + c.w[i] * y[iq0 + i] / v[i];
  for (int i = 0; i < nq; ++i) dpnu = dpnu + c.w[i] * y[iq0 + i] * v[i];
  dpnu = dpnu / 3.0;
  for (int i = 0; i < nq; ++i) fnu = fnu + c.w[i] * y[iq1 + i];
  for (int i = 0; i < nq; ++i) shearnu = shearnu + c.w[i] * y[iq2 + i] * v[i];
  shearnu = shearnu * 2.0 / 3.0;
  (void)shearnu;

  T dgrho = c.grhom * (Oc * dc + c.Ob * db) / a
          + (c.grhog * dg + c.grhor * (c.Neff * dr + c.Nmnu * drhonu)) / a2
          + c.grhom * c.ODE * dq * rhoQ * a2;
  T dgpres = (c.grhog * dg + c.grhor * c.Neff * dr) / a2 / 3.0
           + c.grhor * c.Nmnu * dpnu / a2
           + (c.cs2Q * c.grhom * c.ODE * dq * rhoQ * a2 + (c.cs2Q - ca2) * (3.0 * aH * rptQ / k2));
  T dgtheta = c.grhom * (Oc * tc + c.Ob * tb) / a
            + 4.0 / 3.0 * (c.grhog * tg + c.Neff * c.grhor * tr) / a2
            + c.Nmnu * c.grhor * k * fnu / a2 + rptQ;
  f[1] = -(dgrho + 3.0 * dgpres) * a;
  T hp = (2.0 * k2 * eta + dgrho) / aH;
  T etap = 0.5 * dgtheta / k2;
  T alpha = (hp + 6.0 * etap) / 2.0 / k2;
  f[2] = etap;
  f[3] = -tc - 0.5 * hp;
  f[4] = -aH * tc;
  f[5] = -tb - 0.5 * hp;
  f[6] = -aH * tb + k2 * cs2 * db + pb43 * opac * (tg - tb);
  const int ig = 7, igp = D.idxgp, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  T polter = y[ig + 2] + y[igp] + y[igp + 2];
  f[ig] = 4.0 / 3.0 * (-tg - 0.5 * hp);
  f[ig + 1] = k2 * (0.25 * dg - sg) - opac * (tg - tb);
  f[ig + 2] = 8.0 / 15.0 * (tg + k2 * alpha) - 3.0 / 5.0 * k * y[ig + 3] - opac * (y[ig + 2] - 0.1 * polter);
  for (int l = 3; l < lg; ++l)
    f[ig + l] = k / (2.0 * l + 1.0) * ((double)l * y[ig + l - 1] - (l + 1.0) * y[ig + l + 1]) - opac * y[ig + l];
  f[ig + lg] = k * y[ig + lg - 1] - (lg + 1.0) / tau * y[ig + lg] - opac * y[ig + lg];
  for (int l = 0; l < lgp; ++l)
    f[igp + l] = k / (2.0 * l + 1.0) * ((double)l * y[igp + l - 1] - (l + 1.0) * y[igp + l + 1]) - opac * y[igp + l];
  f[igp] = f[igp] + opac * polter / 2.0;
  f[igp + 2] = f[igp + 2] + opac * polter / 10.0;
  f[igp + lgp] = k * y[igp + lgp - 1] - (lgp + 1.0) / tau * y[igp + lgp] - opac * y[igp + lgp];
  f[ir] = 4.0 / 3.0 * (-tr - 0.5 * hp);
  f[ir + 1] = k2 * (0.25 * dr - sr);
  f[ir + 2] = 8.0 / 15.0 * (tr + k2 * alpha) - 0.6 * k * y[ir + 3];
  for (int l = 3; l < lr; ++l)
    f[ir + l] = k / (2.0 * l + 1.0) * ((double)l * y[ir + l - 1] - (l + 1.0) * y[ir + l + 1]);
  f[ir + lr] = k * y[ir + lr - 1] - (lr + 1.0) / tau * y[ir + lr];
  for (int i = 0; i < nq; ++i) {
    double q = c.q[i];
    double dlfdlq = -q / (1.0 + std::exp(-q));
    f[iq0 + i] = -k * v[i] * y[iq1 + i] + hp * dlfdlq / 6.0;
    f[iq1 + i] = k * v[i] * (y[iq0 + i] - 2.0 * y[iq2 + i]) / 3.0;
    f[iq2 + i] = k * v[i] * (2.0 * y[iq1 + i] - 3.0 * y[iq3 + i]) / 5.0 - (hp / 15.0 + 2.0 / 5.0 * etap) * dlfdlq;
    for (int l = 3; l < lnu; ++l)
      f[iq0 + l * nq + i] = k * v[i] / (2.0 * l + 1.0) *
          ((double)l * y[iq0 + (l - 1) * nq + i] - (l + 1.0) * y[iq0 + (l + 1) * nq + i]);
    f[iq0 + lnu * nq + i] = k * v[i] * y[iq0 + (lnu - 1) * nq + i] - (lnu + 1.0) / tau * y[iq0 + lnu * nq + i];
  }
  (void)iq4;
  f[n - 2] = -(1.0 + wQ) * (tq + 0.5 * hp) - 3.0 * (c.cs2Q - wQ) * aH * dq
           - 9.0 * (1.0 + wQ) * (c.cs2Q - ca2) * aH * aH / k2 * tq;
  f[n - 1] = -(1.0 - 3.0 * c.cs2Q) * aH * tq + c.cs2Q / (1.0 + wQ) * k2 * dq;
}

// ---------------------------------------------------------------- outputs
// convert_to_output_variables, perturbations.py:374-523
void outputs(const Cosmo& c, const Dims& D, double k, const double* y, double* o) {
  const int nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, iq2 = iq1 + nq, n = D.n;
  const double Oc = c.Om - c.Ob, k2 = k * k;
  double a = y[0], eta = y[2], dc = y[3], tc = y[4], db = y[5], tb = y[6], dg = y[7], tg = y[8];
  double dr = y[D.idxr], tr = y[D.idxr + 1];
  double la = std::log(a);
  double rhonu = std::exp(spline_eval(c.sp[SP_LRHONU_LOGA], la));
  double pnu = std::exp(spline_eval(c.sp[SP_LPNU_LOGA], la));
  double drhonu = 0, fnu = 0;
  for (int i = 0; i < nq; ++i) {
    double aq = a * c.amnu / c.q[i];
    double v = 1.0 / std::sqrt(1.0 + aq * aq);
    drhonu += c.w[i] * y[iq0 + i] / v;
    fnu += c.w[i] * y[iq1 + i];
  }
  (void)iq2;
  double dnu = drhonu / rhonu, tnu = k * fnu / (rhonu + pnu);
  double dq = y[n - 2], tq = y[n - 1];
  double wQ = c.w0 + c.wa * (1.0 - a);
  double rhoQ = rho_Q(c, a);
  double a2 = a * a;
  double rptQ = (1.0 + wQ) * rhoQ * c.grhom * c.ODE * tq * a2;
  double grho = c.grhom * c.Om / a + (c.grhog + c.grhor * (c.Neff + c.Nmnu * rhonu)) / a2
              + c.grhom * c.ODE * rhoQ * a2 + c.grhom * c.Ok;
  double aH = std::sqrt(grho / 3.0);
  double dgrho = c.grhom * (Oc * dc + c.Ob * db) / a
               + (c.grhog * dg + c.grhor * (c.Neff * dr + c.Nmnu * drhonu)) / a2
               + c.grhom * c.ODE * dq * rhoQ * a2;
  double dgtheta = c.grhom * (Oc * tc + c.Ob * tb) / a + 4.0 / 3.0 * (c.grhog * tg + c.Neff * c.grhor * tr) / a2
                 + c.Nmnu * c.grhor * k * fnu / a2 + rptQ;
  double hp = (2.0 * k2 * eta + dgrho) / aH;
  double etap = 0.5 * dgtheta / k2;
  double alpha = (hp + 6.0 * etap) / 2.0 / k2;
  double dm = (c.grhom * (Oc * dc + c.Ob * db) / a + (c.grhor * c.Nmnu * drhonu) / a2)
            / (c.grhom * c.Om / a + (c.grhor * c.Nmnu * rhonu) / a2);
  double tm = (c.grhom * (Oc * tc + c.Ob * tb) / a + c.Nmnu * c.grhor * k * fnu / a2)
            / (3.0 * (c.grhom * c.Om / a + c.grhor * c.Nmnu * rhonu / a2));
  double dbc = (c.grhom * (Oc * dc + c.Ob * db) / a) / (c.grhom * c.Om / a);
  double tbc = (c.grhom * (Oc * tc + c.Ob * tb) / a) / (3.0 * (c.grhom * c.Om / a) / a2);
  tm += alpha * k2;
  tbc += alpha * k2;
  double r[20] = {eta, etap, hp, alpha, dm, tm / aH, dbc, tbc / aH, dc, tc / aH, db, tb / aH,
                  dg, tg / aH, dr, tr / aH, dnu, tnu / aH, dq, tq / aH};
  std::memcpy(o, r, sizeof r);
}

// ---------------------------------------------------------------- ICs
// adiabatic_ics_one_mode, perturbations.py:526-627
void initial_conditions(const Cosmo& c, const Dims& D, double k, double tau, double* y) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, iq2 = iq1 + nq;
  std::fill(y, y + n, 0.0);
  double a = spline_eval(c.sp[SP_A_TAU], tau);
  double rn = std::exp(spline_eval(c.sp[SP_LRHONU_LOGA], std::log(a)));
  double rhom = c.grhom * c.Om / (a * a * a);
  double rhor = (c.grhog + c.grhor * (c.Neff + c.Nmnu * rn)) / (a * a * a * a);
  double rhonu = c.grhor * (c.Neff + c.Nmnu * rn) / (a * a * a * a);
  double fracb = c.Ob / c.Om, fracnu = rhonu / rhor;
  double om = a * rhom / std::sqrt(rhor);
  const double ci = -1.0, s2 = 1.0;
  double kt = k * tau;
  double dg = -(kt * kt) / 3.0 * (1.0 - om * tau / 5.0) * ci * s2;
  double tg = -(kt * kt * kt) / tau / 36.0 * (1.0 - 3.0 * (1.0 + 5.0 * fracb - fracnu) / 20.0 / (1.0 - fracnu) * om * tau) * ci * s2;
  double db = 0.75 * dg, tb = tg, dc = 0.75 * dg;
  double dr = dg;
  double tr = -(kt * kt * kt * kt) / tau / 36.0 / (4.0 * fracnu + 15.0) *
              (4.0 * fracnu + 11.0 + 12.0 - 3.0 * (8.0 * fracnu * fracnu + 50.0 * fracnu + 275.0) / 20.0 / (2.0 * fracnu + 15.0) * tau * om) * ci;
  double sr = (kt * kt) / (45.0 + 12.0 * fracnu) * (3.0 * s2 - 1.0) * (1.0 + (4.0 * fracnu - 5.0) / 4.0 / (2.0 * fracnu + 15.0) * tau * om) * ci;
  double wQ = c.w0 + c.wa * (1.0 - a);
  double dq = (kt * kt) / 4.0 * (1.0 + wQ) * (4.0 - 3.0 * c.cs2Q) / (4.0 - 6.0 * wQ + 3.0 * c.cs2Q) * ci * s2;
  double tq = (kt * kt * kt * kt) / tau / 4.0 * c.cs2Q / (4.0 - 6.0 * wQ + 3.0 * c.cs2Q) * ci * s2;
  double eta = ci * (1.0 - (kt * kt) / 12.0 / (15.0 + 4.0 * fracnu) *
               (5.0 + 4.0 * s2 * fracnu - (16.0 * fracnu * fracnu + 280.0 * fracnu + 325.0) / 10.0 / (2.0 * fracnu + 15.0) * tau * om));
  y[0] = a; y[1] = 0.0; y[2] = eta; y[3] = dc; y[4] = 0.0; y[5] = db; y[6] = tb; y[7] = dg; y[8] = tg;
  y[D.idxr] = dr; y[D.idxr + 1] = tr; y[D.idxr + 2] = sr * 2.0;
  for (int i = 0; i < nq; ++i) {
    double q = c.q[i];
    double aq = a * c.amnu / q;
    double v = 1.0 / std::sqrt(1.0 + aq * aq);
    double dlfdlq = -q / (1.0 + std::exp(-q));
    y[iq0 + i] = -0.25 * dlfdlq * dr;
    y[iq1 + i] = -dlfdlq * tr / v / k / 3.0;
    y[iq2 + i] = -0.5 * dlfdlq * sr;
  }
  y[n - 2] = dq; y[n - 1] = tq;
}

// ---------------------------------------------------------------- start time
// determine_starting_time, perturbations.py:630-681 (root_find_bisect util.py:365-396)
double start_time(const Cosmo& c, double k) {
  const double small_k = 0.0004, large_k = 0.07;
  double tau0 = c.taumin;
  double tau1 = spline_eval(c.sp[SP_TAU_A], 0.1);
  double tau_k = 1.0 / k;
  auto cond_small = [&](double lt) {
    double tau = std::exp(lt);
    double akthom = 2.3048e-9 * (1.0 - c.YHe) * c.Ob * c.H0 * c.H0;
    double xe = spline_eval(c.sp[SP_XE_TAU], tau);
    double a = spline_eval(c.sp[SP_A_TAU], tau);
    double opac = xe * akthom / (a * a);
    double aH = aprimeoa(c, a);
    return (1.0 / opac) / (1.0 / aH) / small_k - 1.0;
  };
  auto cond_large = [&](double lt) {
    double tau = std::exp(lt);
    double a = spline_eval(c.sp[SP_A_TAU], tau);
    double aH = aprimeoa(c, a);
    return (1.0 / aH) / tau_k / large_k - 1.0;
  };
  auto bisect = [&](auto&& fn) {
    double xl = std::log(tau0), xr = std::log(tau1);
    for (int it = 0; it < 7; ++it) {
      double xm = 0.5 * (xl + xr);
      if (fn(xm) * fn(xl) > 0.0) xl = xm; else xr = xm;
    }
    return 0.5 * (xl + xr);
  };
  double lt_large = bisect(cond_large);
  double lt_small = bisect(cond_small);
  return std::exp(std::min(lt_small, lt_large));
}

// ---------------------------------------------------------------- Rodas5 constants
// Published transformed Rodas5 tableau (Hairer & Wanner; as listed in
// ode_integrators_stiff.py:622-687).  The tableau has to be identical for the
// step sequence to be the reference's.
const double R_gamma = 0.19;
const double R_a[8][8] = {
  {0}, {2.0},
  {3.040894194418781, 1.041747909077569},
  {2.576417536461461, 1.622083060776640, -0.9089668560264532},
  {2.760842080225597, 1.446624659844071, -0.3036980084553738, 0.2877498600325443},
  {-14.09640773051259, 6.925207756232704, -41.47510893210728, 2.343771018586405, 24.13215229196062},
};
const double R_C[8][8] = {
  {0},
  {-10.31323885133993},
  {-21.04823117650003, -7.234992135176716},
  {32.22751541853323, -4.943732386540191, 19.44922031041879},
  {-20.69865579590063, -8.816374604402768, 1.260436877740897, -0.7495647613787146},
  {-46.22004352711257, -17.49534862857472, -289.6389582892057, 93.60855400400906, 318.3822534212147},
  {34.20013733472935, -14.15535402717690, 57.82335640988400, 25.83362985412365, 1.408950972071624, -6.551835421242162},
  {42.57076742291101, -13.80770672017997, 93.98938432427124, 18.77919633714503, -31.58359187223370, -6.685968952921985, -5.810979938412932},
};
const double R_c[8] = {0.0, 0.38, 0.3878509998321533, 0.4839718937873840, 0.4570477008819580, 1.0, 1.0, 1.0};
const double R_d[8] = {0.19, -0.1823079225333714636, -0.319231832186874912, 0.3449828624725343, -0.377417564392089818, 0, 0, 0};

struct Cfg {
  double rtol, atol, pcoeff, icoeff, dcoeff, fmax, fmin, error_order, safety;
  int max_steps, hist_on_reject, step_ts;
};

enum { ST_OK = 0, ST_MAX_STEPS = 1, ST_DT_UNDERFLOW = 2, ST_NONFINITE = 3, ST_BAD_INPUT = 4 };

// dense Jacobian via dual numbers: column j = directional derivative e_j
void jacobian(const Cosmo& c, const Dims& D, double k, double tau, const double* y, double* J,
              std::vector<Dual>& yd, std::vector<Dual>& fd) {
  const int n = D.n;
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) yd[i] = Dual(y[i], i == j ? 1.0 : 0.0);
    rhs<Dual>(c, D, k, Dual(tau), yd.data(), fd.data());
    for (int i = 0; i < n; ++i) J[(size_t)i * n + j] = fd[i].d;
  }
}

void dfdt(const Cosmo& c, const Dims& D, double k, double tau, const double* y, double* dT,
          std::vector<Dual>& yd, std::vector<Dual>& fd) {
  const int n = D.n;
  for (int i = 0; i < n; ++i) yd[i] = Dual(y[i]);
  rhs<Dual>(c, D, k, Dual(tau, 1.0), yd.data(), fd.data());
  for (int i = 0; i < n; ++i) dT[i] = fd[i].d;
}

// LU with partial pivoting (first maximal |pivot|, like LAPACK getrf); in place
void lu_factor(double* A, int n, int* piv) {
  for (int kk = 0; kk < n; ++kk) {
    int p = kk; double m = std::fabs(A[(size_t)kk * n + kk]);
    for (int i = kk + 1; i < n; ++i) { double v = std::fabs(A[(size_t)i * n + kk]); if (v > m) { m = v; p = i; } }
    piv[kk] = p;
    if (p != kk) for (int j = 0; j < n; ++j) std::swap(A[(size_t)kk * n + j], A[(size_t)p * n + j]);
    double d = A[(size_t)kk * n + kk];
    for (int i = kk + 1; i < n; ++i) {
      double l = A[(size_t)i * n + kk] / d;
      A[(size_t)i * n + kk] = l;
      if (l != 0.0) for (int j = kk + 1; j < n; ++j) A[(size_t)i * n + j] -= l * A[(size_t)kk * n + j];
    }
  }
}

void lu_solve(const double* A, int n, const int* piv, double* b) {
  for (int kk = 0; kk < n; ++kk) if (piv[kk] != kk) std::swap(b[kk], b[piv[kk]]);
  for (int i = 1; i < n; ++i) { double s = b[i]; for (int j = 0; j < i; ++j) s -= A[(size_t)i * n + j] * b[j]; b[i] = s; }
  for (int i = n - 1; i >= 0; --i) { double s = b[i]; for (int j = i + 1; j < n; ++j) s -= A[(size_t)i * n + j] * b[j]; b[i] = s / A[(size_t)i * n + i]; }
}

struct ModeResult { int status, accepted, rejected; };

ModeResult solve_mode(const Cosmo& c, const Dims& D, double k, const double* tau_out, int nout,
                      const Cfg& cfg, int return_full, double* yout) {
  const int n = D.n;
  ModeResult R{ST_OK, 0, 0};
  double tau_max = tau_out[0], tau_min_out = tau_out[0];
  for (int i = 1; i < nout; ++i) { tau_max = std::max(tau_max, tau_out[i]); tau_min_out = std::min(tau_min_out, tau_out[i]); }
  double t0 = 0.99 * std::min(tau_min_out, start_time(c, k));
  std::vector<double> y(n), y1(n), u(n), du(n), dT(n), J((size_t)n * n), K((size_t)8 * n), sc(n);
  std::vector<int> piv(n);
  std::vector<Dual> yd(n), fd(n);
  initial_conditions(c, D, k, t0, y.data());
  const int osz = return_full ? n : 20;
  // sort outputs by time, keep original index
  std::vector<int> order(nout);
  for (int i = 0; i < nout; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return tau_out[a] < tau_out[b]; });
  int next_out = 0;
  const double T1 = tau_max;
  double t1 = std::min(t0 + std::min(t0 / 4.0, 0.5 * (T1 - t0)), T1);
  // optional diffrax PIDController(step_ts=tau_out): never step across an output time
  auto clip_ts = [&](double tstart, double tend) {
    if (!cfg.step_ts) return tend;
    for (int i = 0; i < nout; ++i) if (tau_out[i] > tstart && tau_out[i] < tend) tend = tau_out[i];
    return tend;
  };
  t1 = clip_ts(t0, t1);
  double prev_inv = 1.0, prev_prev_inv = 1.0;
  const double beta1 = (cfg.icoeff + cfg.pcoeff + cfg.dcoeff) / cfg.error_order;
  const double beta2 = -(cfg.pcoeff + 2.0 * cfg.dcoeff) / cfg.error_order;
  const double beta3 = cfg.dcoeff / cfg.error_order;
  static const int err_idx[6] = {0, 2, 3, 5, 6, 7};
  const double err_w[6] = {1.0, k * k, 1.0, 1.0, 1.0 / (k * k), 1.0};
  int steps = 0;
  while (t0 < T1) {
    if (steps >= cfg.max_steps) { R.status = ST_MAX_STEPS; break; }
    const double dt = t1 - t0;
    // ---- Rodas5 transformed step (ode_integrators_stiff.py:718-834)
    jacobian(c, D, k, t0, y.data(), J.data(), yd, fd);
    const double dtg = dt * R_gamma;
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) J[(size_t)i * n + j] = (i == j ? 1.0 / dtg : 0.0) - J[(size_t)i * n + j];
    lu_factor(J.data(), n, piv.data());
    dfdt(c, D, k, t0, y.data(), dT.data(), yd, fd);
    for (int s = 0; s < 8; ++s) {
      double* ks = &K[(size_t)s * n];
      if (s == 0) {
        for (int i = 0; i < n; ++i) u[i] = y[i];
      } else if (s <= 5) {
        for (int i = 0; i < n; ++i) { double acc = y[i]; for (int j = 0; j < s; ++j) acc += R_a[s][j] * K[(size_t)j * n + i]; u[i] = acc; }
      } else {
        for (int i = 0; i < n; ++i) u[i] += K[(size_t)(s - 1) * n + i];
      }
      rhs<double>(c, D, k, t0 + R_c[s] * dt, u.data(), du.data());
      for (int i = 0; i < n; ++i) {
        double r = du[i];
        if (s <= 4) r += dt * R_d[s] * dT[i];
        double acc = 0.0;
        for (int j = 0; j < s; ++j) acc += (R_C[s][j] / dt) * K[(size_t)j * n + i];
        ks[i] = r + acc;
      }
      lu_solve(J.data(), n, piv.data(), ks);
    }
    const double* k8 = &K[(size_t)7 * n];
    bool nan = false;
    for (int i = 0; i < n; ++i) { y1[i] = u[i] + k8[i]; if (!std::isfinite(y1[i])) nan = true; }
    // ---- PID controller (diffrax PIDController.adapt_step_size)
    double ss = 0.0;
    for (int m = 0; m < 6; ++m) {
      int i = err_idx[m];
      double yc = nan ? y[i] : y1[i];
      double s = k8[i] / (cfg.atol + std::max(std::fabs(y[i]), std::fabs(yc)) * cfg.rtol);
      s *= err_w[m];
      ss += s * s;
    }
    double err = std::sqrt(ss / 6.0);
    if (!std::isfinite(err)) { R.status = ST_NONFINITE; break; }
    bool keep = err < 1.0;
    double inv = 1.0 / err;
    double f1 = beta1 == 0.0 ? 1.0 : std::pow(inv, beta1);
    double f2 = beta2 == 0.0 ? 1.0 : std::pow(prev_inv, beta2);
    double f3 = beta3 == 0.0 ? 1.0 : std::pow(prev_prev_inv, beta3);
    double factor = cfg.safety * f1 * f2 * f3;
    double fmin = keep ? 1.0 : cfg.fmin;
    factor = std::min(std::max(factor, fmin), cfg.fmax);
    double dtn = dt * factor;
    if (inv == 0.0 || std::isinf(inv)) inv = 1.0;
    ++steps;
    if (keep) {
      ++R.accepted;
      // SaveAt(ts): LocalLinearInterpolation between (t0, y) and (t1, y1)
      while (next_out < nout && tau_out[order[next_out]] <= t1) {
        double tt = tau_out[order[next_out]];
        double cf = (tt - t0) / (t1 - t0);
        for (int i = 0; i < n; ++i) sc[i] = y[i] + cf * (y1[i] - y[i]);
        double* dst = yout + (size_t)order[next_out] * osz;
        if (return_full) std::memcpy(dst, sc.data(), sizeof(double) * n);
        else outputs(c, D, k, sc.data(), dst);
        ++next_out;
      }
      std::swap(y, y1);
      t0 = t1;
      prev_prev_inv = prev_inv;
      prev_inv = inv;
    } else {
      ++R.rejected;
      if (cfg.hist_on_reject) { prev_prev_inv = prev_inv; prev_inv = inv; }
    }
    double tn = clip_ts(t0, t0 + dtn);
    if (tn > T1 - 1e-10) tn = T1;
    if (!(tn > t0)) { if (t0 < T1) { R.status = ST_DT_UNDERFLOW; break; } }
    t1 = tn;
  }
  return R;
}

// evolve_modes_batched (perturbations.py:835-922) with Rodas5Batched
// (ode_integrators_stiff.py:846-1010): B modes start together at the smallest
// of their start times (perturbations.py:786-803), take one step sequence,
// and the PID controller sees the RMS over the six filtered entries of all B
// modes (rms_norm_filtered_batched, perturbations.py:690-694).  Each mode's
// Rodas5 step is the per-mode step above.
ModeResult solve_group(const Cosmo& c, const Dims& D, const double* ks, int B, const double* tau_out, int nout,
                       const Cfg& cfg, double* yout /* [B, nout, 20] */) {
  const int n = D.n;
  ModeResult R{ST_OK, 0, 0};
  double tau_max = tau_out[0], tau_min_out = tau_out[0];
  for (int i = 1; i < nout; ++i) { tau_max = std::max(tau_max, tau_out[i]); tau_min_out = std::min(tau_min_out, tau_out[i]); }
  double t0 = 1e300;
  for (int b = 0; b < B; ++b) t0 = std::min(t0, 0.99 * std::min(tau_min_out, start_time(c, ks[b])));
  std::vector<std::vector<double>> y(B, std::vector<double>(n)), y1(B, std::vector<double>(n)), K(B, std::vector<double>((size_t)8 * n));
  std::vector<double> u(n), du(n), dT(n), J((size_t)n * n), sc(n);
  std::vector<int> piv(n);
  std::vector<Dual> yd(n), fd(n);
  for (int b = 0; b < B; ++b) initial_conditions(c, D, ks[b], t0, y[b].data());
  std::vector<int> order(nout);
  for (int i = 0; i < nout; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return tau_out[a] < tau_out[b]; });
  int next_out = 0;
  const double T1 = tau_max;
  double t1 = std::min(t0 + std::min(t0 / 4.0, 0.5 * (T1 - t0)), T1);
  double prev_inv = 1.0, prev_prev_inv = 1.0;
  const double beta1 = (cfg.icoeff + cfg.pcoeff + cfg.dcoeff) / cfg.error_order;
  const double beta2 = -(cfg.pcoeff + 2.0 * cfg.dcoeff) / cfg.error_order;
  const double beta3 = cfg.dcoeff / cfg.error_order;
  static const int err_idx[6] = {0, 2, 3, 5, 6, 7};
  int steps = 0;
  while (t0 < T1) {
    if (steps >= cfg.max_steps) { R.status = ST_MAX_STEPS; break; }
    const double dt = t1 - t0;
    double ss = 0.0;
    for (int b = 0; b < B; ++b) {
      const double k = ks[b];
      jacobian(c, D, k, t0, y[b].data(), J.data(), yd, fd);
      const double dtg = dt * R_gamma;
      for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) J[(size_t)i * n + j] = (i == j ? 1.0 / dtg : 0.0) - J[(size_t)i * n + j];
      lu_factor(J.data(), n, piv.data());
      dfdt(c, D, k, t0, y[b].data(), dT.data(), yd, fd);
      double* Kb = K[b].data();
      for (int st = 0; st < 8; ++st) {
        double* kst = &Kb[(size_t)st * n];
        if (st == 0) {
          for (int i = 0; i < n; ++i) u[i] = y[b][i];
        } else if (st <= 5) {
          for (int i = 0; i < n; ++i) { double acc = y[b][i]; for (int j = 0; j < st; ++j) acc += R_a[st][j] * Kb[(size_t)j * n + i]; u[i] = acc; }
        } else {
          for (int i = 0; i < n; ++i) u[i] += Kb[(size_t)(st - 1) * n + i];
        }
        rhs<double>(c, D, k, t0 + R_c[st] * dt, u.data(), du.data());
        for (int i = 0; i < n; ++i) {
          double r = du[i];
          if (st <= 4) r += dt * R_d[st] * dT[i];
          double acc = 0.0;
          for (int j = 0; j < st; ++j) acc += (R_C[st][j] / dt) * Kb[(size_t)j * n + i];
          kst[i] = r + acc;
        }
        lu_solve(J.data(), n, piv.data(), kst);
      }
      const double* k8 = &Kb[(size_t)7 * n];
      bool nan = false;
      for (int i = 0; i < n; ++i) { y1[b][i] = u[i] + k8[i]; if (!std::isfinite(y1[b][i])) nan = true; }
      const double err_w[6] = {1.0, k * k, 1.0, 1.0, 1.0 / (k * k), 1.0};
      for (int m = 0; m < 6; ++m) {
        int i = err_idx[m];
        double yc = nan ? y[b][i] : y1[b][i];
        double s = k8[i] / (cfg.atol + std::max(std::fabs(y[b][i]), std::fabs(yc)) * cfg.rtol);
        s *= err_w[m];
        ss += s * s;
      }
    }
    double err = std::sqrt(ss / (6.0 * B));
    if (!std::isfinite(err)) { R.status = ST_NONFINITE; break; }
    bool keep = err < 1.0;
    double inv = 1.0 / err;
    double f1 = beta1 == 0.0 ? 1.0 : std::pow(inv, beta1);
    double f2 = beta2 == 0.0 ? 1.0 : std::pow(prev_inv, beta2);
    double f3 = beta3 == 0.0 ? 1.0 : std::pow(prev_prev_inv, beta3);
    double factor = cfg.safety * f1 * f2 * f3;
    double fmin = keep ? 1.0 : cfg.fmin;
    factor = std::min(std::max(factor, fmin), cfg.fmax);
    double dtn = dt * factor;
    if (inv == 0.0 || std::isinf(inv)) inv = 1.0;
    ++steps;
    if (keep) {
      ++R.accepted;
      while (next_out < nout && tau_out[order[next_out]] <= t1) {
        double tt = tau_out[order[next_out]];
        double cf = (tt - t0) / (t1 - t0);
        for (int b = 0; b < B; ++b) {
          for (int i = 0; i < n; ++i) sc[i] = y[b][i] + cf * (y1[b][i] - y[b][i]);
          outputs(c, D, ks[b], sc.data(), yout + ((size_t)b * nout + order[next_out]) * 20);
        }
        ++next_out;
      }
      for (int b = 0; b < B; ++b) std::swap(y[b], y1[b]);
      t0 = t1;
      prev_prev_inv = prev_inv;
      prev_inv = inv;
    } else {
      ++R.rejected;
      if (cfg.hist_on_reject) { prev_prev_inv = prev_inv; prev_inv = inv; }
    }
    double tn = t0 + dtn;
    if (tn > T1 - 1e-10) tn = T1;
    if (!(tn > t0)) { if (t0 < T1) { R.status = ST_DT_UNDERFLOW; break; } }
    t1 = tn;
  }
  return R;
}

}  // namespace

extern "C" {

// Groups of batch_size consecutive modes of one cosmology sharing one step
// sequence (evolve_perturbations_batched, perturbations.py:1000-1061);
// arguments as oracle_solve, nmode a multiple of batch_size, no return_full.
int oracle_solve_grouped(const double* tables, int ncosmo, int blob_len, const double* kmodes, const int* cosmo_of_mode,
                         int nmode, const double* tau_out, int nout, const int* dims, const double* cfgv, int max_steps,
                         int batch_size, double* y_out, int* stats, int nthreads) {
  if (ncosmo <= 0 || nmode < 0 || nout <= 0 || batch_size < 1 || nmode % batch_size) return -1;
  std::vector<Cosmo> cs(ncosmo);
  for (int i = 0; i < ncosmo; ++i) if (!load_cosmo(tables + (size_t)i * blob_len, cs[i])) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  if (D.lg < 3 || D.lgp < 3 || D.lr < 3 || D.lnu < 3) return -3;
  for (int i = 0; i < ncosmo; ++i) if (cs[i].nq != D.nq) return -4;
  Cfg cfg{cfgv[0], cfgv[1], cfgv[2], cfgv[3], cfgv[4], cfgv[5], cfgv[6], cfgv[7], cfgv[8], max_steps, (int)cfgv[9], 0};
  const int ngroup = nmode / batch_size;
  for (int g = 0; g < ngroup; ++g) {
    const int c0 = cosmo_of_mode ? cosmo_of_mode[g * batch_size] : 0;
    for (int b = 1; b < batch_size; ++b) if ((cosmo_of_mode ? cosmo_of_mode[g * batch_size + b] : 0) != c0) return -5;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int g = 0; g < ngroup; ++g) {
    const int m0 = g * batch_size;
    const int ci = cosmo_of_mode ? cosmo_of_mode[m0] : 0;
    double* dst = y_out + (size_t)m0 * nout * 20;
    std::fill(dst, dst + (size_t)batch_size * nout * 20, std::numeric_limits<double>::quiet_NaN());
    ModeResult r = solve_group(cs[ci], D, kmodes + m0, batch_size, tau_out + (size_t)ci * nout, nout, cfg, dst);
    for (int b = 0; b < batch_size; ++b) {
      stats[3 * (m0 + b)] = r.status; stats[3 * (m0 + b) + 1] = r.accepted; stats[3 * (m0 + b) + 2] = r.rejected;
    }
  }
  (void)nthreads;
  return 0;
}

int oracle_n_vars(int lg, int lgp, int lr, int lnu, int nq) { return make_dims(lg, lgp, lr, lnu, nq).n; }

// Solve nmode modes.  tables: [ncosmo, blob_len]; tau_out: [ncosmo, nout];
// dims = {lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax}; cfg = {rtol, atol, pcoeff,
// icoeff, dcoeff, factormax, factormin, error_order, safety, hist_on_reject,
// step_to_outputs};
// y_out: [nmode, nout, 20 or n]; stats: [nmode, 3] = status, accepted, rejected.
int oracle_solve(const double* tables, int ncosmo, int blob_len, const double* kmodes, const int* cosmo_of_mode,
                 int nmode, const double* tau_out, int nout, const int* dims, const double* cfgv, int max_steps,
                 int return_full, double* y_out, int* stats, int nthreads) {
  if (ncosmo <= 0 || nmode < 0 || nout <= 0) return -1;
  std::vector<Cosmo> cs(ncosmo);
  for (int i = 0; i < ncosmo; ++i) if (!load_cosmo(tables + (size_t)i * blob_len, cs[i])) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  if (D.lg < 3 || D.lgp < 3 || D.lr < 3 || D.lnu < 3) return -3;
  for (int i = 0; i < ncosmo; ++i) if (cs[i].nq != D.nq) return -4;
  Cfg cfg{cfgv[0], cfgv[1], cfgv[2], cfgv[3], cfgv[4], cfgv[5], cfgv[6], cfgv[7], cfgv[8], max_steps, (int)cfgv[9],
          (int)cfgv[10]};
  const int osz = return_full ? D.n : 20;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int m = 0; m < nmode; ++m) {
    int ci = cosmo_of_mode ? cosmo_of_mode[m] : 0;
    double* dst = y_out + (size_t)m * nout * osz;
    std::fill(dst, dst + (size_t)nout * osz, std::numeric_limits<double>::quiet_NaN());
    ModeResult r = solve_mode(cs[ci], D, kmodes[m], tau_out + (size_t)ci * nout, nout, cfg, return_full, dst);
    stats[3 * m] = r.status; stats[3 * m + 1] = r.accepted; stats[3 * m + 2] = r.rejected;
  }
  (void)nthreads;
  return 0;
}

int oracle_rhs(const double* blob, const int* dims, double k, double tau, const double* y, double* f) {
  Cosmo c; if (!load_cosmo(blob, c)) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  rhs<double>(c, D, k, tau, y, f);
  return 0;
}

int oracle_jacobian(const double* blob, const int* dims, double k, double tau, const double* y, double* J, double* dT) {
  Cosmo c; if (!load_cosmo(blob, c)) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  std::vector<Dual> yd(D.n), fd(D.n);
  jacobian(c, D, k, tau, y, J, yd, fd);
  if (dT) dfdt(c, D, k, tau, y, dT, yd, fd);
  return 0;
}

int oracle_initial(const double* blob, const int* dims, double k, double tau_out_min, double* tau_start, double* y0) {
  Cosmo c; if (!load_cosmo(blob, c)) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  double t0 = 0.99 * std::min(tau_out_min, start_time(c, k));
  *tau_start = t0;
  initial_conditions(c, D, k, t0, y0);
  return 0;
}

int oracle_outputs(const double* blob, const int* dims, double k, const double* y, double* out20) {
  Cosmo c; if (!load_cosmo(blob, c)) return -2;
  Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  outputs(c, D, k, y, out20);
  return 0;
}

int oracle_spline_eval(const double* blob, int which, const double* x, int nx, double* out) {
  Cosmo c; if (!load_cosmo(blob, c)) return -2;
  if (which < 0 || which >= NSPL) return -3;
  for (int i = 0; i < nx; ++i) out[i] = spline_eval(c.sp[which], x[i]);
  return 0;
}

}  // extern "C"
