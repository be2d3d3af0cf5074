// deb_core.cuh -- per-mode perturbation solver: physics, structured linear
// algebra, Rodas5 step and PID control.  Written once as host/device code:
// the CUDA kernel (deb_solver.cu) runs it with one thread per k-mode; the
// test suite also compiles it for the host to check the exact kernel logic
// against the oracle without a GPU.
//
// Reference correspondence (file:line of DISCO-EB):
//   spline evaluate            src/discoeb/spline_interpolation.py:130-153
//   conformal Hubble rate      src/discoeb/background.py:100-122
//   synchronous-gauge RHS      src/discoeb/perturbations.py:84-371 (nu_perturb :22-50)
//   output conversion          src/discoeb/perturbations.py:374-523
//   adiabatic ICs              src/discoeb/perturbations.py:526-627
//   start time                 src/discoeb/perturbations.py:630-681, util.py:365-396
//   Rodas5 transformed step    src/discoeb/ode_integrators_stiff.py:622-834
//   PID control + error norm   src/discoeb/perturbations.py:701-724, 756-771
//
// Linear algebra.  The reference factors W = I/(gamma h) - J densely (LU
// with partial pivoting).  Here W is factored exactly through its structure:
//   * row 0 (a' depends only on a) is solved first and column 0 moved to the
//     right-hand side; variable 1 (a h', never read by the RHS) is solved last;
//   * the remaining J is  B + u_h g_h^T + u_e g_e^T : B holds the local
//     couplings (tridiagonal multipole chains, an 8x8 photon-baryon core,
//     2x2 CDM and DE blocks) and the two rank-1 terms are the metric
//     functionals h' and eta' that every species reads;
//   * M = I/(gamma h) - B is factored block by block (chain tails eliminated
//     from lmax downwards, 8x8 core with partial pivoting) and the rank-2
//     term is applied exactly with the Woodbury identity.
// The result equals the dense solution to rounding; the work is O(n).
#pragma once

#include <cstring>
#include <type_traits>

#ifdef __CUDACC__
#define HD __host__ __device__ __forceinline__
#ifdef __CUDA_ARCH__
#define LDG(p) __ldg(p)
#else
#define LDG(p) (*(p))
#endif
#else
#include <cmath>
#include <algorithm>
#define HD inline
#define LDG(p) (*(p))
#endif

namespace deb {

#ifndef __CUDACC__
using std::exp; using std::log; using std::sqrt; using std::fabs; using std::pow;
using std::min; using std::max;
HD bool isfinite_(double x) { return std::isfinite(x); }
#else
HD bool isfinite_(double x) { return isfinite(x); }
#endif

// Reciprocal for nonzero normal arguments whose reciprocal is normal (all
// uses here: pivots, a, tau, aH, error scales).  Device: the
// PTX approximate reciprocal as seed (relative error below 2^-19), then one
// third-order Newton-Raphson step y <- y (1 + e + e^2), e = 1 - x y, whose
// error e^3 < 2^-57 leaves at most 1 ulp; three FMAs where an FP64
// division costs several times as many FP64 instructions.
HD double rcp(double x) {
#ifdef __CUDA_ARCH__
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
#else
  return 1.0 / x;
#endif
}
// Ordering key of |x| from the high word of its bit pattern: integer
// compares choose pivots without FP64 instructions (ties within 2^-20
// relative are broken by index, harmless for partial pivoting).
HD int abs_key(double x) {
#ifdef __CUDA_ARCH__
  return __double2hiint(x) & 0x7fffffff;
#else
  unsigned long long u;
  std::memcpy(&u, &x, 8);
  return (int)((u >> 32) & 0x7fffffffu);
#endif
}
#ifdef __CUDACC__
HD double rsqrt_(double x) { return rsqrt(x); }
#else
HD double rsqrt_(double x) { return 1.0 / std::sqrt(x); }
#endif

// ------------------------------------------------------------------ blob layout
enum { H_OMEGAM = 0, H_OMEGAB, H_OMEGADE, H_OMEGAK, H_GRHOM, H_GRHOG, H_GRHOR, H_NEFF, H_NMNU,
       H_AMNU, H_W0, H_WA, H_CS2DE, H_YHE, H_H0, H_TAUMIN, H_AS, H_NS, H_KP, H_NQ,
       H_NSPL0 = 20, H_BLOBLEN = 27, H_MAGIC = 28, H_DERIVED = 29, HDR_LEN = 32 };
enum { SP_XE_LOGA = 0, SP_CS2A_LOGA, SP_LRHONU_LOGA, SP_LPNU_LOGA, SP_A_TAU, SP_TAU_A, SP_XE_TAU, NSPL };
constexpr double TABLE_MAGIC = 20231103.0;

enum { ST_OK = 0, ST_MAX_STEPS = 1, ST_DT_UNDERFLOW = 2, ST_NONFINITE = 3, ST_BAD_INPUT = 4 };

constexpr int LMAX_TABLE = 128;

// ------------------------------------------------------------------ dual numbers
// Forward-mode scalar for the a-column of the Jacobian (d f / d a).
struct Dual {
  double v, d;
  HD Dual() : v(0), d(0) {}
  HD Dual(double x) : v(x), d(0) {}
  HD Dual(double x, double dx) : v(x), d(dx) {}
};
HD Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
HD Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
HD Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
HD Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
HD Dual operator/(Dual a, Dual b) { double r = rcp(b.v); double q = a.v * r; return Dual(q, (a.d - q * b.d) * r); }
HD Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
HD Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
HD Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
HD Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
HD Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
HD Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
HD Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
HD Dual operator/(double a, Dual b) { double r = rcp(b.v); double q = a * r; return Dual(q, -q * b.d * r); }
HD Dual dexp(Dual a) { double e = exp(a.v); return Dual(e, e * a.d); }
HD Dual dlog(Dual a) { return Dual(log(a.v), a.d / a.v); }
HD Dual dsqrt(Dual a) { double s = sqrt(a.v); return Dual(s, 0.5 * a.d / s); }
HD double dexp(double a) { return exp(a); }
HD double dlog(double a) { return log(a); }
HD double dsqrt(double a) { return sqrt(a); }
HD Dual drsqrt(Dual a) { double r = rsqrt_(a.v); return Dual(r, -0.5 * r * r * r * a.d); }
HD double drsqrt(double a) { return rsqrt_(a); }
HD Dual drcp(Dual a) { double r = rcp(a.v); return Dual(r, -r * r * a.d); }
HD double drcp(double a) { return rcp(a); }
HD double val(double x) { return x; }
HD double val(Dual x) { return x.v; }
HD double der(double) { return 0.0; }
HD double der(Dual x) { return x.d; }
template <class S> HD S make_var(double v);
template <> HD double make_var<double>(double v) { return v; }
template <> HD Dual make_var<Dual>(double v) { return Dual(v, 1.0); }
template <class S> HD S mk(double v, double d);
template <> HD double mk<double>(double v, double) { return v; }
template <> HD Dual mk<Dual>(double v, double d) { return Dual(v, d); }

// ------------------------------------------------------------------ tables
// x, y, S: the reference's spline fields; c: per-interval polynomial
// coefficients (4 per interval); xf: knots rounded to FP32 for the search.
struct Spl { const double *x, *y, *S, *c; const float* xf; int n; };

struct Cosmo {
  const double* b;
  Spl sp[NSPL];
  const double *q, *w;
  int nq;
};

HD bool load_cosmo(const double* b, int blob_len, Cosmo& c) {
  if (LDG(b + H_MAGIC) != TABLE_MAGIC) return false;
  c.b = b;
  c.nq = (int)LDG(b + H_NQ);
  const double* p = b + HDR_LEN;
  long tot = HDR_LEN;
  for (int s = 0; s < NSPL; ++s) {
    int n = (int)LDG(b + H_NSPL0 + s);
    if (n < 2) return false;
    c.sp[s].n = n; c.sp[s].x = p; c.sp[s].y = p + n; c.sp[s].S = p + 2 * n;
    p += 3 * n; tot += 3 * n;
  }
  c.q = p; c.w = p + c.nq;
  tot += 2 * c.nq;
  const long doff = (long)LDG(b + H_DERIVED);
  if (doff != tot) return false;
  const double* dp = b + doff;
  for (int s = 0; s < NSPL; ++s) {
    const int n = c.sp[s].n;
    c.sp[s].c = dp;
    dp += 4 * (n - 1);
    c.sp[s].xf = reinterpret_cast<const float*>(dp);
    dp += (n + 1) / 2;
    tot += 4 * (n - 1) + (n + 1) / 2;
  }
  return tot <= blob_len && (int)LDG(b + H_BLOBLEN) == blob_len;
}

HD double hdr(const Cosmo& c, int i) { return LDG(c.b + i); }

// left searchsorted clipped to [0, n-2] (spline_interpolation.py:143): the
// largest i with x[i] < xv, or 0.  An FP32 binary search on the rounded knots
// lands within a knot or two; FP64 compares then fix the index exactly.
HD int spl_locate(const Spl& s, double xv) {
  const float xfv = (float)xv;
  int lo = 0, hi = s.n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (LDG(s.xf + mid) < xfv) lo = mid + 1; else hi = mid;
  }
  int i = lo - 1;
  i = i < 0 ? 0 : i;
  i = i > s.n - 2 ? s.n - 2 : i;
  while (i > 0 && !(LDG(s.x + i) < xv)) --i;
  while (i < s.n - 2 && LDG(s.x + i + 1) < xv) ++i;
  return i;
}

// Natural cubic spline value (spline_interpolation.py:130-153) in polynomial
// form about the left knot.
template <class S> HD S spl_eval(const Spl& s, S x) {
  const int i = spl_locate(s, val(x));
  const double* cf = s.c + 4 * i;
  const S u = x - LDG(s.x + i);
  return LDG(cf) + u * (LDG(cf + 1) + u * (LDG(cf + 2) + u * LDG(cf + 3)));
}

// ------------------------------------------------------------------ dimensions
struct Dims {
  int lg, lgp, lr, lnu, nq, n;
  int igp, ir, iq0;
};

HD Dims make_dims(int lg, int lgp, int lr, int lnu, int nq) {
  Dims d;
  d.lg = lg; d.lgp = lgp; d.lr = lr; d.lnu = lnu; d.nq = nq;
  d.n = 7 + (lg + 1) + (lgp + 1) + (lr + 1) + nq * (lnu + 1) + 2;
  d.igp = 8 + lg; d.ir = 9 + lg + lgp; d.iq0 = 10 + lg + lgp + lr;
  return d;
}

// ------------------------------------------------------------------ workspace
// Per-mode scratch: NV vectors of length n plus a MISC block.  Two state
// vectors swap roles on every accepted step: y0, and the stage state that
// ends the step holding y1.  The RHS writes straight into the stage vector
// it feeds.  Slot layout:
// [vectors 0 .. V_K0-1][MISC][stage vectors k1..k8]; element e of a slot lives
// at base[e * stride] (stride 32 interleaves the 32 modes of a warp so that
// every access of the warp is one coalesced transaction).  The warp-per-mode
// kernel keeps the first two parts in shared memory and may keep the stage
// vectors in global memory (kp).
enum { V_Y = 0, V_U, V_JC0, V_LO, V_UP, V_PI, V_ZH, V_ZE, V_K0, NV = V_K0 + 8 };
// MISC block offsets
enum { M_CORE = 0,          // 8x8 core LU (row-major)           64
       M_CPIV = 64,         // (unused)                             8
       M_DE = 72,           // DE 2x2 LU + pivot flag              5
       M_CINV = 77,         // Woodbury capacitance inverse        4
       M_SCAL = 81,         // cached per-step scalars            56
       M_CINV8 = 137,       // explicit inverse of the 8x8 core    64
       M_Q = 201 };         // per-q arrays: v, dv/da, dlfdlq, ghq, geq, r1q, dTq, m_nu/q  (8 nq)
enum { Q_V = 0, Q_DV, Q_DLF, Q_DT, Q_AMQ, NQARR };
// After the per-q arrays: three gather lists of nq + 6 coefficients each --
// the metric functionals h' and eta' as rows (d h'/d y, d eta'/d y) and row 1
// of J -- over the elements gather_index() names, so that each product is
// one lane-parallel FMA plus one reduction.
enum { GL_H = 0, GL_E, GL_R1, NGL };
enum { S_D = 0, S_W00I, S_ID, S_IDAH,
       S_FT, S_FP,     // folds of the photon T / P tails into the core diagonal
       S_LEAD = 8,     // RHS lead rows: per-call scalars sigma[17], derived values [5] (22)
       S_LEADD = 32 }; // and their d / d a (forward-mode RHS)                          (22)
HD int misc_len(int nq) { return M_Q + NQARR * nq + NGL * (nq + 6); }
HD int gl_off(int nq, int list) { return M_Q + NQARR * nq + list * (nq + 6); }

// element of the state read by entry t of gather list `list` (t < nq + 6):
// the massive-neutrino l = 0 (h', row 1) or l = 1 (eta') moments first, then
// six (five for eta', plus one zero entry) fluid / metric elements
HD int gather_index(const Dims& D, int list, int t) {
  if (t < D.nq) return D.iq0 + (list == GL_E ? D.nq : 0) + t;
  const int u = t - D.nq;
  if (list == GL_H) return u == 0 ? 2 : u == 1 ? 3 : u == 2 ? 5 : u == 3 ? 7 : u == 4 ? D.ir : D.n - 2;
  if (list == GL_E) return u == 0 ? 4 : u == 1 ? 6 : u == 2 ? 8 : u == 3 ? D.ir + 1 : D.n - 1;
  return u == 0 ? 3 : u == 1 ? 5 : u == 2 ? 7 : u == 3 ? D.ir : u == 4 ? D.n - 2 : D.n - 1;
}
HD long slot_len(const Dims& D) { return (long)NV * D.n + misc_len(D.nq); }
HD long hot_len(const Dims& D) { return (long)V_K0 * D.n + misc_len(D.nq); }     // vectors before k1 + MISC
HD long stage_len(const Dims& D) { return (long)(NV - V_K0) * D.n; }             // k1..k8
HD long dense_len(const Dims& D) { return (long)D.n * D.n + D.n; }

// Element stride follows the group width: one thread per mode interleaves
// the 32 modes of a warp (stride 32), one warp per mode is contiguous.
template <int G>
struct WS {
  static constexpr int S = (G == 1) ? 32 : 1;
  double* p;      // vectors 0 .. V_K0-1, then MISC at misc0 = V_K0 n
  double* kp;     // stage vectors: element (s, j) of k_{s+1} at kp[(s n + j) S]
  int n;
  int misc0;
  double* dp;     // dense matrix + pivots (dense path only)
  HD double& v(int vec, int j) const { return vec < V_K0 ? p[(vec * n + j) * S] : kp[((vec - V_K0) * n + j) * S]; }
  HD double& m(int off) const { return p[(misc0 + off) * S]; }
  HD double& e(int off) const { return dp[off * S]; }
};

// A group of G lanes that cooperates on one mode: G = 1 (one thread per
// mode; also the host build) or G = 32 (one warp per mode, state in shared
// memory).  Vector loops stride by G, chains are spread over lanes, scalar
// work is done redundantly or by the leading lane.  No sync/shuffle may sit
// inside a lane-divergent branch.
template <int G>
struct Grp {
  int lane;
  HD bool lead() const { return lane == 0; }
  HD void sync() const {
#ifdef __CUDA_ARCH__
    if (G > 1) __syncwarp();
#endif
  }
  HD double sum(double x) const {
#ifdef __CUDA_ARCH__
    if (G > 1)
      for (int o = G / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
#endif
    return x;
  }
  HD Dual sum(Dual x) const { Dual r = x; sum2(r.v, r.d); return r; }
  // Two or three sums at once.  Every FP64 add costs a full issue slot of the
  // FP64 unit whatever the number of active lanes, so the first exchanges
  // split the values over half- and quarter-warps: 5 adds for two sums and
  // 6 for three instead of 10 and 15.
  HD void sum2(double& a, double& b) const {
#ifdef __CUDA_ARCH__
    if (G == 32) {
      const bool lo = lane < 16;
      double k = (lo ? a : b) + __shfl_xor_sync(0xffffffffu, lo ? b : a, 16);
      for (int o = 8; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
      a = __shfl_sync(0xffffffffu, k, 0);
      b = __shfl_sync(0xffffffffu, k, 16);
      return;
    }
#endif
    a = sum(a);
    b = sum(b);
  }
  HD void sum3(double& a, double& b, double& c) const {
#ifdef __CUDA_ARCH__
    if (G == 32) {
      const bool lo = lane < 16, q = (lane & 8) == 0;
      const double k1 = (lo ? a : b) + __shfl_xor_sync(0xffffffffu, lo ? b : a, 16);    // lo: a, hi: b
      const double k2 = (lo ? c : 0.0) + __shfl_xor_sync(0xffffffffu, lo ? 0.0 : c, 16);  // lo: c, hi: 0
      double k = (q ? k1 : k2) + __shfl_xor_sync(0xffffffffu, q ? k2 : k1, 8);
      for (int o = 4; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
      a = __shfl_sync(0xffffffffu, k, 0);
      c = __shfl_sync(0xffffffffu, k, 8);
      b = __shfl_sync(0xffffffffu, k, 16);
      return;
    }
#endif
    a = sum(a);
    b = sum(b);
    c = sum(c);
  }
  HD double bcast(double x, int src) const {
#ifdef __CUDA_ARCH__
    if (G > 1) return __shfl_sync(0xffffffffu, x, src);
#endif
    return x;
  }
  HD Dual bcast(Dual x, int src) const { return Dual(bcast(x.v, src), bcast(x.d, src)); }
  HD bool any(bool b) const {
#ifdef __CUDA_ARCH__
    if (G > 1) return __any_sync(0xffffffffu, b);
#endif
    return b;
  }
  // index of the largest |value| (first index on ties) across the group
  HD void argmax(double& best, int& bi) const {
#ifdef __CUDA_ARCH__
    if (G > 1)
      for (int o = G / 2; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
#endif
  }
};

// ------------------------------------------------------------------ constants
struct Tab { double lo[LMAX_TABLE + 2], up[LMAX_TABLE + 2]; };  // l/(2l+1), (l+1)/(2l+1)

// Published transformed Rodas5 tableau (Hairer & Wanner), as listed in
// ode_integrators_stiff.py:622-687: identical coefficients are required for
// the reference's step sequence.
struct Rodas {
  double gamma;
  double a[8][8];
  double C[8][8];
  double c[8];
  double d[8];
};

// ------------------------------------------------------------------ scalars of the RHS at a given a
template <class S> struct Bg {
  S a, ia, ia2, a2, la, cs2, xe, rhonu, rhoQ, aH, iaH, wQ, ca2, opac, pb43;
};

struct ModeConst {
  double k, k2, ik, ik2;
  double Om, Ob, Oc, ODE, Ok, grhom, grhog, grhor, Neff, Nmnu, amnu, w0, wa, cs2Q, YHe, H0;
  double akthom, pQ, photbar0;
  // products of the constants above that the RHS uses every call
  double gOm, gOc, gOb, gODE, gOk, grN, grM, grr, grMk, g43g, g43N, pb43c;
};

HD void mode_const(const Cosmo& c, double k, ModeConst& m) {
  m.k = k; m.k2 = k * k; m.ik = 1.0 / k; m.ik2 = 1.0 / (k * k);
  m.Om = hdr(c, H_OMEGAM); m.Ob = hdr(c, H_OMEGAB); m.Oc = m.Om - m.Ob; m.ODE = hdr(c, H_OMEGADE);
  m.Ok = hdr(c, H_OMEGAK); m.grhom = hdr(c, H_GRHOM); m.grhog = hdr(c, H_GRHOG); m.grhor = hdr(c, H_GRHOR);
  m.Neff = hdr(c, H_NEFF); m.Nmnu = hdr(c, H_NMNU); m.amnu = hdr(c, H_AMNU); m.w0 = hdr(c, H_W0);
  m.wa = hdr(c, H_WA); m.cs2Q = hdr(c, H_CS2DE); m.YHe = hdr(c, H_YHE); m.H0 = hdr(c, H_H0);
  m.akthom = 2.3038921003709498e-9 * (1.0 - m.YHe) * m.Ob * m.H0 * m.H0;
  m.pQ = -3.0 * (1.0 + m.w0 + m.wa);
  m.photbar0 = m.grhog / (m.grhom * m.Ob);
  m.gOm = m.grhom * m.Om; m.gOc = m.grhom * m.Oc; m.gOb = m.grhom * m.Ob; m.gODE = m.grhom * m.ODE; m.gOk = m.grhom * m.Ok;
  m.grN = m.grhor * m.Neff; m.grM = m.grhor * m.Nmnu; m.grr = m.grhog + m.grN; m.grMk = m.grM * k;
  m.g43g = (4.0 / 3.0) * m.grhog; m.g43N = (4.0 / 3.0) * m.grN; m.pb43c = (4.0 / 3.0) * m.photbar0;
}

template <class S>
HD void background_finish(const ModeConst& m, S a, Bg<S>& g, S cs2a, S xe, S rhonu, S rhoQ) {
  g.cs2 = cs2a * g.ia;
  g.xe = xe;
  g.rhonu = rhonu;
  g.rhoQ = rhoQ;
  S grho = m.gOm * g.ia + (m.grr + m.grM * g.rhonu) * g.ia2 + m.gODE * g.rhoQ * g.a2 + m.gOk;
  const S g3 = grho * (1.0 / 3.0);
  g.iaH = drsqrt(g3);
  g.aH = g3 * g.iaH;
  g.wQ = m.w0 + m.wa * (1.0 - a);
  S wQp = -m.wa * g.aH * a;
  g.ca2 = g.wQ - wQp * (1.0 / 3.0) * drcp((1.0 + g.wQ) + 1e-6) * g.iaH;
  g.opac = g.xe * m.akthom * g.ia2;
  g.pb43 = m.pb43c * g.ia;
}

template <class S>
HD void background_start(S a, Bg<S>& g) {
  g.a = a;
  g.ia = drcp(a);
  g.ia2 = g.ia * g.ia;
  g.a2 = a * a;
  g.la = dlog(a);
}

template <class S>
HD void background(const Cosmo& c, const ModeConst& m, S a, Bg<S>& g) {
  background_start(a, g);
  // a^(-3(1+w0+wa)) exp(3(a-1) wa), background.py:111
  background_finish(m, a, g, spl_eval(c.sp[SP_CS2A_LOGA], g.la), spl_eval(c.sp[SP_XE_LOGA], g.la),
                    dexp(spl_eval(c.sp[SP_LRHONU_LOGA], g.la)), dexp(m.pQ * g.la + 3.0 * (a - 1.0) * m.wa));
}

// The same with the three spline look-ups on lanes 0..2 and the two
// exponentials on lanes 0..1 of a warp, broadcast by shuffles.
template <class S, int G>
HD void background_grp(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, S a, Bg<S>& g) {
  if constexpr (G == 1) {
    background(c, m, a, g);
  } else {
    background_start(a, g);
    const int which = gp.lane == 1 ? SP_XE_LOGA : (gp.lane == 2 ? SP_LRHONU_LOGA : SP_CS2A_LOGA);
    const S sv = spl_eval(c.sp[which], g.la);
    const S cs2a = gp.bcast(sv, 0), xe = gp.bcast(sv, 1), lrhonu = gp.bcast(sv, 2);
    const S ev = dexp(gp.lane == 0 ? lrhonu : S(m.pQ * g.la + 3.0 * (a - 1.0) * m.wa));
    background_finish(m, a, g, cs2a, xe, gp.bcast(ev, 0), gp.bcast(ev, 1));
  }
}

// conformal Hubble rate only (start time)
HD double aprimeoa(const Cosmo& c, const ModeConst& m, double a) {
  double la = log(a);
  double rhonu = exp(spl_eval(c.sp[SP_LRHONU_LOGA], la));
  double rhoQ = exp(m.pQ * la + 3.0 * (a - 1.0) * m.wa);
  double grho = m.grhom * m.Om / a + (m.grhog + m.grhor * (m.Neff + m.Nmnu * rhonu)) / (a * a) +
                m.grhom * m.ODE * rhoQ * a * a + m.grhom * m.Ok;
  return sqrt(grho / 3.0);
}

// ------------------------------------------------------------------ RHS lead rows
// The 21 RHS entries outside the hierarchy loops (metric, CDM, baryons,
// photon l = 0..2 and truncations, massless nu l = 0..2 and truncation, DE
// fluid), each written as a sum of at most six terms kappa * sigma * x:
// kappa a number, sigma one of the per-call scalars below, x a state element
// or a derived value.  One lane evaluates one row, so the whole block costs
// six multiply-adds per lane instead of ~130 scalar operations on one lane.
enum { SG_ONE = 0, SG_K, SG_K2, SG_OP, SG_AH, SG_A, SG_AHA, SG_KCS, SG_PBO, SG_ITG, SG_ITP, SG_ITR, SG_W1, SG_DE1,
       SG_DE2, SG_DE3, SG_DE4, NSIG };
enum { DV_HP = 0, DV_ETAP, DV_ALPHA, DV_P1, DV_ONE, NDV };
// index bases: absolute, igp, ir, n, 7 + lg, igp + lgp, ir + lr, derived value
enum { IB_ABS = 0, IB_IGP, IB_IR, IB_N, IB_LG7, IB_IGPL, IB_IRL, IB_DV };
struct LeadTerm { double kap; int base, off, sig; };
constexpr int NLEAD = 21, NLT = 6;
#define DEB_LEAD_ROWS {                                                                                               \
  /* a' = aH a */                                                                                                    \
  {{1.0, IB_DV, DV_ONE, SG_AHA}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},   \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* (a h')' = -(dgrho + 3 dgpres) a */                                                                              \
  {{-1.0, IB_DV, DV_P1, SG_A}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},    \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* eta' */                                                                                                         \
  {{1.0, IB_DV, DV_ETAP, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* delta_c' = -theta_c - h'/2 */                                                                                   \
  {{-1.0, IB_ABS, 4, SG_ONE}, {-0.5, IB_DV, DV_HP, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},  \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* theta_c' = -aH theta_c */                                                                                       \
  {{-1.0, IB_ABS, 4, SG_AH}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},      \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* delta_b' = -theta_b - h'/2 */                                                                                   \
  {{-1.0, IB_ABS, 6, SG_ONE}, {-0.5, IB_DV, DV_HP, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},  \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* theta_b' = -aH theta_b + k^2 cs2 delta_b + R opac (theta_g - theta_b) */                                        \
  {{-1.0, IB_ABS, 6, SG_AH}, {1.0, IB_ABS, 5, SG_KCS}, {1.0, IB_ABS, 8, SG_PBO}, {-1.0, IB_ABS, 6, SG_PBO},          \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* delta_g' = 4/3 (-theta_g - h'/2) */                                                                             \
  {{-4.0 / 3.0, IB_ABS, 8, SG_ONE}, {-2.0 / 3.0, IB_DV, DV_HP, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},                  \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                               \
  /* theta_g' = k^2 (delta_g/4 - sigma_g) - opac (theta_g - theta_b) */                                              \
  {{0.25, IB_ABS, 7, SG_K2}, {-0.5, IB_ABS, 9, SG_K2}, {-1.0, IB_ABS, 8, SG_OP}, {1.0, IB_ABS, 6, SG_OP},            \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* photon l = 2: 8/15 (theta_g + k^2 alpha) - 3/5 k F3 - opac (F2 - Pi / 10), Pi = F2 + G0 + G2 */                 \
  {{8.0 / 15.0, IB_ABS, 8, SG_ONE}, {8.0 / 15.0, IB_DV, DV_ALPHA, SG_K2}, {-0.6, IB_ABS, 10, SG_K},                  \
   {-0.9, IB_ABS, 9, SG_OP}, {0.1, IB_IGP, 0, SG_OP}, {0.1, IB_IGP, 2, SG_OP}},                                      \
  /* photon l = lmax: k F_{l-1} - (l + 1) / tau F_l - opac F_l */                                                    \
  {{1.0, IB_LG7, -1, SG_K}, {1.0, IB_LG7, 0, SG_ITG}, {-1.0, IB_LG7, 0, SG_OP}, {0, IB_DV, DV_ONE, SG_ONE},          \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* polarisation l = 0: -k G1 - opac G0 + opac Pi / 2 */                                                            \
  {{-1.0, IB_IGP, 1, SG_K}, {-0.5, IB_IGP, 0, SG_OP}, {0.5, IB_ABS, 9, SG_OP}, {0.5, IB_IGP, 2, SG_OP},              \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* polarisation l = 1: k (G0 / 3 - 2 G2 / 3) - opac G1 */                                                          \
  {{1.0 / 3.0, IB_IGP, 0, SG_K}, {-2.0 / 3.0, IB_IGP, 2, SG_K}, {-1.0, IB_IGP, 1, SG_OP}, {0, IB_DV, DV_ONE, SG_ONE}, \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* polarisation l = 2: k (2 G1 / 5 - 3 G3 / 5) - opac G2 + opac Pi / 10 */                                         \
  {{0.4, IB_IGP, 1, SG_K}, {-0.6, IB_IGP, 3, SG_K}, {-0.9, IB_IGP, 2, SG_OP}, {0.1, IB_ABS, 9, SG_OP},               \
   {0.1, IB_IGP, 0, SG_OP}, {0, IB_DV, DV_ONE, SG_ONE}},                                                              \
  /* polarisation l = lmax */                                                                                        \
  {{1.0, IB_IGPL, -1, SG_K}, {1.0, IB_IGPL, 0, SG_ITP}, {-1.0, IB_IGPL, 0, SG_OP}, {0, IB_DV, DV_ONE, SG_ONE},       \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* massless nu l = 0: 4/3 (-theta_r - h'/2) */                                                                     \
  {{-4.0 / 3.0, IB_IR, 1, SG_ONE}, {-2.0 / 3.0, IB_DV, DV_HP, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},                   \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                               \
  /* l = 1: k^2 (delta_r / 4 - sigma_r) */                                                                           \
  {{0.25, IB_IR, 0, SG_K2}, {-0.5, IB_IR, 2, SG_K2}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},          \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* l = 2: 8/15 (theta_r + k^2 alpha) - 3/5 k F3 */                                                                 \
  {{8.0 / 15.0, IB_IR, 1, SG_ONE}, {8.0 / 15.0, IB_DV, DV_ALPHA, SG_K2}, {-0.6, IB_IR, 3, SG_K},                     \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                               \
  /* l = lmax */                                                                                                     \
  {{1.0, IB_IRL, -1, SG_K}, {1.0, IB_IRL, 0, SG_ITR}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},         \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* DE fluid delta: -(1+w)(theta + h'/2) - 3 (cs2 - w) aH delta - 9 (1+w)(cs2 - ca2) aH^2 theta / k^2 */             \
  {{-1.0, IB_N, -1, SG_W1}, {-0.5, IB_DV, DV_HP, SG_W1}, {-1.0, IB_N, -2, SG_DE1}, {-1.0, IB_N, -1, SG_DE2},         \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}},                                                           \
  /* DE fluid theta: -(1 - 3 cs2) aH theta + cs2 / (1+w) k^2 delta */                                                \
  {{-1.0, IB_N, -1, SG_DE3}, {1.0, IB_N, -2, SG_DE4}, {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE},         \
   {0, IB_DV, DV_ONE, SG_ONE}, {0, IB_DV, DV_ONE, SG_ONE}}}
// row targets (base, offset), in the order above
#define DEB_LEAD_TARGETS {{IB_ABS, 0}, {IB_ABS, 1}, {IB_ABS, 2}, {IB_ABS, 3}, {IB_ABS, 4}, {IB_ABS, 5}, {IB_ABS, 6},   \
                          {IB_ABS, 7}, {IB_ABS, 8}, {IB_ABS, 9}, {IB_LG7, 0}, {IB_IGP, 0}, {IB_IGP, 1}, {IB_IGP, 2},  \
                          {IB_IGPL, 0}, {IB_IR, 0}, {IB_IR, 1}, {IB_IR, 2}, {IB_IRL, 0}, {IB_N, -2}, {IB_N, -1}}
#ifdef __CUDACC__
__device__ const LeadTerm d_lead_rows[NLEAD][NLT] = DEB_LEAD_ROWS;
__device__ const int d_lead_tgt[NLEAD][2] = DEB_LEAD_TARGETS;
#endif
static const LeadTerm h_lead_rows[NLEAD][NLT] = DEB_LEAD_ROWS;
static const int h_lead_tgt[NLEAD][2] = DEB_LEAD_TARGETS;

HD const LeadTerm& lead_term(int r, int t) {
#ifdef __CUDA_ARCH__
  return d_lead_rows[r][t];
#else
  return h_lead_rows[r][t];
#endif
}
HD int lead_tgt(int r, int f) {
#ifdef __CUDA_ARCH__
  return d_lead_tgt[r][f];
#else
  return h_lead_tgt[r][f];
#endif
}
// state index of (base, offset), or -1 - k for derived value k
HD int lead_index(const Dims& D, int base, int off) {
  switch (base) {
    case IB_IGP: return D.igp + off;
    case IB_IR: return D.ir + off;
    case IB_N: return D.n + off;
    case IB_LG7: return 7 + D.lg + off;
    case IB_IGPL: return D.igp + D.lgp + off;
    case IB_IRL: return D.ir + D.lr + off;
    case IB_DV: return -1 - off;
    default: return off;
  }
}

// ------------------------------------------------------------------ RHS
// f = model_synchronous(tau, y) (perturbations.py:84-371).  With S = Dual the
// a-dependence is differentiated: vout receives f, vjc receives d f / d a.
// With kAcc, f is added to vout instead.  Ends with a group sync; expects
// vin to be complete (synced) on entry.
template <class S, int G, bool kAcc = false>
HD void rhs(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T, double tau, const WS<G>& w,
            int vin, int vout, int vjc, Bg<double>* gout = nullptr) {
  constexpr bool kDual = !std::is_same<S, double>::value;
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, iq2 = iq1 + nq, iq3 = iq2 + nq;
  const int igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  const double k = m.k, k2 = m.k2;
  const double itau = rcp(tau);
  Bg<S> g;
  background_grp<S, G>(gp, c, m, make_var<S>(w.v(vin, 0)), g);
  if (gout) {
    gout->a = val(g.a); gout->ia = val(g.ia); gout->ia2 = val(g.ia2); gout->a2 = val(g.a2); gout->la = val(g.la);
    gout->cs2 = val(g.cs2); gout->xe = val(g.xe); gout->rhonu = val(g.rhonu); gout->rhoQ = val(g.rhoQ);
    gout->aH = val(g.aH); gout->iaH = val(g.iaH); gout->wQ = val(g.wQ); gout->ca2 = val(g.ca2);
    gout->opac = val(g.opac); gout->pb43 = val(g.pb43);
  }
  auto Y = [&](int j) -> double { return w.v(vin, j); };
  auto put = [&](int j, S f) {
    if constexpr (kAcc) w.v(vout, j) += val(f);
    else w.v(vout, j) = val(f);
    if constexpr (kDual) w.v(vjc, j) = der(f);
  };
  // massive neutrino momentum sums (nu_perturb, perturbations.py:22-50)
  S drhonu = 0.0, dpnu = 0.0, fnu = 0.0;
  for (int i = gp.lane; i < nq; i += G) {
    S aq = g.a * w.m(M_Q + Q_AMQ * nq + i);
    const S s2 = 1.0 + aq * aq;
    S v = drsqrt(s2);                           // v = 1 / sqrt(1 + (a m / q)^2)
    const double wq = LDG(c.w + i);
    const double wp0 = wq * Y(iq0 + i);
    drhonu = drhonu + wp0 * (s2 * v);
    dpnu = dpnu + wp0 * v;
    fnu = fnu + wq * Y(iq1 + i);
    w.m(M_Q + Q_V * nq + i) = val(v);         // v_q and d v_q / d a for the element loop
    if constexpr (kDual) w.m(M_Q + Q_DV * nq + i) = der(v);
  }
  if constexpr (kDual) {
    gp.sum3(drhonu.v, dpnu.v, fnu.v);
    gp.sum3(drhonu.d, dpnu.d, fnu.d);
  } else {
    gp.sum3(drhonu, dpnu, fnu);
  }
  gp.sync();
  dpnu = dpnu * (1.0 / 3.0);
  const double eta = Y(2), dc = Y(3), tc = Y(4), db = Y(5), tb = Y(6), dg = Y(7), tg = Y(8), y9 = Y(9);
  const double dr = Y(ir), tr = Y(ir + 1), y_r2 = Y(ir + 2);
  const double dq = Y(n - 2), tq = Y(n - 1);
  const S rQ = m.gODE * g.rhoQ * g.a2;   // grhom Omega_DE rho_Q(a) a^2
  S rptQ = (1.0 + g.wQ) * rQ * tq;
  S dgrho = (m.gOc * dc + m.gOb * db) * g.ia + (m.grhog * dg + m.grN * dr + m.grM * drhonu) * g.ia2 + rQ * dq;
  S hp = (2.0 * k2 * eta + dgrho) * g.iaH;
  S dgtheta = (m.gOc * tc + m.gOb * tb) * g.ia + (m.g43g * tg + m.g43N * tr + m.grMk * fnu) * g.ia2 + rptQ;
  S etap = 0.5 * dgtheta * m.ik2;
  // per-call scalars and derived values of the lead rows, through MISC
  if (gp.lead()) {
    const S dgpres = ((m.grhog * dg + m.grN * dr) * (1.0 / 3.0) + m.grM * dpnu) * g.ia2 +
                     (m.cs2Q * rQ * dq + (m.cs2Q - g.ca2) * (3.0 * g.aH * rptQ * m.ik2));
    const S w1 = 1.0 + g.wQ;
    const S sg[NSIG] = {S(1.0), S(k), S(k2), g.opac, g.aH, g.a, g.aH * g.a, k2 * g.cs2, g.pb43 * g.opac,
                        S(-(lg + 1.0) * itau), S(-(lgp + 1.0) * itau), S(-(lr + 1.0) * itau), w1,
                        3.0 * (m.cs2Q - g.wQ) * g.aH, 9.0 * w1 * (m.cs2Q - g.ca2) * g.aH * g.aH * m.ik2,
                        (1.0 - 3.0 * m.cs2Q) * g.aH, m.cs2Q * drcp(w1) * k2};
    const S dv[NDV] = {hp, etap, (hp + 6.0 * etap) * 0.5 * m.ik2, dgrho + 3.0 * dgpres, S(1.0)};
    for (int i = 0; i < NSIG; ++i) {
      w.m(M_SCAL + S_LEAD + i) = val(sg[i]);
      if constexpr (kDual) w.m(M_SCAL + S_LEADD + i) = der(sg[i]);
    }
    for (int i = 0; i < NDV; ++i) {
      w.m(M_SCAL + S_LEAD + NSIG + i) = val(dv[i]);
      if constexpr (kDual) w.m(M_SCAL + S_LEADD + NSIG + i) = der(dv[i]);
    }
  }
  gp.sync();
  auto scal = [&](int i) -> S {
    if constexpr (kDual) return mk<S>(w.m(M_SCAL + S_LEAD + i), w.m(M_SCAL + S_LEADD + i));
    else return w.m(M_SCAL + S_LEAD + i);
  };
  for (int r = gp.lane; r < NLEAD; r += G) {
    S acc = 0.0;
#pragma unroll
    for (int t = 0; t < NLT; ++t) {
      const LeadTerm& e = lead_term(r, t);
      const int src = lead_index(D, e.base, e.off);
      const S x = src >= 0 ? S(Y(src)) : scal(NSIG - 1 - src);
      acc = acc + (e.kap * scal(e.sig)) * x;
    }
    put(lead_index(D, lead_tgt(r, 0), lead_tgt(r, 1)), acc);
  }
  // photon T and P and massless nu hierarchies, 3 <= l < lmax, in one pass:
  // element e walks photon T, then P, then nu; only photons scatter
  {
    const int nt = lg - 3, np = lgp - 3, nr = lr - 3;
    for (int e = gp.lane; e < nt + np + nr; e += G) {
      const bool ph = e < nt + np;
      const int l = 3 + (e < nt ? e : (ph ? e - nt : e - nt - np));
      const int j = (e < nt ? 7 : (ph ? igp : ir)) + l;
      const S damp = ph ? g.opac : S(0.0);
      put(j, k * (T.lo[l] * Y(j - 1) - T.up[l] * Y(j + 1)) - damp * Y(j));
    }
  }
  // massive neutrinos, l-major [l][q].  l = 0, 1, 2 and lmax in one pass over
  // q, then 3 <= l < lmax with element e = (l - 3) nq + i walked as
  // incremental (l, i): every lane of a pass evaluates the same formula.
  const S hp6 = hp * (1.0 / 6.0);
  const S hp_eta = hp * (1.0 / 15.0) + 0.4 * etap;
  auto vq = [&](int i) -> S {
    if constexpr (kDual) return mk<S>(w.m(M_Q + Q_V * nq + i), w.m(M_Q + Q_DV * nq + i));
    else return w.m(M_Q + Q_V * nq + i);
  };
  for (int i = gp.lane; i < nq; i += G) {
    const S kv = k * vq(i);
    const double dlf = w.m(M_Q + Q_DLF * nq + i);
    const int jt = iq0 + lnu * nq + i;
    put(iq0 + i, -kv * Y(iq1 + i) + hp6 * dlf);
    put(iq1 + i, kv * (Y(iq0 + i) - 2.0 * Y(iq2 + i)) * (1.0 / 3.0));
    put(iq2 + i, kv * (2.0 * Y(iq1 + i) - 3.0 * Y(iq3 + i)) * 0.2 - hp_eta * dlf);
    put(jt, kv * Y(jt - nq) - (lnu + 1.0) * itau * Y(jt));
  }
  const int ngen = (lnu - 3) * nq;
  const int dl = G / nq, di = G - dl * nq;
  int l = 3 + gp.lane / nq, i = gp.lane - (l - 3) * nq;
  for (int e = gp.lane; e < ngen; e += G) {
    const int j = iq3 + e;
    put(j, k * vq(i) * (T.lo[l] * Y(j - nq) - T.up[l] * Y(j + nq)));
    l += dl;
    i += di;
    if (i >= nq) { i -= nq; ++l; }
  }
  gp.sync();
}

// ------------------------------------------------------------------ outputs
// convert_to_output_variables (perturbations.py:374-523) of the state held in
// vector vin; Friedmann aH from the tables, 20 fields to out[0..19*ostride].
// Scalar work: called by one lane.
template <int G>
HD void outputs(const Cosmo& c, const ModeConst& m, const Dims& D, const WS<G>& w, int vin, double* out, long ostride) {
  const int nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, n = D.n;
  const double k = m.k, k2 = m.k2;
  auto Y = [&](int j) -> double { return w.v(vin, j); };
  const double a = Y(0), eta = Y(2), dc = Y(3), tc = Y(4), db = Y(5), tb = Y(6), dg = Y(7), tg = Y(8);
  const double dr = Y(D.ir), tr = Y(D.ir + 1);
  const double la = log(a);
  const double rhonu = exp(spl_eval(c.sp[SP_LRHONU_LOGA], la));
  const double pnu = exp(spl_eval(c.sp[SP_LPNU_LOGA], la));
  double drhonu = 0.0, fnu = 0.0;
  for (int i = 0; i < nq; ++i) {
    const double aq = a * m.amnu / LDG(c.q + i);
    const double v = 1.0 / sqrt(1.0 + aq * aq);
    drhonu += LDG(c.w + i) * Y(iq0 + i) / v;
    fnu += LDG(c.w + i) * Y(iq1 + i);
  }
  const double dnu = drhonu / rhonu, tnu = k * fnu / (rhonu + pnu);
  const double dq = Y(n - 2), tq = Y(n - 1);
  const double wQ = m.w0 + m.wa * (1.0 - a);
  const double rhoQ = exp(m.pQ * la + 3.0 * (a - 1.0) * m.wa);
  const double a2 = a * a;
  const double rptQ = (1.0 + wQ) * rhoQ * m.grhom * m.ODE * tq * a2;
  const double grho = m.grhom * m.Om / a + (m.grhog + m.grhor * (m.Neff + m.Nmnu * rhonu)) / a2 +
                      m.grhom * m.ODE * rhoQ * a2 + m.grhom * m.Ok;
  const double aH = sqrt(grho / 3.0);
  const double dgrho = m.grhom * (m.Oc * dc + m.Ob * db) / a +
                       (m.grhog * dg + m.grhor * (m.Neff * dr + m.Nmnu * drhonu)) / a2 + m.grhom * m.ODE * dq * rhoQ * a2;
  const double dgtheta = m.grhom * (m.Oc * tc + m.Ob * tb) / a + 4.0 / 3.0 * (m.grhog * tg + m.Neff * m.grhor * tr) / a2 +
                         m.Nmnu * m.grhor * k * fnu / a2 + rptQ;
  const double hp = (2.0 * k2 * eta + dgrho) / aH;
  const double etap = 0.5 * dgtheta / k2;
  const double alpha = (hp + 6.0 * etap) / 2.0 / k2;
  const double dm = (m.grhom * (m.Oc * dc + m.Ob * db) / a + (m.grhor * m.Nmnu * drhonu) / a2) /
                    (m.grhom * m.Om / a + (m.grhor * m.Nmnu * rhonu) / a2);
  double tm = (m.grhom * (m.Oc * tc + m.Ob * tb) / a + m.Nmnu * m.grhor * k * fnu / a2) /
              (3.0 * (m.grhom * m.Om / a + m.grhor * m.Nmnu * rhonu / a2));
  const double dbc = (m.grhom * (m.Oc * dc + m.Ob * db) / a) / (m.grhom * m.Om / a);
  double tbc = (m.grhom * (m.Oc * tc + m.Ob * tb) / a) / (3.0 * (m.grhom * m.Om / a) / a2);
  tm += alpha * k2;
  tbc += alpha * k2;
  const double r[20] = {eta, etap, hp, alpha, dm, tm / aH, dbc, tbc / aH, dc, tc / aH, db, tb / aH,
                        dg, tg / aH, dr, tr / aH, dnu, tnu / aH, dq, tq / aH};
  for (int i = 0; i < 20; ++i) out[i * ostride] = r[i];
}

// ------------------------------------------------------------------ initial conditions
// adiabatic_ics_one_mode (perturbations.py:526-627), written into vector vout.
template <int G>
HD void initial_conditions(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, double tau, const WS<G>& w,
                           int vout) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, iq1 = iq0 + nq, iq2 = iq1 + nq;
  const double k = m.k;
  for (int j = gp.lane; j < n; j += G) w.v(vout, j) = 0.0;
  gp.sync();
  const double a = spl_eval(c.sp[SP_A_TAU], tau);
  const double rn = exp(spl_eval(c.sp[SP_LRHONU_LOGA], log(a)));
  const double a4 = a * a * a * a;
  const double rhom = m.grhom * m.Om / (a * a * a);
  const double rhor = (m.grhog + m.grhor * (m.Neff + m.Nmnu * rn)) / a4;
  const double rhonu = m.grhor * (m.Neff + m.Nmnu * rn) / a4;
  const double fracb = m.Ob / m.Om, fracnu = rhonu / rhor;
  const double om = a * rhom / sqrt(rhor);
  const double ci = -1.0, s2 = 1.0;
  const double kt = k * tau;
  const double dg = -(kt * kt) / 3.0 * (1.0 - om * tau / 5.0) * ci * s2;
  const double tg = -(kt * kt * kt) / tau / 36.0 *
                    (1.0 - 3.0 * (1.0 + 5.0 * fracb - fracnu) / 20.0 / (1.0 - fracnu) * om * tau) * ci * s2;
  const double dr = dg;
  const double tr = -(kt * kt * kt * kt) / tau / 36.0 / (4.0 * fracnu + 15.0) *
                    (4.0 * fracnu + 11.0 + 12.0 -
                     3.0 * (8.0 * fracnu * fracnu + 50.0 * fracnu + 275.0) / 20.0 / (2.0 * fracnu + 15.0) * tau * om) * ci;
  const double sr = (kt * kt) / (45.0 + 12.0 * fracnu) * (3.0 * s2 - 1.0) *
                    (1.0 + (4.0 * fracnu - 5.0) / 4.0 / (2.0 * fracnu + 15.0) * tau * om) * ci;
  if (gp.lead()) {
    const double wQ = m.w0 + m.wa * (1.0 - a);
    const double dq = (kt * kt) / 4.0 * (1.0 + wQ) * (4.0 - 3.0 * m.cs2Q) / (4.0 - 6.0 * wQ + 3.0 * m.cs2Q) * ci * s2;
    const double tq = (kt * kt * kt * kt) / tau / 4.0 * m.cs2Q / (4.0 - 6.0 * wQ + 3.0 * m.cs2Q) * ci * s2;
    const double eta = ci * (1.0 - (kt * kt) / 12.0 / (15.0 + 4.0 * fracnu) *
                                       (5.0 + 4.0 * s2 * fracnu -
                                        (16.0 * fracnu * fracnu + 280.0 * fracnu + 325.0) / 10.0 / (2.0 * fracnu + 15.0) * tau * om));
    w.v(vout, 0) = a; w.v(vout, 2) = eta; w.v(vout, 3) = 0.75 * dg;
    w.v(vout, 5) = 0.75 * dg; w.v(vout, 6) = tg; w.v(vout, 7) = dg; w.v(vout, 8) = tg;
    w.v(vout, D.ir) = dr; w.v(vout, D.ir + 1) = tr; w.v(vout, D.ir + 2) = sr * 2.0;
    w.v(vout, n - 2) = dq; w.v(vout, n - 1) = tq;
  }
  for (int i = gp.lane; i < nq; i += G) {
    const double q = LDG(c.q + i);
    const double aq = a * m.amnu / q;
    const double v = 1.0 / sqrt(1.0 + aq * aq);
    const double dlf = -q / (1.0 + exp(-q));
    w.v(vout, iq0 + i) = -0.25 * dlf * dr;
    w.v(vout, iq1 + i) = -dlf * tr / v / k / 3.0;
    w.v(vout, iq2 + i) = -0.5 * dlf * sr;
    w.m(M_Q + Q_DLF * nq + i) = dlf;
    w.m(M_Q + Q_AMQ * nq + i) = m.amnu / q;
  }
  gp.sync();
}

// determine_starting_time (perturbations.py:630-681) with root_find_bisect
// (util.py:365-396).  Scalar; every lane computes the same value.
HD double start_time(const Cosmo& c, const ModeConst& m) {
  const double small_k = 0.0004, large_k = 0.07;
  const double tau0 = hdr(c, H_TAUMIN);
  const double tau1 = spl_eval(c.sp[SP_TAU_A], 0.1);
  const double tau_k = 1.0 / m.k;
  const double akthom_st = 2.3048e-9 * (1.0 - m.YHe) * m.Ob * m.H0 * m.H0;  // as perturbations.py:648
  double lt[2];
  for (int which = 0; which < 2; ++which) {
    double xl = log(tau0), xr = log(tau1);
    for (int it = 0; it < 7; ++it) {
      const double xm = 0.5 * (xl + xr);
      double fv[2];
      for (int e = 0; e < 2; ++e) {
        const double tau = exp(e == 0 ? xm : xl);
        const double a = spl_eval(c.sp[SP_A_TAU], tau);
        const double aH = aprimeoa(c, m, a);
        if (which == 0) {
          fv[e] = (1.0 / aH) / tau_k / large_k - 1.0;
        } else {
          const double xe = spl_eval(c.sp[SP_XE_TAU], tau);
          const double opac = xe * akthom_st / (a * a);
          fv[e] = (1.0 / opac) / (1.0 / aH) / small_k - 1.0;
        }
      }
      if (fv[0] * fv[1] > 0.0) xl = xm; else xr = xm;
    }
    lt[which] = 0.5 * (xl + xr);
  }
  return exp(lt[1] < lt[0] ? lt[1] : lt[0]);
}

// ------------------------------------------------------------------ structured factorization
// Chains of M = d I - B (see file header).  A chain is the list of indices
// start, start + stride, ...; its raw entries are lo = M[i, prev] and
// up = M[i, next].  Bottom-up elimination: p_last = M_ii,
// p_i = M_ii - up_i lo_next / p_next.  Every chain pivot is >= d > 0:
// up_i lo_next < 0 for every free-streaming hierarchy and the diagonal
// damping (opacity, truncation (l+1)/tau) is non-negative.  Stored per
// element: PI = 1/p, UP = up / p_next (forward-sweep multiplier) and
// LO = lo / p (back-substitution multiplier), so each sweep step is one
// FMA on the dependency chain.
// Chain numbering: 0 massless nu, 1..nq massive nu q-1, nq+1 photon T tail
// (l >= 3, attached to T2 = index 9), nq+2 photon P tail (attached to P2).
struct Chain { int start, stride, cnt, attach, lmax, l0; double kv; };

template <int G>
HD Chain chain_of(const ModeConst& m, const Dims& D, const WS<G>& w, int ch) {
  Chain c;
  c.kv = m.k;
  if (ch == 0) { c.start = D.ir; c.stride = 1; c.cnt = D.lr + 1; c.attach = -1; c.lmax = D.lr; c.l0 = 0; }
  else if (ch <= D.nq) {
    c.start = D.iq0 + ch - 1; c.stride = D.nq; c.cnt = D.lnu + 1; c.attach = -1; c.lmax = D.lnu; c.l0 = 0;
    c.kv = m.k * w.m(M_Q + Q_V * D.nq + ch - 1);
  } else if (ch == D.nq + 1) { c.start = 10; c.stride = 1; c.cnt = D.lg - 2; c.attach = 9; c.lmax = D.lg; c.l0 = 3; }
  else { c.start = D.igp + 3; c.stride = 1; c.cnt = D.lgp - 2; c.attach = D.igp + 2; c.lmax = D.lgp; c.l0 = 3; }
  return c;
}

// raw entries of the chain element with multipole l (l = 2: a tail's attach
// row).  Massless nu l = 0..2 follow the fluid equations of the RHS.
HD void chain_entry(const ModeConst& m, const Tab& T, int ch, const Chain& c, int l, double& lo, double& up) {
  if (ch == 0 && l <= 2) {
    lo = l == 1 ? -0.25 * m.k2 : (l == 2 ? -8.0 / 15.0 : 0.0);
    up = l == 0 ? 4.0 / 3.0 : (l == 1 ? 0.5 * m.k2 : 0.6 * m.k);
  } else if (l == c.lmax) {
    lo = -c.kv; up = 0.0;
  } else if (c.attach >= 0 && l == 2) {
    lo = 0.0; up = 0.6 * m.k;
  } else {
    lo = -c.kv * T.lo[l]; up = c.kv * T.up[l];
  }
}

// Factor chain ch (one lane).  A tail also stores its attach multiplier and
// the fold up_attach lo_start / p_start of its elimination into the core.
template <int G>
HD void chain_factor(const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w, double d, double itau, double op,
                     int ch) {
  const Chain c = chain_of<G>(m, D, w, ch);
  const double d_rest = c.attach >= 0 ? d + op : d;
  int i = c.start + (c.cnt - 1) * c.stride;
  double lo, up;
  chain_entry(m, T, ch, c, c.l0 + c.cnt - 1, lo, up);
  double pinv = rcp(d_rest + (c.lmax + 1.0) * itau);
  w.v(V_PI, i) = pinv;
  w.v(V_LO, i) = lo * pinv;
  double lo_next = lo;
  for (int j = c.cnt - 2; j >= 0; --j) {
    i -= c.stride;
    chain_entry(m, T, ch, c, c.l0 + j, lo, up);
    const double qf = up * pinv;
    pinv = rcp(d_rest - qf * lo_next);
    w.v(V_UP, i) = qf;
    w.v(V_PI, i) = pinv;
    w.v(V_LO, i) = lo * pinv;
    lo_next = lo;
  }
  if (c.attach >= 0) {
    chain_entry(m, T, ch, c, 2, lo, up);
    const double qa = up * pinv;
    w.v(V_UP, c.attach) = qa;
    w.m(M_SCAL + (ch == D.nq + 1 ? S_FT : S_FP)) = qa * lo_next;
  }
}

// 8x8 core: explicit inverse by Gauss-Jordan elimination with partial
// pivoting, rows over lanes 0..7.  The matrix is in MISC column-major at
// M_CORE (overwritten), the inverse goes column-major to M_CINV8.  A pivot
// row stays unscaled until the end, so a step costs one reciprocal, one
// multiply per row and one FMA per remaining entry; rows are permuted into
// place with the final scaling.
template <int G>
HD void core_invert(const Grp<G>& gp, const WS<G>& w) {
  auto A = [&](int i, int j) -> double& { return w.m(M_CORE + j * 8 + i); };
  auto X = [&](int i, int j) -> double& { return w.m(M_CINV8 + j * 8 + i); };
  for (int e = gp.lane; e < 64; e += G) X(e & 7, e >> 3) = ((e & 7) == (e >> 3)) ? 1.0 : 0.0;
  gp.sync();
  unsigned done = 0u;
  int prow[8];
  double pinv[8];
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    int p = 0;
#ifdef __CUDA_ARCH__
    if (G == 32) {
      int key = (gp.lane < 8 && !((done >> gp.lane) & 1u)) ? abs_key(A(gp.lane, kk)) : -1;
      int idx = gp.lane;
      for (int o = 4; o > 0; o >>= 1) {
        const int ok = __shfl_xor_sync(0xffffffffu, key, o), oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ok > key || (ok == key && oi < idx)) { key = ok; idx = oi; }
      }
      p = __shfl_sync(0xffffffffu, idx, 0);
    } else
#endif
    {
      int best = -1;
      for (int i = 0; i < 8; ++i)
        if (!((done >> i) & 1u) && abs_key(A(i, kk)) > best) { best = abs_key(A(i, kk)); p = i; }
    }
    done |= 1u << p;
    prow[kk] = p;
    const double pi = rcp(A(p, kk));
    pinv[kk] = pi;
    for (int i = gp.lane; i < 8; i += G) {
      if (i != p) {
        const double f = A(i, kk) * pi;
        for (int j = kk + 1; j < 8; ++j) A(i, j) -= f * A(p, j);
        for (int j = 0; j < 8; ++j) X(i, j) -= f * X(p, j);
      }
    }
    gp.sync();
  }
  // row kk of the inverse = row prow[kk] / its pivot, through M_CORE
  for (int e = gp.lane; e < 64; e += G) {
    const int kk = e & 7, j = e >> 3;
    A(kk, j) = X(prow[kk], j) * pinv[kk];
  }
  gp.sync();
  for (int e = gp.lane; e < 64; e += G) X(e & 7, e >> 3) = A(e & 7, e >> 3);
  gp.sync();
}

// entries of the 8x8 photon-baryon core of M (db, tb, dg, tg, T2, P0, P1, P2)
// and of the 2x2 dark-energy block, before the tail folds
HD void core_entries(const ModeConst& m, const Tab& T, const Bg<double>& g, double d, double* core, double* de) {
  const double k = m.k, k2 = m.k2, op = g.opac;
  for (int i = 0; i < 64; ++i) core[i] = 0.0;
  core[0] = d; core[1] = 1.0;
  core[8] = -k2 * g.cs2; core[9] = d + g.aH + g.pb43 * op; core[11] = -g.pb43 * op;
  core[18] = d; core[19] = 4.0 / 3.0;
  core[25] = -op; core[26] = -0.25 * k2; core[27] = d + op; core[28] = 0.5 * k2;
  core[35] = -8.0 / 15.0; core[36] = d + 0.9 * op; core[37] = -0.1 * op; core[39] = -0.1 * op;
  core[44] = -0.5 * op; core[45] = d + 0.5 * op; core[46] = k; core[47] = -0.5 * op;
  core[53] = -k * T.lo[1]; core[54] = d + op; core[55] = k * T.up[1];
  core[60] = -0.1 * op; core[61] = -0.1 * op; core[62] = -k * T.lo[2]; core[63] = d + 0.9 * op;
  de[0] = d + 3.0 * (m.cs2Q - g.wQ) * g.aH;
  de[1] = (1.0 + g.wQ) + 9.0 * (1.0 + g.wQ) * (m.cs2Q - g.ca2) * g.aH * g.aH * m.ik2;
  de[2] = -m.cs2Q * rcp(1.0 + g.wQ) * k2;
  de[3] = d + (1.0 - 3.0 * m.cs2Q) * g.aH;
}

// Fill chain coefficients and factor M (chains per lane; core and DE on the
// leading lane).  Needs v_q in MISC (written by the RHS at this a).
template <int G>
HD void factor_M(const Grp<G>& gp, const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w, double d, double tau,
                 const Bg<double>& g) {
  const int nq = D.nq;
  const double itau = rcp(tau), op = g.opac;
  for (int ch = gp.lane; ch < nq + 3; ch += G) chain_factor<G>(m, D, T, w, d, itau, op, ch);
  gp.sync();
  if (gp.lead()) {
    double core[64], de[4];
    core_entries(m, T, g, d, core, de);
    core[36] -= w.m(M_SCAL + S_FT);
    core[63] -= w.m(M_SCAL + S_FP);
    for (int i = 0; i < 64; ++i) w.m(M_CORE + (i & 7) * 8 + (i >> 3)) = core[i];   // column-major
    // dark energy 2x2 (rows n-2, n-1): LU with partial pivoting, M_DE+4 = 1 if swapped
    double a00 = de[0], a01 = de[1], a10 = de[2], a11 = de[3];
    double sw = 0.0;
    if (fabs(a10) > fabs(a00)) { double t0_ = a00, t1_ = a01; a00 = a10; a01 = a11; a10 = t0_; a11 = t1_; sw = 1.0; }
    const double i00 = rcp(a00), l = a10 * i00;
    w.m(M_DE + 0) = i00; w.m(M_DE + 1) = a01; w.m(M_DE + 2) = l; w.m(M_DE + 3) = rcp(a11 - l * a01);
    w.m(M_DE + 4) = sw;
    w.m(M_SCAL + S_ID) = rcp(d);
    w.m(M_SCAL + S_IDAH) = rcp(d + g.aH);
  }
  gp.sync();
  // explicit inverse of the core, so each stage's core solve is an 8-lane
  // matrix-vector product
  core_invert<G>(gp, w);
}

// z = M^{-1} r on indices >= 2, in place on vector vr.  Expects vr synced.
template <int G>
HD void solve_M(const Grp<G>& gp, const ModeConst& m, const Dims& D, const WS<G>& w, double d, double aH, int vr) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  (void)m;
  (void)d; (void)aH;
  if (gp.lead()) {
    const double id = w.m(M_SCAL + S_ID);
    w.v(vr, 2) = w.v(vr, 2) * id;                      // eta
    const double z4 = w.v(vr, 4) * w.m(M_SCAL + S_IDAH);  // CDM [[d, 1], [0, d + aH]]
    w.v(vr, 4) = z4;
    w.v(vr, 3) = (w.v(vr, 3) - z4) * id;
    double r0 = w.v(vr, n - 2), r1 = w.v(vr, n - 1);   // DE
    if (w.m(M_DE + 4) != 0.0) { double t = r0; r0 = r1; r1 = t; }
    r1 -= w.m(M_DE + 2) * r0;
    const double z1 = r1 * w.m(M_DE + 3);
    const double z0 = (r0 - w.m(M_DE + 1) * z1) * w.m(M_DE + 0);
    w.v(vr, n - 2) = z0; w.v(vr, n - 1) = z1;
  }
  for (int ch = gp.lane; ch < nq + 3; ch += G) {
    // forward sweep from the top, r_i -= (up_i / p_next) r_next; a full chain
    // then back-substitutes from l = 0, a tail folds into its attach row
    const bool tail = ch > nq;
    const int start = ch == 0 ? ir : (!tail ? iq0 + ch - 1 : (ch == nq + 1 ? 10 : igp + 3));
    const int stride = (ch == 0 || tail) ? 1 : nq;
    const int cnt = ch == 0 ? lr + 1 : (!tail ? lnu + 1 : (ch == nq + 1 ? lg - 2 : lgp - 2));
    // groups of eight elements load ahead of their dependent FMAs, so the
    // memory latency (shared or L2) is paid once per group
    int i = start + (cnt - 1) * stride;
    double rn = w.v(vr, i);
    int j = cnt - 2;
    for (; j >= 7; j -= 8) {
      double rv[8], uv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) { rv[q] = w.v(vr, i - (q + 1) * stride); uv[q] = w.v(V_UP, i - (q + 1) * stride); }
#pragma unroll
      for (int q = 0; q < 8; ++q) { rn = rv[q] - uv[q] * rn; w.v(vr, i - (q + 1) * stride) = rn; }
      i -= 8 * stride;
    }
    for (; j >= 0; --j) {
      i -= stride;
      rn = w.v(vr, i) - w.v(V_UP, i) * rn;
      w.v(vr, i) = rn;
    }
    if (!tail) {
      double z = rn * w.v(V_PI, start);
      w.v(vr, start) = z;
      int jb = 1;
      for (; jb + 7 < cnt; jb += 8) {
        double sv[8], lv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int ii = i + (q + 1) * stride;
          sv[q] = w.v(vr, ii) * w.v(V_PI, ii);
          lv[q] = w.v(V_LO, ii);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) { z = sv[q] - lv[q] * z; w.v(vr, i + (q + 1) * stride) = z; }
        i += 8 * stride;
      }
      for (; jb < cnt; ++jb) {
        i += stride;
        z = w.v(vr, i) * w.v(V_PI, i) - w.v(V_LO, i) * z;
        w.v(vr, i) = z;
      }
    } else {
      w.v(vr, start - 1) -= w.v(V_UP, start - 1) * rn;
    }
  }
  gp.sync();
  {
    const int cidx[8] = {5, 6, 7, 8, 9, igp, igp + 1, igp + 2};
    double r[8];
    for (int j = 0; j < 8; ++j) r[j] = w.v(vr, cidx[j]);
    gp.sync();
    for (int row = gp.lane; row < 8; row += G) {
      double z = 0.0;
      for (int j = 0; j < 8; ++j) z += w.m(M_CINV8 + j * 8 + row) * r[j];
      w.v(vr, cidx[row]) = z;
    }
  }
  gp.sync();
  for (int t = gp.lane; t < 2; t += G) {
    const int start = t == 0 ? 10 : igp + 3;
    const int cnt = t == 0 ? lg - 2 : lgp - 2;
    double z = w.v(vr, start - 1);
    int j = 0;
    for (; j + 7 < cnt; j += 8) {
      double sv[8], lv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = start + j + q;
        sv[q] = w.v(vr, i) * w.v(V_PI, i);
        lv[q] = w.v(V_LO, i);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) { z = sv[q] - lv[q] * z; w.v(vr, start + j + q) = z; }
    }
    for (; j < cnt; ++j) {
      const int i = start + j;
      z = w.v(vr, i) * w.v(V_PI, i) - w.v(V_LO, i) * z;
      w.v(vr, i) = z;
    }
  }
  gp.sync();
}

// g_h . v and g_e . v (the metric functionals h', eta' as rows); all lanes get the sums
template <int G>
HD void functionals(const Grp<G>& gp, const Dims& D, const WS<G>& w, int vr, double& sh, double& se) {
  const int nq = D.nq, oh = gl_off(nq, GL_H), oe = gl_off(nq, GL_E);
  double h = 0.0, e = 0.0;
  for (int t = gp.lane; t < nq + 6; t += G) {
    h += w.m(oh + t) * w.v(vr, gather_index(D, GL_H, t));
    e += w.m(oe + t) * w.v(vr, gather_index(D, GL_E, t));
  }
  gp.sum2(h, e);
  sh = h;
  se = e;
}

// Per-step factorization of W = d I - J at (t0, y0).  Needs JC0 (d f/d a),
// the background g at a0 and v_q in MISC.  Writes LO/UP/PI, core/DE LU, ZH,
// ZE, the capacitance inverse and the sparse row-1 / functional coefficients.
template <int G>
HD void factor_W(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w,
                 double d, double tau, const Bg<double>& g) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, ir = D.ir;
  const double a = g.a, iaH = g.iaH, h2 = 0.5 * m.ik2;
  if (gp.lead()) {
    w.m(M_SCAL + S_D) = d;
    w.m(M_SCAL + S_W00I) = 1.0 / (d - w.v(V_JC0, 0));
    // functional coefficients (d h'/d y and d eta'/d y) and row 1,
    // J[1, j] = -a (d dgrho/d y_j + 3 d dgpres/d y_j); entries nq.. of the lists
    const int oh = gl_off(nq, GL_H) + nq, oe = gl_off(nq, GL_E) + nq, o1 = gl_off(nq, GL_R1) + nq;
    const double rQ = m.gODE * g.rhoQ * g.a2;
    w.m(oh + 0) = 2.0 * m.k2 * iaH;
    w.m(oh + 1) = m.gOc * g.ia * iaH;
    w.m(oh + 2) = m.gOb * g.ia * iaH;
    w.m(oh + 3) = m.grhog * g.ia2 * iaH;
    w.m(oh + 4) = m.grN * g.ia2 * iaH;
    w.m(oh + 5) = rQ * iaH;
    w.m(oe + 0) = m.gOc * g.ia * h2;
    w.m(oe + 1) = m.gOb * g.ia * h2;
    w.m(oe + 2) = m.g43g * g.ia2 * h2;
    w.m(oe + 3) = m.g43N * g.ia2 * h2;
    w.m(oe + 4) = (1.0 + g.wQ) * rQ * h2;
    w.m(oe + 5) = 0.0;
    w.m(o1 + 0) = -m.gOc;
    w.m(o1 + 1) = -m.gOb;
    w.m(o1 + 2) = -2.0 * m.grhog * g.ia;
    w.m(o1 + 3) = -2.0 * m.grN * g.ia;
    w.m(o1 + 4) = -rQ * a * (1.0 + 3.0 * m.cs2Q);
    w.m(o1 + 5) = -9.0 * (m.cs2Q - g.ca2) * g.aH * (1.0 + g.wQ) * rQ * a * m.ik2;
  }
  for (int i = gp.lane; i < nq; i += G) {
    const double v = w.m(M_Q + Q_V * nq + i);
    const double iv = rcp(v);
    const double wq = LDG(c.w + i);
    w.m(gl_off(nq, GL_H) + i) = m.grM * wq * iv * g.ia2 * iaH;
    w.m(gl_off(nq, GL_E) + i) = m.grMk * wq * g.ia2 * h2;
    w.m(gl_off(nq, GL_R1) + i) = -m.grM * wq * (iv + v) * g.ia;
  }
  for (int j = gp.lane; j < n; j += G) { w.v(V_ZH, j) = 0.0; w.v(V_ZE, j) = 0.0; }
  factor_M<G>(gp, m, D, T, w, d, tau, g);   // syncs
  // u_h into ZH, u_e into ZE (sparse), then M^{-1}
  if (gp.lead()) {
    w.v(V_ZH, 3) = -0.5; w.v(V_ZH, 5) = -0.5; w.v(V_ZH, 7) = -2.0 / 3.0; w.v(V_ZH, 9) = 4.0 / 15.0;
    w.v(V_ZH, ir) = -2.0 / 3.0; w.v(V_ZH, ir + 2) = 4.0 / 15.0; w.v(V_ZH, n - 2) = -0.5 * (1.0 + g.wQ);
    w.v(V_ZE, 2) = 1.0; w.v(V_ZE, 9) = 1.6; w.v(V_ZE, ir + 2) = 1.6;
  }
  for (int i = gp.lane; i < nq; i += G) {
    const double dlf = w.m(M_Q + Q_DLF * nq + i);
    w.v(V_ZH, iq0 + i) = dlf / 6.0;
    w.v(V_ZH, iq0 + 2 * nq + i) = -dlf / 15.0;
    w.v(V_ZE, iq0 + 2 * nq + i) = -0.4 * dlf;
  }
  gp.sync();
  solve_M<G>(gp, m, D, w, d, g.aH, V_ZH);
  solve_M<G>(gp, m, D, w, d, g.aH, V_ZE);
  double hh, eh, he, ee;
  functionals<G>(gp, D, w, V_ZH, hh, eh);
  functionals<G>(gp, D, w, V_ZE, he, ee);
  // C = I - G^T Z = [[1 - hh, -he], [-eh, 1 - ee]]
  if (gp.lead()) {
    const double c00 = 1.0 - hh, c01 = -he, c10 = -eh, c11 = 1.0 - ee;
    const double idet = 1.0 / (c00 * c11 - c01 * c10);
    w.m(M_CINV + 0) = c11 * idet; w.m(M_CINV + 1) = -c01 * idet;
    w.m(M_CINV + 2) = -c10 * idet; w.m(M_CINV + 3) = c00 * idet;
  }
  gp.sync();
}

// x = W^{-1} b in place on vector vb.  Expects vb synced; ends synced.
template <int G>
HD void solve_W(const Grp<G>& gp, const ModeConst& m, const Dims& D, const WS<G>& w, double aH, int vb) {
  const int n = D.n, nq = D.nq;
  const double d = w.m(M_SCAL + S_D);
  const double x0 = w.v(vb, 0) * w.m(M_SCAL + S_W00I);
  gp.sync();
  for (int j = 1 + gp.lane; j < n; j += G) w.v(vb, j) += w.v(V_JC0, j) * x0;
  if (gp.lead()) w.v(vb, 0) = x0;
  gp.sync();
  solve_M<G>(gp, m, D, w, d, aH, vb);
  double sh, se;
  functionals<G>(gp, D, w, vb, sh, se);
  const double th = w.m(M_CINV + 0) * sh + w.m(M_CINV + 1) * se;
  const double te = w.m(M_CINV + 2) * sh + w.m(M_CINV + 3) * se;
  gp.sync();
  for (int j = 2 + gp.lane; j < n; j += G) w.v(vb, j) += w.v(V_ZH, j) * th + w.v(V_ZE, j) * te;
  gp.sync();
  double s1 = 0.0;
  const int o1 = gl_off(nq, GL_R1);
  for (int t = gp.lane; t < nq + 6; t += G) s1 += w.m(o1 + t) * w.v(vb, gather_index(D, GL_R1, t));
  s1 = gp.sum(s1);
  if (gp.lead()) w.v(vb, 1) = (w.v(vb, 1) + s1) * w.m(M_SCAL + S_ID);
  gp.sync();
}

// ------------------------------------------------------------------ dense reference-method path
// W = d I - J assembled densely from the same pieces and factored by LU with
// partial pivoting, like the reference's lu_factor / lu_solve
// (ode_integrators_stiff.py:774-776, 783).  Kept for validation and as the
// plain method; O(n^3) per step.  Rows are spread over the lanes.
template <int G, class F>
HD void visit_u(const Dims& D, const WS<G>& w, double wQ, F f) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, ir = D.ir;
  f(3, -0.5, 0.0); f(5, -0.5, 0.0); f(7, -2.0 / 3.0, 0.0); f(9, 4.0 / 15.0, 1.6);
  f(ir, -2.0 / 3.0, 0.0); f(ir + 2, 4.0 / 15.0, 1.6); f(n - 2, -0.5 * (1.0 + wQ), 0.0); f(2, 0.0, 1.0);
  for (int i = 0; i < nq; ++i) {
    const double dlf = w.m(M_Q + Q_DLF * nq + i);
    f(iq0 + i, dlf / 6.0, 0.0);
    f(iq0 + 2 * nq + i, -dlf / 15.0, -0.4 * dlf);
  }
}

template <int G, class F>
HD void visit_g(const Dims& D, const WS<G>& w, F f) {
  const int nq = D.nq;
  for (int t = 0; t < nq + 6; ++t) {
    f(gather_index(D, GL_H, t), w.m(gl_off(nq, GL_H) + t), 0.0);
    f(gather_index(D, GL_E, t), 0.0, w.m(gl_off(nq, GL_E) + t));
  }
}

// Assemble and factor the dense W after factor_W (which leaves the chain
// coefficients and functional/row-1 coefficients in place).
template <int G>
HD void dense_factor(const Grp<G>& gp, const ModeConst& m, const Dims& D, const Tab& T, const WS<G>& w, double d, double tau,
                     const Bg<double>& g) {
  const int n = D.n, nq = D.nq, igp = D.igp;
  auto A = [&](int i, int j) -> double& { return w.e(i * n + j); };
  const double itau = 1.0 / tau, op = g.opac;
  for (int i = gp.lane; i < n; i += G) {
    for (int j = 0; j < n; ++j) A(i, j) = (i == j) ? d : 0.0;
    A(i, 0) -= w.v(V_JC0, i);
  }
  gp.sync();
  for (int ch = gp.lane; ch < nq + 3; ch += G) {
    const Chain cc = chain_of<G>(m, D, w, ch);
    const double damp = cc.attach >= 0 ? op : 0.0;
    for (int j = 0; j < cc.cnt; ++j) {
      const int i = cc.start + j * cc.stride;
      double lo, up;
      chain_entry(m, T, ch, cc, cc.l0 + j, lo, up);
      if (j > 0 || cc.attach >= 0) A(i, i - cc.stride) = lo;
      if (j < cc.cnt - 1) A(i, i + cc.stride) = up;
      A(i, i) = d + damp + (j == cc.cnt - 1 ? (cc.lmax + 1.0) * itau : 0.0);
    }
  }
  gp.sync();
  if (gp.lead()) {
    A(3, 4) = 1.0; A(4, 4) = d + g.aH;
    A(9, 10) = 0.6 * m.k;
    A(igp + 2, igp + 3) = 0.6 * m.k;
    double core[64], de[4];
    core_entries(m, T, g, d, core, de);
    const int cidx[8] = {5, 6, 7, 8, 9, igp, igp + 1, igp + 2};
    for (int r = 0; r < 8; ++r) for (int cc = 0; cc < 8; ++cc) A(cidx[r], cidx[cc]) = core[r * 8 + cc];
    A(n - 2, n - 2) = de[0]; A(n - 2, n - 1) = de[1]; A(n - 1, n - 2) = de[2]; A(n - 1, n - 1) = de[3];
    visit_u<G>(D, w, g.wQ, [&](int i, double uh, double ue) {
      visit_g<G>(D, w, [&](int j, double gh, double ge) { A(i, j) -= uh * gh + ue * ge; });
    });
    for (int j = 1; j < n; ++j) A(1, j) = (j == 1) ? d : 0.0;
    A(1, 0) = -w.v(V_JC0, 1);
    for (int t = 0; t < nq + 6; ++t) A(1, gather_index(D, GL_R1, t)) = -w.m(gl_off(nq, GL_R1) + t);
  }
  gp.sync();
  // LU with partial pivoting (first maximal |pivot|), rows over lanes
  const int P0 = n * n;
  for (int kk = 0; kk < n; ++kk) {
    double best = -1.0;
    int bi = kk;
    for (int i = kk + gp.lane; i < n; i += G) {
      const double v = fabs(A(i, kk));
      if (v > best) { best = v; bi = i; }
    }
    gp.argmax(best, bi);
    if (gp.lead()) w.e(P0 + kk) = (double)bi;
    if (bi != kk)
      for (int j = gp.lane; j < n; j += G) { const double t = A(kk, j); A(kk, j) = A(bi, j); A(bi, j) = t; }
    gp.sync();
    const double inv = 1.0 / A(kk, kk);
    for (int i = kk + 1 + gp.lane; i < n; i += G) {
      const double l = A(i, kk) * inv;
      A(i, kk) = l;
      if (l != 0.0) for (int j = kk + 1; j < n; ++j) A(i, j) -= l * A(kk, j);
    }
    gp.sync();
  }
}

template <int G>
HD void dense_solve(const Grp<G>& gp, const Dims& D, const WS<G>& w, int vb) {
  const int n = D.n;
  const int P0 = n * n;
  auto A = [&](int i, int j) -> double { return w.e(i * n + j); };
  if (gp.lead())
    for (int kk = 0; kk < n; ++kk) {
      const int p = (int)w.e(P0 + kk);
      if (p != kk) { const double t = w.v(vb, kk); w.v(vb, kk) = w.v(vb, p); w.v(vb, p) = t; }
    }
  gp.sync();
  for (int i = 1; i < n; ++i) {
    double s = 0.0;
    for (int j = gp.lane; j < i; j += G) s += A(i, j) * w.v(vb, j);
    s = gp.sum(s);
    if (gp.lead()) w.v(vb, i) -= s;
    gp.sync();
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = 0.0;
    for (int j = i + 1 + gp.lane; j < n; j += G) s += A(i, j) * w.v(vb, j);
    s = gp.sum(s);
    if (gp.lead()) w.v(vb, i) = (w.v(vb, i) - s) / A(i, i);
    gp.sync();
  }
}

// ------------------------------------------------------------------ controller + step
struct Ctl {
  double rtol, atol, b1, b2, b3, safety, fmin, fmax;
  int max_steps, hist_on_reject, dense, return_full, nout;
  int record;   // store tau_start and every accepted step's end time
  int replay;   // take the stored step times instead of controlling the step
  int step_ts;  // clip steps to land on every output time (diffrax PIDController(step_ts=ts))
};

// first output time strictly after t (or +inf) and its index (or -1)
HD double next_output_after(const double* tau_out, int nout, double t, int* which = nullptr) {
  double best = 1e300;
  int bi = -1;
  for (int o = 0; o < nout; ++o) {
    const double to = LDG(tau_out + o);
    if (to > t && to < best) { best = to; bi = o; }
  }
  if (which) *which = bi;
  return best;
}

// Integration state; every lane of a group holds an identical copy.
// rec: [tau_start, t_1, ..., t_nrec] of the nominal run (record / replay);
// a step that was clipped to output time o is stored as -(o + 1).
struct Run {
  double t0, t1, T1, lprev, lprev_prev;   // logs of the previous two inverse errors
  int vy, vu, steps, acc, rej, status;   // vector ids of y0 and of the stage state / y1
  double* rec;
  int rec_cap, nrec;
  double scale;   // replay: tau_start / nominal tau_start
  int t1_out;     // index of the output time the current step is clipped to, or -1
  // record with checkpoints (the adjoint's forward states): ck[slot n + j]
  // holds y after accepted step slot * ck_stride; when the ck_cap slots are
  // full, every other one is dropped and the stride doubles, so a run keeps
  // between ck_cap / 2 and ck_cap evenly spaced states.  ck = null: none.
  double* ck = nullptr;
  int ck_cap = 0, ck_stride = 1;
};

// Store the state of vector vec as the checkpoint after accepted step j
// (j = 0: the initial state), thinning as described at Run::ck.
template <int G>
HD void checkpoint_store(const Grp<G>& gp, const WS<G>& w, int n, Run& r, int vec, int j) {
  if (!r.ck || j % r.ck_stride) return;
  int slot = j / r.ck_stride;
  if (slot >= r.ck_cap) {
    const int half = r.ck_cap / 2;
    for (int i = 1; i < half; ++i)
      for (int e = gp.lane; e < n; e += G) r.ck[(long)i * n + e] = r.ck[(long)(2 * i) * n + e];
    gp.sync();
    r.ck_stride *= 2;
    if (j % r.ck_stride) return;
    slot = j / r.ck_stride;
  }
  for (int e = gp.lane; e < n; e += G) r.ck[(long)slot * n + e] = w.v(vec, e);
  gp.sync();
}

// replay: end time of recorded step j (1-based) for this table set
HD double replay_time(const Run& r, const double* tau_out, int j) {
  const double v = LDG(r.rec + j);
  return v < 0.0 ? LDG(tau_out + (int)(-v) - 1) : v * r.scale;
}

// start time of one mode: 0.99 min(min tau_out, determine_starting_time)
// (perturbations.py:742-743)
HD double mode_start(const Cosmo& c, const ModeConst& m, const Ctl& ctl, const double* tau_out) {
  double tmin = LDG(tau_out);
  for (int o = 1; o < ctl.nout; ++o) { const double t = LDG(tau_out + o); tmin = t < tmin ? t : tmin; }
  const double ts = start_time(c, m);
  return 0.99 * (tmin < ts ? tmin : ts);
}

// start a mode: start time, ICs, first step size (perturbations.py:742-756);
// t0_forced > 0 starts it at that time instead (a group's common start)
template <int G>
HD void mode_begin(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Ctl& ctl, const WS<G>& w,
                   const double* tau_out, Run& r, double t0_forced = -1.0) {
  double tmax = LDG(tau_out);
  for (int o = 1; o < ctl.nout; ++o) { const double t = LDG(tau_out + o); tmax = t > tmax ? t : tmax; }
  // start time of this table set.  In a replay the recorded step times are
  // scaled by tau_start / nominal tau_start: with the step-size factors
  // frozen every step length is proportional to dt0 = tau_start / 4, which
  // is how jax.jacfwd sees the diffrax step sequence.
  const double t0 = t0_forced > 0.0 ? t0_forced : mode_start(c, m, ctl, tau_out);
  initial_conditions<G>(gp, c, m, D, t0, w, V_Y);
  r.t0 = t0; r.T1 = tmax;
  r.t1_out = -1;
  if (ctl.replay) {
    r.scale = t0 / LDG(r.rec);
    const double tn = r.nrec > 1 ? replay_time(r, tau_out, 1) : tmax;
    r.t1 = (r.nrec <= 1 || tn >= tmax) ? tmax : tn;
  } else {
    r.scale = 1.0;
    const double dt0 = (t0 / 4.0 < 0.5 * (tmax - t0)) ? t0 / 4.0 : 0.5 * (tmax - t0);
    r.t1 = t0 + dt0 < tmax ? t0 + dt0 : tmax;
    if (ctl.step_ts) {
      int o;
      const double to = next_output_after(tau_out, ctl.nout, t0, &o);
      if (r.t1 >= to) { r.t1 = to; r.t1_out = o; }
    }
    if (ctl.record && gp.lead()) r.rec[0] = t0;
  }
  r.lprev = 0.0; r.lprev_prev = 0.0;
  r.vy = V_Y; r.vu = V_U; r.steps = 0; r.acc = 0; r.rej = 0; r.status = ST_OK;
  if (ctl.record && r.ck) { r.ck_stride = 1; checkpoint_store<G>(gp, w, D.n, r, V_Y, 0); }
}

// Stage S >= 1 before its RHS: u = y0 + sum_q a_Sq k_q (S <= 5) or
// u += k_{S-1} (S >= 6), and k_S = sum_q (C_Sq / dt) k_q, to which the RHS
// then adds f(u).  One pass reads every earlier stage vector once.
template <int G, int S>
HD void stage_prep(const Grp<G>& gp, const Rodas& R, const WS<G>& w, int n, int vy, int vu, double idt) {
  double a[S], cc[S];
#pragma unroll
  for (int q = 0; q < S; ++q) { a[q] = R.a[S][q]; cc[q] = R.C[S][q] * idt; }
#pragma unroll 2
  for (int j = gp.lane; j < n; j += G) {
    double kq[S];
#pragma unroll
    for (int q = 0; q < S; ++q) kq[q] = w.v(V_K0 + q, j);
    double p = cc[0] * kq[0];
#pragma unroll
    for (int q = 1; q < S; ++q) p += cc[q] * kq[q];
    double u;
    if constexpr (S <= 5) {
      u = w.v(vy, j);
#pragma unroll
      for (int q = 0; q < S; ++q) u += a[q] * kq[q];
    } else {
      u = w.v(vu, j) + kq[S - 1];
    }
    w.v(vu, j) = u;
    w.v(V_K0 + S, j) = p;
  }
}

// One attempted Rodas5 step (ode_integrators_stiff.py:718-834): the eight
// stages from (r.t0, y0) over r.t1 - r.t0, y1 = u + k8 into the stage state
// vector.  Returns the sum of squares of the six scaled error entries of the
// PID norm (perturbations.py:701-705, 759-760); bad = y1 not finite.
template <int G>
HD double step_attempt(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T,
                       const Rodas& R, const Ctl& ctl, const WS<G>& w, const Run& r, bool& bad_out,
                       Bg<double>* g0 = nullptr) {
  const int n = D.n, nq = D.nq, iq0 = D.iq0, igp = D.igp, ir = D.ir, lg = D.lg, lgp = D.lgp, lr = D.lr, lnu = D.lnu;
  const double t0 = r.t0, dt = r.t1 - r.t0;
  const int vy = r.vy, vu = r.vu;
  // f(t0, y0) into k1 and d f / d a in one forward-mode pass
  Bg<double> g;
  rhs<Dual, G>(gp, c, m, D, T, t0, w, vy, V_K0, V_JC0, &g);
  if (g0) *g0 = g;
  const double d = rcp(dt * R.gamma);
  factor_W<G>(gp, c, m, D, T, w, d, t0, g);
  if (ctl.dense) dense_factor<G>(gp, m, D, T, w, d, t0, g);
  // d f / d tau: only the (l+1)/tau truncation terms
  const double it2 = rcp(t0 * t0);
  const double dTT = (lg + 1.0) * it2 * w.v(vy, 7 + lg);
  const double dTP = (lgp + 1.0) * it2 * w.v(vy, igp + lgp);
  const double dTR = (lr + 1.0) * it2 * w.v(vy, ir + lr);
  for (int i = gp.lane; i < nq; i += G) w.m(M_Q + Q_DT * nq + i) = (lnu + 1.0) * it2 * w.v(vy, iq0 + lnu * nq + i);
  const double idt = rcp(dt);
  for (int s = 0; s < 8; ++s) {
    const int vk = V_K0 + s;
    if (s > 0) {
      switch (s) {
        case 1: stage_prep<G, 1>(gp, R, w, n, vy, vu, idt); break;
        case 2: stage_prep<G, 2>(gp, R, w, n, vy, vu, idt); break;
        case 3: stage_prep<G, 3>(gp, R, w, n, vy, vu, idt); break;
        case 4: stage_prep<G, 4>(gp, R, w, n, vy, vu, idt); break;
        case 5: stage_prep<G, 5>(gp, R, w, n, vy, vu, idt); break;
        case 6: stage_prep<G, 6>(gp, R, w, n, vy, vu, idt); break;
        default: stage_prep<G, 7>(gp, R, w, n, vy, vu, idt); break;
      }
      gp.sync();
      rhs<double, G, true>(gp, c, m, D, T, t0 + R.c[s] * dt, w, vu, vk, -1);   // ends synced
    }
    if (s <= 4) {
      const double dd = dt * R.d[s];
      if (gp.lead()) {
        w.v(vk, 7 + lg) += dd * dTT;
        w.v(vk, igp + lgp) += dd * dTP;
        w.v(vk, ir + lr) += dd * dTR;
      }
      for (int i = gp.lane; i < nq; i += G) w.v(vk, iq0 + lnu * nq + i) += dd * w.m(M_Q + Q_DT * nq + i);
      gp.sync();
    }
    if (ctl.dense) dense_solve<G>(gp, D, w, vk);
    else solve_W<G>(gp, m, D, w, g.aH, vk);
  }
  // y1 = u + k8 in place of u; error estimate k8
  const int vy1 = vu, vk8 = V_K0 + 7;
  bool bad = false;
  for (int j = gp.lane; j < n; j += G) {
    const double v = w.v(vu, j) + w.v(vk8, j);
    w.v(vy1, j) = v;
    bad = bad || !isfinite_(v);
  }
  bad = gp.any(bad);
  gp.sync();
  const int eidx[6] = {0, 2, 3, 5, 6, 7};
  const double ew[6] = {1.0, m.k2, 1.0, 1.0, m.ik2, 1.0};
  double ss = 0.0;
  for (int q = 0; q < 6; ++q) {
    const int j = eidx[q];
    const double y0 = fabs(w.v(vy, j));
    const double y1 = bad ? y0 : fabs(w.v(vy1, j));
    const double sc = w.v(vk8, j) * rcp(ctl.atol + (y0 > y1 ? y0 : y1) * ctl.rtol) * ew[q];
    ss += sc * sc;
  }
  bad_out = bad;
  return ss;
}

// The PID decision on an attempted step with error norm err (computed over
// this mode, or over a group of modes sharing one step sequence), SaveAt
// outputs inside an accepted step, and the next step.  Returns true while
// the mode still needs steps.
template <int G>
HD bool step_decide(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Ctl& ctl,
                    const WS<G>& w, const double* tau_out, double* yout, long ostride, Run& r, double err, bool bad) {
  const int n = D.n;
  const double dt = r.t1 - r.t0;
  const int vy = r.vy, vu = r.vu, vy1 = vu;
  ++r.steps;
  if (!isfinite_(err) || (ctl.replay && bad)) { r.status = ST_NONFINITE; return false; }
  const bool keep = ctl.replay ? true : err < 1.0;
  // PID factor safety inv^b1 prev^b2 prevprev^b3, as one exp of a sum of
  // logs (the logs of the previous inverse errors are kept)
  const double linv = -log(err);
  double lf = 0.0;
  if (ctl.b1 != 0.0) lf += ctl.b1 * linv;
  if (ctl.b2 != 0.0) lf += ctl.b2 * r.lprev;
  if (ctl.b3 != 0.0) lf += ctl.b3 * r.lprev_prev;
  double factor = ctl.safety * exp(lf);
  const double fmin = keep ? 1.0 : ctl.fmin;
  factor = factor < fmin ? fmin : factor;
  factor = factor > ctl.fmax ? ctl.fmax : factor;
  const double dtn = dt * factor;
  const double linv_kept = isfinite_(linv) ? linv : 0.0;
  if (keep) {
    ++r.acc;
    // SaveAt(ts) with LocalLinearInterpolation between (t0, y0) and (t1, y1)
    for (int o = 0; o < ctl.nout; ++o) {
      const double tt = LDG(tau_out + o);
      if (tt > r.t0 && tt <= r.t1) {
        const double cf = (tt - r.t0) / (r.t1 - r.t0);
        double* dst = yout + (long)o * (ctl.return_full ? n : 20) * ostride;
        if (ctl.return_full) {
          for (int j = gp.lane; j < n; j += G) { const double y0 = w.v(vy, j); dst[(long)j * ostride] = y0 + cf * (w.v(vy1, j) - y0); }
        } else {
          // interpolated state in k1 (free once the step is complete)
          for (int j = gp.lane; j < n; j += G) { const double y0 = w.v(vy, j); w.v(V_K0, j) = y0 + cf * (w.v(vy1, j) - y0); }
          gp.sync();
          if (gp.lead()) outputs<G>(c, m, D, w, V_K0, dst, ostride);
        }
        gp.sync();
      }
    }
    r.vy = vy1; r.vu = vy;
    r.t0 = r.t1;
    r.lprev_prev = r.lprev;
    r.lprev = linv_kept;
    if (ctl.record && gp.lead() && r.acc < r.rec_cap) r.rec[r.acc] = r.t1_out >= 0 ? -(r.t1_out + 1.0) : r.t1;
    if (ctl.record && r.ck) checkpoint_store<G>(gp, w, n, r, r.vy, r.acc);
    if (ctl.replay) {
      // next recorded end time; the run ends at this table set's own final
      // output time (the recorded one is the nominal cosmology's)
      if (r.t0 >= r.T1) return false;
      double tn = r.acc + 1 < r.nrec ? replay_time(r, tau_out, r.acc + 1) : r.T1;
      if (r.acc + 1 >= r.nrec || tn >= r.T1) tn = r.T1;
      r.t1 = tn;
      return true;
    }
  } else {
    ++r.rej;
    if (ctl.hist_on_reject) { r.lprev_prev = r.lprev; r.lprev = linv_kept; }
  }
  double tn = r.t0 + dtn;
  r.t1_out = -1;
  if (ctl.step_ts) {
    int o;
    const double to = next_output_after(tau_out, ctl.nout, r.t0, &o);
    if (tn >= to) { tn = to; r.t1_out = o; }
  }
  if (tn > r.T1 - 1e-10) tn = r.T1;
  if (!(tn > r.t0) && r.t0 < r.T1) { r.status = ST_DT_UNDERFLOW; return false; }
  r.t1 = tn;
  return r.t0 < r.T1;
}

// One attempted step of one mode plus its PID decision.  Returns true while
// the mode still needs steps.
template <int G>
HD bool mode_step(const Grp<G>& gp, const Cosmo& c, const ModeConst& m, const Dims& D, const Tab& T, const Rodas& R,
                  const Ctl& ctl, const WS<G>& w, const double* tau_out, double* yout, long ostride, Run& r) {
  if (!(r.t0 < r.T1)) return false;
  if (r.steps >= ctl.max_steps) { r.status = ST_MAX_STEPS; return false; }
  bool bad;
  const double ss = step_attempt<G>(gp, c, m, D, T, R, ctl, w, r, bad);
  const double err = ctl.replay ? 0.0 : sqrt(ss / 6.0);
  return step_decide<G>(gp, c, m, D, ctl, w, tau_out, yout, ostride, r, err, bad);
}

// One mode of a group as group_solve sees it.
template <int G>
struct ModeCtx {
  Cosmo c;
  ModeConst m;
  WS<G> w;
  const double* tau_out;
  double* yout;
};

// B <= 32 modes sharing one step sequence: the reference's batched variant
// (evolve_modes_batched, perturbations.py:835-922, with Rodas5Batched,
// ode_integrators_stiff.py:846-1010).  The modes start together at the
// smallest of their start times (determine_start_times_per_batch,
// perturbations.py:786-803), take the same steps, and the PID controller
// sees one error norm: the RMS over the six filtered entries of every mode
// (rms_norm_filtered_batched, perturbations.py:690-694).  ctx(b) returns
// mode b's ModeCtx; its outputs follow the same SaveAt rule as one mode's.
// r ends with the group's status and step counts.
template <int G, class CtxFn>
HD void group_solve(const Grp<G>& gp, const Dims& D, const Tab& T, const Rodas& R, const Ctl& ctl, int B, CtxFn ctx,
                    long ostride, Run& r) {
  double t0 = 1e300;
  for (int b = 0; b < B; ++b) {
    const ModeCtx<G> x = ctx(b);
    const double ts = mode_start(x.c, x.m, ctl, x.tau_out);
    t0 = ts < t0 ? ts : t0;
  }
  for (int b = 0; b < B; ++b) {
    const ModeCtx<G> x = ctx(b);
    mode_begin<G>(gp, x.c, x.m, D, ctl, x.w, x.tau_out, r, t0);
  }
  for (;;) {
    if (!(r.t0 < r.T1)) break;
    if (r.steps >= ctl.max_steps) { r.status = ST_MAX_STEPS; break; }
    double ss = 0.0;
    unsigned badm = 0u;
    for (int b = 0; b < B; ++b) {
      const ModeCtx<G> x = ctx(b);
      bool bad;
      ss += step_attempt<G>(gp, x.c, x.m, D, T, R, ctl, x.w, r, bad);
      if (bad) badm |= 1u << b;
    }
    const double err = sqrt(ss / (6.0 * B));
    const Run r0 = r;
    bool more = false;
    for (int b = 0; b < B; ++b) {
      const ModeCtx<G> x = ctx(b);
      Run rb = r0;
      more = step_decide<G>(gp, x.c, x.m, D, ctl, x.w, x.tau_out, x.yout, ostride, rb, err, ((badm >> b) & 1u) != 0u);
      if (b == B - 1) r = rb;
    }
    if (!more) break;
  }
}

HD void fill_tables(Tab& T) {
  for (int l = 0; l < LMAX_TABLE + 2; ++l) { T.lo[l] = (double)l / (2.0 * l + 1.0); T.up[l] = (l + 1.0) / (2.0 * l + 1.0); }
}

HD void fill_rodas(Rodas& R) {
  for (int i = 0; i < 8; ++i) for (int j = 0; j < 8; ++j) { R.a[i][j] = 0.0; R.C[i][j] = 0.0; }
  R.gamma = 0.19;
  R.a[1][0] = 2.0;
  R.a[2][0] = 3.040894194418781; R.a[2][1] = 1.041747909077569;
  R.a[3][0] = 2.576417536461461; R.a[3][1] = 1.622083060776640; R.a[3][2] = -0.9089668560264532;
  R.a[4][0] = 2.760842080225597; R.a[4][1] = 1.446624659844071; R.a[4][2] = -0.3036980084553738; R.a[4][3] = 0.2877498600325443;
  R.a[5][0] = -14.09640773051259; R.a[5][1] = 6.925207756232704; R.a[5][2] = -41.47510893210728;
  R.a[5][3] = 2.343771018586405; R.a[5][4] = 24.13215229196062;
  R.C[1][0] = -10.31323885133993;
  R.C[2][0] = -21.04823117650003; R.C[2][1] = -7.234992135176716;
  R.C[3][0] = 32.22751541853323; R.C[3][1] = -4.943732386540191; R.C[3][2] = 19.44922031041879;
  R.C[4][0] = -20.69865579590063; R.C[4][1] = -8.816374604402768; R.C[4][2] = 1.260436877740897; R.C[4][3] = -0.7495647613787146;
  R.C[5][0] = -46.22004352711257; R.C[5][1] = -17.49534862857472; R.C[5][2] = -289.6389582892057;
  R.C[5][3] = 93.60855400400906; R.C[5][4] = 318.3822534212147;
  R.C[6][0] = 34.20013733472935; R.C[6][1] = -14.15535402717690; R.C[6][2] = 57.82335640988400;
  R.C[6][3] = 25.83362985412365; R.C[6][4] = 1.408950972071624; R.C[6][5] = -6.551835421242162;
  R.C[7][0] = 42.57076742291101; R.C[7][1] = -13.80770672017997; R.C[7][2] = 93.98938432427124;
  R.C[7][3] = 18.77919633714503; R.C[7][4] = -31.58359187223370; R.C[7][5] = -6.685968952921985; R.C[7][6] = -5.810979938412932;
  const double c_[8] = {0.0, 0.38, 0.3878509998321533, 0.4839718937873840, 0.4570477008819580, 1.0, 1.0, 1.0};
  const double d_[8] = {0.19, -0.1823079225333714636, -0.319231832186874912, 0.3449828624725343, -0.377417564392089818, 0, 0, 0};
  for (int i = 0; i < 8; ++i) { R.c[i] = c_[i]; R.d[i] = d_[i]; }
}

}  // namespace deb
