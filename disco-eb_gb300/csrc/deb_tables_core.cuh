// deb_tables_core.cuh -- the table producer's per-set work, written once as
// host/device code: tables_kernel (deb_tables.cu) runs it with the 32 lanes
// of a warp, the test suite compiles it for the host (one lane) to check the
// C++ restatement against the host producer without a GPU.
//
// Reference correspondence (file:line of DISCO-EB):
//   densities, neutrino tables, closure   src/discoeb/background.py:140-188, 47-68
//   Friedmann d tau / d a, a'/a            src/discoeb/background.py:71-122
//   evolve_background (RECFAST branch)     src/discoeb/background.py:191-305
//   ionisation RHS                         src/discoeb/thermodynamics_recfast.py:124-281
//   GRK4A step (all stages at t0)          src/discoeb/ode_integrators_stiff.py:117-223
//   adaptive solve per interval            src/discoeb/thermodynamics_recfast.py:283-300
//   HeII Saha fraction                     src/discoeb/thermodynamics_recfast.py:302-321
//   thermal history loop, 4 cases          src/discoeb/thermodynamics_recfast.py:362-452
//   x_e, c_s^2, tau by Romberg             src/discoeb/thermodynamics_recfast.py:455-501
//   natural cubic spline                   src/discoeb/spline_interpolation.py:47-153
// The physical constants and fitting parameters of RECFAST are the published
// model; the host passes them in (deb_tables_const order) so that host and
// device tables are built from identical numbers.
#pragma once

#include <cmath>

#include "discoeb_gb300.h"

#ifdef __CUDACC__
#define HD __host__ __device__ __forceinline__
#else
#define HD inline
#endif

namespace debt {

#ifndef __CUDACC__
using std::exp; using std::log; using std::pow; using std::sqrt; using std::fabs; using std::fmin; using std::fmax;
using std::isnan;
#endif

HD void lane_sync(int G) {
#ifdef __CUDA_ARCH__
  if (G > 1) __syncwarp();
#else
  (void)G;
#endif
}


// constants vector (order fixed by DEB_TC_* in the header)
struct TC {
  const double* c;
  HD double operator[](int i) const { return c[i]; }
};

// value + gradient with respect to the three ionisation variables (the 3x3
// Jacobian in one pass, exact like the reference's jacfwd)
struct D3 {
  double v, d[3];
  HD D3() : v(0) { d[0] = d[1] = d[2] = 0; }
  HD D3(double x) : v(x) { d[0] = d[1] = d[2] = 0; }
};
HD D3 operator+(D3 a, D3 b) { D3 r(a.v + b.v); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
HD D3 operator-(D3 a, D3 b) { D3 r(a.v - b.v); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
HD D3 operator-(D3 a) { D3 r(-a.v); for (int i = 0; i < 3; ++i) r.d[i] = -a.d[i]; return r; }
HD D3 operator*(D3 a, D3 b) { D3 r(a.v * b.v); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
HD D3 operator/(D3 a, D3 b) {
  const double q = a.v / b.v;
  D3 r(q);
  for (int i = 0; i < 3; ++i) r.d[i] = (a.d[i] - q * b.d[i]) / b.v;
  return r;
}
HD D3 operator+(D3 a, double b) { a.v += b; return a; }
HD D3 operator+(double a, D3 b) { b.v += a; return b; }
HD D3 operator-(D3 a, double b) { a.v -= b; return a; }
HD D3 operator-(double a, D3 b) { return D3(a) - b; }
HD D3 operator*(D3 a, double b) { D3 r(a.v * b); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] * b; return r; }
HD D3 operator*(double a, D3 b) { return b * a; }
HD D3 operator/(D3 a, double b) { D3 r(a.v / b); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] / b; return r; }
HD D3 operator/(double a, D3 b) { return D3(a) / b; }
HD D3 dexp(D3 a) { const double e = exp(a.v); D3 r(e); for (int i = 0; i < 3; ++i) r.d[i] = e * a.d[i]; return r; }
HD D3 dsqrt(D3 a) { const double s = sqrt(a.v); D3 r(s); for (int i = 0; i < 3; ++i) r.d[i] = 0.5 * a.d[i] / s; return r; }
HD D3 dpow(D3 a, double p) {
  const double v = pow(a.v, p), dv = p * pow(a.v, p - 1.0);
  D3 r(v);
  for (int i = 0; i < 3; ++i) r.d[i] = dv * a.d[i];
  return r;
}
HD double dexp(double a) { return exp(a); }
HD double dsqrt(double a) { return sqrt(a); }
HD double dpow(double a, double p) { return pow(a, p); }
HD double val(double a) { return a; }
HD double val(const D3& a) { return a.v; }

// ---------------------------------------------------------------- splines
// second derivatives with natural ends, Thomas elimination in the order of
// spline_interpolation.py:50-85; cp, dp: n doubles of scratch each
HD void natural_S(const double* x, const double* y, double* S, int n, double* cp, double* dp) {
  for (int i = 0; i < n; ++i) S[i] = 0.0;
  const int m = n - 2;
  if (m <= 0) return;
  // rows i = 0 .. m-1 stand for knots 1 .. n-2
  auto hh = [&](int j) { return x[j + 1] - x[j]; };
  {
    const double h0 = hh(0), h1 = hh(1);
    const double di = 2.0 * (h0 + h1), up = h1;
    const double rhs = 6.0 * ((y[2] - y[1]) / h1 - (y[1] - y[0]) / h0);
    cp[0] = up / di;
    dp[0] = rhs / di;
  }
  for (int i = 1; i < m; ++i) {
    const double hl = hh(i), hr = hh(i + 1);
    const double lo = hl, di = 2.0 * (hl + hr), up = hr;
    const double rhs = 6.0 * ((y[i + 2] - y[i + 1]) / hr - (y[i + 1] - y[i]) / hl);
    const double den = di - lo * cp[i - 1];
    cp[i] = i < m - 1 ? up / den : 0.0;
    dp[i] = (rhs - lo * dp[i - 1]) / den;
  }
  S[m] = dp[m - 1];
  for (int i = m - 2; i >= 0; --i) S[i + 1] = dp[i] - cp[i] * S[i + 2];
}

// A/B form evaluation with a left searchsorted (spline_interpolation.py:130-153)
HD double spl_ab(const double* x, const double* y, const double* S, int n, double xv) {
  int lo = 0, hi = n;   // first index with x[i] >= xv
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] < xv) lo = mid + 1; else hi = mid;
  }
  int i = lo - 1;
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  const double h = x[i + 1] - x[i];
  const double t = (xv - x[i]) / h;
  const double A = 1.0 - t, B = t;
  return A * y[i] + B * y[i + 1] + ((A * A * A - A) * S[i] + (B * B * B - B) * S[i + 1]) * (h * h) / 6.0;
}

// ---------------------------------------------------------------- background
struct Bk {
  double Om, Ob, H0, Tcmb, YHe, Neff, Nmnu, w0, wa, Ok;
  double grhom, grhog, grhor, ODE, fHe;
  const double *lx, *ly, *lS;   // log rho_nu(log a) spline
  int nnu;
};

HD double rho_de(double a, double w0, double wa) { return pow(a, -3.0 * (1.0 + w0 + wa)) * exp(3.0 * (a - 1.0) * wa); }

HD double dtauda(const Bk& B, double a) {
  const double rhonu = exp(spl_ab(B.lx, B.ly, B.lS, B.nnu, log(a)));
  const double grho2 = B.grhom * B.Om * a + (B.grhog + B.grhor * (B.Neff + B.Nmnu * rhonu)) +
                       B.grhom * B.ODE * rho_de(a, B.w0, B.wa) * a * a * a * a + B.grhom * B.Ok * a * a;
  return sqrt(3.0 / grho2);
}

HD double aprimeoa(const Bk& B, double a) {
  const double rhonu = exp(spl_ab(B.lx, B.ly, B.lS, B.nnu, log(a)));
  const double grho = B.grhom * B.Om / a + (B.grhog + B.grhor * (B.Neff + B.Nmnu * rhonu)) / (a * a) +
                      B.grhom * B.ODE * rho_de(a, B.w0, B.wa) * a * a + B.grhom * B.Ok;
  return sqrt(grho / 3.0);
}

// Romberg on [a, b], 2^(i-1) new midpoints per level, depth divmax
// (jax_cosmo romb, divmax 6, as background.py:182 / thermodynamics_recfast.py:484 call it)
HD double romberg_dtauda(const Bk& B, double a, double b, int divmax) {
  double R[8], nR[8];
  const double rng = b - a;
  R[0] = rng * 0.5 * (dtauda(B, a) + dtauda(B, b));
  for (int i = 1; i <= divmax; ++i) {
    const int npan = 1 << (i - 1);
    const double h = rng / npan;
    double s = 0.0;
    for (int j = 0; j < npan; ++j) s += dtauda(B, a + h * (j + 0.5));
    nR[0] = 0.5 * R[0] + 0.5 * h * s;
    double fac = 1.0;
    for (int j = 1; j <= i; ++j) {
      fac *= 4.0;
      nR[j] = (fac * nR[j - 1] - R[j - 1]) / (fac - 1.0);
    }
    for (int j = 0; j <= i; ++j) R[j] = nR[j];
  }
  return R[divmax];
}

// ---------------------------------------------------------------- RECFAST
// The branch decisions of one RHS evaluation (nine conditions on the state
// values, one bit each): taken freely (no Br), recorded (mode 1: bits out)
// or replayed from a leading set's record (mode 2: bits in), so that a
// theta +- eps set evaluates the branches the nominal values selected, as
// jax.jacfwd differentiates a jnp.where on the nominal values.
struct Br {
  int mode = 0;
  unsigned bits = 0;
};
enum { BR_TSIGN = 0, BR_BOLTZ, BR_HE_EDGE, BR_H_PARTIAL, BR_H_SAHA, BR_H_PEEBLES0, BR_HE_ZERO, BR_H_FULL, BR_TM_LOCK,
       BR_NBITS };

HD bool take(Br* b, int bit, bool c) {
  if (!b) return c;
  if (b->mode == 2) return ((b->bits >> bit) & 1u) != 0;
  if (c) b->bits |= 1u << bit;
  return c;
}

// d(x_H, x_He, T_m)/da (thermodynamics_recfast.py:124-281); branch
// conditions on the values (or replayed, see Br); aH = a'/a at a
template <class S>
HD void ion_rhs(const TC& K, const Bk& B, double a, const S* y, double aH, S* f, Br* br = nullptr) {
  const double z = 1.0 / a - 1.0;
  const double H = B.H0 / 100.0;
  const double HO = H * K[DEB_TC_BIG_H];
  const double mu_H = 1.0 / (1.0 - B.YHe);
  const double fHe = B.fHe;
  const double Nnow = K[DEB_TC_DENS_FAC] * H * H * B.Ob / mu_H;
  const S x_H = y[0], x_He = y[1], T2 = y[2];
  const S x = x_H + fHe * x_He;
  const S Tmat = take(br, BR_TSIGN, val(T2) >= 0.0) ? T2 : -T2;
  const double zt = 1.0 + z;
  const double n = Nnow * zt * zt * zt;
  const double n_He = fHe * n;
  const double Trad = B.Tcmb * zt;
  const double Hz = (1e-5 * aH) / a * K[DEB_TC_C] * K[DEB_TC_BIG_H];
  const S Tm4 = Tmat / 1e4;
  const S CRT15 = dpow(K[DEB_TC_CR] * Tmat, 1.5);
  const S Rdown = 1e-19 * K[DEB_TC_A_PPB] * dpow(Tm4, K[DEB_TC_B_PPB]) / (1.0 + K[DEB_TC_C_PPB] * dpow(Tm4, K[DEB_TC_D_PPB]));
  const S Rup = Rdown * CRT15 * dexp(-K[DEB_TC_CDB] / Tmat);
  const S sq0 = dsqrt(Tmat / K[DEB_TC_T0]);
  const S sq1 = dsqrt(Tmat / K[DEB_TC_T1]);
  const S Rdown_He = K[DEB_TC_A_VF] / (sq0 * dpow(1.0 + sq0, 1.0 - K[DEB_TC_B_VF]) * dpow(1.0 + sq1, 1.0 + K[DEB_TC_B_VF]));
  const S Rup_He = 4.0 * Rdown_He * CRT15 * dexp(-K[DEB_TC_CDB_HE] / Tmat);
  const S bt = K[DEB_TC_BFACT] / Tmat;
  const S He_Boltz = dexp(take(br, BR_BOLTZ, val(bt) < 680.0) ? bt : S(680.0));
  const S Rdown_trip = K[DEB_TC_A_TRIP] / (sq0 * dpow(1.0 + sq0, 1.0 - K[DEB_TC_B_TRIP]) * dpow(1.0 + sq1, 1.0 + K[DEB_TC_B_TRIP]));
  const S Rup_trip = Rdown_trip * dexp(-K[DEB_TC_HCL_HE2ST_ION_KB] / Tmat) * CRT15 * (4.0 / 3.0);
  const double lz = log(zt);
  const double g1 = (lz - K[DEB_TC_ZGAUSS1]) / K[DEB_TC_WGAUSS1], g2 = (lz - K[DEB_TC_ZGAUSS2]) / K[DEB_TC_WGAUSS2];
  const double KK = K[DEB_TC_CK] / Hz * (1.0 + K[DEB_TC_AGAUSS1] * exp(-(g1 * g1)) + K[DEB_TC_AGAUSS2] * exp(-(g2 * g2)));
  const S omxHe = 1.0 - x_He;
  const S omxH = 1.0 - x_H;
  const S nHe1 = n_He * omxHe;
  const double Hzz = Hz * zt;
  const double xHe_r = val(x_He), xH_r = val(x_H);
  const bool he_edge = take(br, BR_HE_EDGE, (xHe_r < 5e-9) || (xHe_r > 0.98));
  const double c2 = K[DEB_TC_C] * K[DEB_TC_C];
  S K_He;
  if (he_edge) {
    K_He = S(K[DEB_TC_CK_HE] / Hz);
  } else {
    const S tauHe_s = K[DEB_TC_A2P_S] * K[DEB_TC_CK_HE] * 3.0 * nHe1 / Hz;
    const S pHe_s = (1.0 - dexp(-tauHe_s)) / tauHe_s;
    if (take(br, BR_H_PARTIAL, xH_r < 0.9999999)) {
      const S Dop = dsqrt(2.0 * K[DEB_TC_KB] * Tmat / (K[DEB_TC_MH] * K[DEB_TC_MHE_MH] * c2));
      const S Dop_2p = K[DEB_TC_C] * K[DEB_TC_L_HE_2P] * Dop;
      const double cl = K[DEB_TC_C] * K[DEB_TC_L_HE_2P];
      const S g2Ps = (3.0 * K[DEB_TC_A2P_S] * fHe * omxHe * c2) /
                     (K[DEB_TC_SQRT_PI] * K[DEB_TC_SIGMA_HE_2PS] * 8.0 * K[DEB_TC_PI] * Dop_2p * omxH * (cl * cl));
      const S AHcon = K[DEB_TC_A2P_S] / (1.0 + 0.36 * dpow(g2Ps, 0.86));
      K_He = 1.0 / ((K[DEB_TC_A2P_S] * pHe_s + AHcon) * 3.0 * nHe1);
    } else {
      K_He = 1.0 / (K[DEB_TC_A2P_S] * pHe_s * 3.0 * nHe1);
    }
  }
  const double Trad4 = Trad * Trad * Trad * Trad;
  const S timeTh = (1.0 / (K[DEB_TC_CT] * Trad4)) * (1.0 + x + fHe) / x;
  const double timeH = 2.0 / (3.0 * HO * pow(zt, 1.5));
  S f0, f1, f2;
  if (take(br, BR_H_SAHA, xH_r > 0.99)) {
    f0 = 0.0 * x_H;
  } else {
    const S rate = x * x_H * n * Rdown - Rup * omxH * dexp(-K[DEB_TC_CL] / Tmat);
    if (take(br, BR_H_PEEBLES0, xH_r > 0.985)) {
      f0 = rate / Hzz;
    } else {
      const S KLn = KK * K[DEB_TC_LAMBDA_H] * n * omxH;
      const S den = 1.0 / K[DEB_TC_FU] + KLn / K[DEB_TC_FU] + KK * Rup * n * omxH;
      f0 = rate * (1.0 + KLn) / (Hzz * den);
    }
  }
  if (take(br, BR_HE_ZERO, xHe_r < 1e-8)) {
    f1 = 0.0 * x_He;
  } else {
    const S rate_He = x * x_He * n * Rdown_He - Rup_He * omxHe * dexp(-K[DEB_TC_CL_HE] / Tmat);
    const S KHL = K_He * K[DEB_TC_LAMBDA_HE] * nHe1 * He_Boltz;
    const S Hden = 1.0 + K_He * (K[DEB_TC_LAMBDA_HE] + Rup_He) * nHe1 * He_Boltz;
    f1 = rate_He * (1.0 + KHL) / (Hzz * Hden);
    if (!he_edge) {
      const double l3 = K[DEB_TC_L_HE_2PT] * K[DEB_TC_L_HE_2PT] * K[DEB_TC_L_HE_2PT];
      const S tauHe_t = K[DEB_TC_A2P_T] * nHe1 * 3.0 / (8.0 * K[DEB_TC_PI] * Hz * l3);
      const S pHe_t = (1.0 - dexp(-tauHe_t)) / tauHe_t;
      const S ePSt = dexp(-K[DEB_TC_CL_PST] / Tmat);
      S CfHe_t;
      if (take(br, BR_H_FULL, xH_r > 0.99999)) {
        CfHe_t = K[DEB_TC_A2P_T] * pHe_t * ePSt;
      } else {
        const S Dop = dsqrt(2.0 * K[DEB_TC_KB] * Tmat / (K[DEB_TC_MH] * K[DEB_TC_MHE_MH] * c2));
        const S Dop_2Pt = K[DEB_TC_C] * K[DEB_TC_L_HE_2PT] * Dop;
        const double cl = K[DEB_TC_C] * K[DEB_TC_L_HE_2PT];
        const S g2Pt = (3.0 * K[DEB_TC_A2P_T] * fHe * omxHe * c2) /
                       (K[DEB_TC_SQRT_PI] * K[DEB_TC_SIGMA_HE_2PT] * 8.0 * K[DEB_TC_PI] * Dop_2Pt * omxH * (cl * cl));
        const S AHcon_t = K[DEB_TC_A2P_T] / (1.0 + 0.66 * dpow(g2Pt, 0.9)) / 3.0;
        CfHe_t = (K[DEB_TC_A2P_T] * pHe_t + AHcon_t) * ePSt;
      }
      CfHe_t = CfHe_t / (Rup_trip + CfHe_t);
      const S trip = x * x_He * n * Rdown_trip - omxHe * 3.0 * Rup_trip * dexp(-K[DEB_TC_HCL_HE2ST_KB] / Tmat);
      f1 = f1 + trip * CfHe_t / Hzz;
    }
  }
  if (take(br, BR_TM_LOCK, val(timeTh) < K[DEB_TC_H_FRAC] * timeH)) {
    f2 = Tmat / zt;
  } else {
    f2 = K[DEB_TC_CT] * Trad4 * x / (1.0 + x + fHe) * (Tmat - Trad) / Hzz + 2.0 * Tmat / zt;
  }
  const double dzda = -1.0 / (a * a);
  f[0] = f0 * dzda;
  f[1] = f1 * dzda;
  f[2] = f2 * dzda;
}

HD void matvec3(const double M[3][3], const double* v, double* o) {
  for (int i = 0; i < 3; ++i) o[i] = M[i][0] * v[0] + M[i][1] * v[1] + M[i][2] * v[2];
}

// inverse of a 3x3 matrix by Gauss-Jordan with partial pivoting
HD void inv3(const double A[3][3], double X[3][3]) {
  double M[3][6];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) { M[i][j] = A[i][j]; M[i][j + 3] = (i == j) ? 1.0 : 0.0; }
  for (int c = 0; c < 3; ++c) {
    int p = c;
    for (int r = c + 1; r < 3; ++r) if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
    if (p != c) for (int j = 0; j < 6; ++j) { const double t = M[c][j]; M[c][j] = M[p][j]; M[p][j] = t; }
    const double ip = 1.0 / M[c][c];
    for (int j = 0; j < 6; ++j) M[c][j] *= ip;
    for (int r = 0; r < 3; ++r) {
      if (r == c) continue;
      const double f = M[r][c];
      for (int j = 0; j < 6; ++j) M[r][j] -= f * M[c][j];
    }
  }
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) X[i][j] = M[i][j + 3];
}

// one GRK4A step, every stage at t0 (ode_integrators_stiff.py:117-223)
HD void grk4a_step(const TC& K, const Bk& B, double t0, double dt, const double* y0, double aH, double* y1,
                           double* err, Br* br3 = nullptr) {
  D3 yd[3], fd[3];
  for (int i = 0; i < 3; ++i) { yd[i] = D3(y0[i]); yd[i].d[i] = 1.0; }
  ion_rhs<D3>(K, B, t0, yd, aH, fd, br3);
  int ev = 0;
  double J[3][3], A[3][3], Ai[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) { J[i][j] = fd[i].d[j] * dt; A[i][j] = (i == j ? 1.0 : 0.0) - K[DEB_TC_G] * J[i][j]; }
  inv3(A, Ai);
  auto f = [&](const double* y, double* o) {
    ion_rhs<double>(K, B, t0, y, aH, o, br3 ? br3 + (++ev) : nullptr);
    for (int i = 0; i < 3; ++i) o[i] *= dt;
  };
  double f0[3] = {fd[0].v * dt, fd[1].v * dt, fd[2].v * dt};
  double k1[3], k2[3], k3[3], k4[3], Jk1[3], Jk2[3], Jk3[3], t[3], u[3], f2[3];
  matvec3(Ai, f0, k1);
  matvec3(J, k1, Jk1);
  for (int i = 0; i < 3; ++i) u[i] = y0[i] + K[DEB_TC_A21] * k1[i];
  f(u, t);
  for (int i = 0; i < 3; ++i) t[i] += K[DEB_TC_G21] * Jk1[i];
  matvec3(Ai, t, k2);
  matvec3(J, k2, Jk2);
  for (int i = 0; i < 3; ++i) u[i] = y0[i] + K[DEB_TC_A31] * k1[i] + K[DEB_TC_A32] * k2[i];
  f(u, f2);
  for (int i = 0; i < 3; ++i) t[i] = f2[i] + K[DEB_TC_G31] * Jk1[i] + K[DEB_TC_G32] * Jk2[i];
  matvec3(Ai, t, k3);
  matvec3(J, k3, Jk3);
  for (int i = 0; i < 3; ++i) t[i] = f2[i] + K[DEB_TC_G41] * Jk1[i] + K[DEB_TC_G42] * Jk2[i] + K[DEB_TC_G43] * Jk3[i];
  matvec3(Ai, t, k4);
  for (int i = 0; i < 3; ++i) {
    y1[i] = y0[i] + K[DEB_TC_C1] * k1[i] + K[DEB_TC_C2] * k2[i] + K[DEB_TC_C3] * k3[i] + K[DEB_TC_C4] * k4[i];
    err[i] = (K[DEB_TC_C1] - K[DEB_TC_CH1]) * k1[i] + (K[DEB_TC_C2] - K[DEB_TC_CH2]) * k2[i] +
             (K[DEB_TC_C3] - K[DEB_TC_CH3]) * k3[i] + K[DEB_TC_C4] * k4[i];
  }
}

// Accepted steps of one set's history: a leading set's adaptive solve
// writes (end, branch word) pairs, steps[2 pos], steps[2 pos + 1], while
// pos < cap (pos keeps counting past cap, so that an overflow shows) and
// the branch word of each interval's closing RHS evaluation into *fin; the
// sets that follow it replay them.
struct StepLog {
  double* steps = nullptr;
  int* pos = nullptr;
  int cap = 0;
  double* fin = nullptr;
};

// the three RHS evaluations of a GRK4A step in one exact integer word
HD double pack3(const Br* b) {
  return (double)(b[0].bits | (b[1].bits << BR_NBITS) | (b[2].bits << (2 * BR_NBITS)));
}
HD void unpack3(double w, Br* b) {
  const unsigned u = (unsigned)w, m = (1u << BR_NBITS) - 1u;
  for (int i = 0; i < 3; ++i) { b[i].mode = 2; b[i].bits = (u >> (i * BR_NBITS)) & m; }
}

// adaptive GRK4A from astart to aend under the I-controller the reference
// inherits (safety 0.9, factor in [0.2, 10], error order 3, RMS norm);
// out: x_H, x_He, T_m and their d/da at aend.  Returns false when the step
// budget ran out before aend.  With `rep` (nrep (end, branch word) pairs,
// the last end aend, and the closing evaluation's word *rep_fin) the steps
// end there and take those branches instead, every step accepted: the
// nominal step sequence a theta +- eps set follows, so that its tables are a
// smooth function of theta -- the derivative jax.jacfwd takes through the
// reference's diffeqsolve (thermodynamics_recfast.py:283-298, forward mode
// through the nominal steps and the branches the nominal values select).
HD bool solve_ionization(const TC& K, const Bk& B, double astart, double aend, const double* ystart, double rtol,
                                 double atol, int max_steps, double* out, StepLog slog = StepLog(),
                                 const double* rep = nullptr, int nrep = 0, double rep_fin = 0.0) {
  double t0 = astart;
  double t1 = fmin(astart + fabs(astart) * 1e-3, aend);
  double y[3] = {ystart[0], ystart[1], ystart[2]};
  int steps = 0;
  Br fin;
  if (rep) {
    bool ok = true;
    for (int j = 0; j < nrep; ++j) {
      double y1[3], e[3];
      Br b3[3];
      unpack3(rep[2 * j + 1], b3);
      grk4a_step(K, B, t0, rep[2 * j] - t0, y, aprimeoa(B, t0), y1, e, b3);
      ok = ok && !(isnan(y1[0]) || isnan(y1[1]) || isnan(y1[2]));
      y[0] = y1[0]; y[1] = y1[1]; y[2] = y1[2];
      t0 = rep[2 * j];
    }
    fin.mode = 2;
    fin.bits = (unsigned)rep_fin;
    double dy[3];
    ion_rhs<double>(K, B, aend, y, aprimeoa(B, aend), dy, &fin);
    out[0] = y[0]; out[1] = y[1]; out[2] = y[2]; out[3] = dy[0]; out[4] = dy[1]; out[5] = dy[2];
    return ok && t0 == aend;
  }
  while (t0 < aend && steps < max_steps) {
    const double dt = t1 - t0;
    const double aH = aprimeoa(B, t0);
    double y1[3], e[3];
    Br b3[3];
    for (int i = 0; i < 3; ++i) b3[i].mode = 1;
    grk4a_step(K, B, t0, dt, y, aH, y1, e, slog.pos ? b3 : nullptr);
    const bool nan1 = isnan(y1[0]) || isnan(y1[1]) || isnan(y1[2]);
    double ss = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double yc = nan1 ? y[i] : y1[i];
      const double sc = e[i] / (atol + rtol * fmax(fabs(y[i]), fabs(yc)));
      ss += sc * sc;
    }
    const double en = sqrt(ss / 3.0);
    const bool keep = en < 1.0;
    const double inv = en == 0.0 ? HUGE_VAL : 1.0 / en;
    double fac = 0.9 * pow(inv, 1.0 / 3.0);
    fac = fmin(fmax(fac, keep ? 1.0 : 0.2), 10.0);
    if (keep) {
      y[0] = y1[0]; y[1] = y1[1]; y[2] = y1[2];
      t0 = t1;
      if (slog.pos) {
        if (*slog.pos < slog.cap) { slog.steps[2 * *slog.pos] = t1; slog.steps[2 * *slog.pos + 1] = pack3(b3); }
        ++*slog.pos;
      }
    }
    t1 = t0 + dt * fac;
    if (t1 > aend - 1e-10) t1 = aend;
    ++steps;
  }
  fin.mode = 1;
  double dy[3];
  ion_rhs<double>(K, B, aend, y, aprimeoa(B, aend), dy, slog.fin ? &fin : nullptr);
  if (slog.fin) *slog.fin = (double)fin.bits;
  out[0] = y[0]; out[1] = y[1]; out[2] = y[2]; out[3] = dy[0]; out[4] = dy[1]; out[5] = dy[2];
  return t0 >= aend;
}

// The positive root of x^2 + b x - c = 0 (c >= 0), (sqrt(b^2 + 4c) - b) / 2,
// the form of the Saha fractions (thermodynamics_recfast.py:302-321,
// 362-452); written as 2c / (sqrt(b^2 + 4c) + b) when b > 0, the same number
// without the cancellation that costs the direct form ~b * 1e-16 absolute
// (1e-7 for the hydrogen fraction near z = 2000), noise that a difference
// quotient over parameter sets would divide by 2 eps.
HD double quad_root(double b, double c) {
  const double s = sqrt(b * b + 4.0 * c);
  return b > 0.0 ? 2.0 * c / (s + b) : 0.5 * (s - b);
}

HD double saha_heii(const TC& K, const Bk& B, double a) {
  const double fHe = B.fHe;
  const double Hfac = 1.0 / (1.0e06 * 3.0856775807e13);
  const double mu_H = 1.0 / (1.0 - B.YHe);
  const double hh = B.H0 * Hfac;
  const double rho_c = 3.0 * hh * hh / (8.0 * K[DEB_TC_PI] * K[DEB_TC_G_N]);
  const double NH = rho_c * B.Ob / (K[DEB_TC_MH] * mu_H) / (a * a * a);
  const double T = B.Tcmb / a;
  const double betaE = K[DEB_TC_E_ION_HE12S] / T;
  const double A = 1.0 + fHe, Bq = 1.0 + 2.0 * fHe;
  const double R = pow(2.0 * K[DEB_TC_PI] * K[DEB_TC_ME] * K[DEB_TC_KB] / (K[DEB_TC_H_PLANCK] * K[DEB_TC_H_PLANCK]) * T, 1.5) / NH *
                   exp(-betaE);
  if (R > 1e5) return fHe * (1.0 - Bq / R + (1.0 + 5.0 * fHe + 6.0 * fHe * fHe) / (R * R));
  return quad_root(R - A, R * Bq) - A;
}

struct TParams {
  const double* params;    // [nset, DEB_BG_NPARAM]
  int nset;
  const double* consts;    // DEB_TC_COUNT
  const double* a_nu;      // [num_nu] neutrino table scale factors
  const double* la_nu;     // [num_nu] their logs
  const double* qw_bg;     // [2 nq_bg] background momentum nodes, weights
  const double* qw;        // [2 nqmax] perturbation momentum nodes, weights
  const double* a_th;      // [num_thermo + 1] thermal sampling
  const double* la_th;     // [num_thermo] log of a_th[1:]
  int num_nu, num_thermo, nq_bg, nqmax, max_steps;
  double amin, rtol, atol;
  double* tables;          // [nset, blob_len]
  int blob_len;
  int* status;             // [nset] DEB_BG_* bits, 0 = ok
  // frozen step sequences (all null/0: every set adaptive, one pass):
  const int* leader = nullptr;   // [nset] -1: adaptive, recorded; j >= 0: follows set j
  double* steps = nullptr;       // [nset, step_stride]: first step of each interval [num_thermo + 1],
                                 // case of each interval and the branch word of its closing RHS
                                 // evaluation [2 num_thermo], (end, branch word) of each step [2 step_cap]
  int step_cap = 0;
  int phase = 0;                 // 1: the adaptive sets, 2: the sets that follow one
};

HD long step_stride(const TParams& P) { return 3L * P.num_thermo + 1 + 2L * P.step_cap; }

HD void put_derived(double* blob, long& p, const double* x, const double* y, const double* S, int n, int lane, int G) {
  double* c = blob + p;
  for (int i = lane; i < n - 1; i += G) {
    const double h = x[i + 1] - x[i];
    c[4 * i] = y[i];
    c[4 * i + 1] = (y[i + 1] - y[i]) / h - h * (S[i + 1] + 2.0 * S[i]) / 6.0;
    c[4 * i + 2] = S[i] / 2.0;
    c[4 * i + 3] = (S[i + 1] - S[i]) / (6.0 * h);
  }
  p += 4L * (n - 1);
  float* xf = reinterpret_cast<float*>(blob + p);
  const int nf = (n + 1) / 2 * 2;
  for (int i = lane; i < nf; i += G) xf[i] = i < n ? (float)x[i] : HUGE_VAL;
  p += (n + 1) / 2;
}

// dynamic shared memory per block, in doubles: the thermal arrays [6 N],
// x_e and tau [2 N], Thomas scratch for the splines built in parallel
// (2 neutrino splines of NN knots or 5 thermal splines of N knots)
HD long tables_smem_doubles(int N, int NN) {
  const long th = 6L * N + 2L * N;
  const long scr = 4L * NN > 10L * N ? 4L * NN : 10L * N;
  return th + scr;
}

// All tables of parameter set `set` into its blob; lanes lane, lane + G, ...
// of a group of G share the sampled work; sh: tables_smem_doubles() doubles.
HD void produce_set(const TParams& P, int set, int lane, int G, double* sh) {
  if (set >= P.nset) return;
  // the set's role with frozen step sequences: leaders in phase 1, the sets
  // that follow one in phase 2 (a leader index out of range or itself a
  // follower is refused with DEB_BG_BAD_LEADER and the set runs adaptive)
  int lead = -1, bad_leader = 0;
  if (P.leader) {
    lead = P.leader[set];
    if ((lead >= 0) != (P.phase == 2)) return;
    if (lead >= 0 && (lead >= P.nset || P.leader[lead] >= 0)) {
      lead = -1;
      bad_leader = DEB_BG_BAD_LEADER;
    }
  }
  const int N = P.num_thermo, NN = P.num_nu;
  double* th = sh;                 // [6][N]: x_H, x_He, T_m, dx_H/da, dx_He/da, dT_m/da
  double* xe = sh + 6 * N;         // [N]
  double* tau = xe + N;            // [N]
  double* scr = tau + N;
  const TC K{P.consts};
  const double* pr = P.params + (long)set * DEB_BG_NPARAM;
  Bk B;
  B.Om = pr[DEB_BG_OMEGAM]; B.Ob = pr[DEB_BG_OMEGAB]; B.H0 = pr[DEB_BG_H0]; B.Tcmb = pr[DEB_BG_TCMB];
  B.YHe = pr[DEB_BG_YHE]; B.Neff = pr[DEB_BG_NEFF]; B.Nmnu = pr[DEB_BG_NMNU]; B.w0 = pr[DEB_BG_W0];
  B.wa = pr[DEB_BG_WA]; B.Ok = pr[DEB_BG_OMEGAK];
  const double mnu = pr[DEB_BG_MNU];
  const double T2 = B.Tcmb * B.Tcmb, T4 = T2 * T2;
  // setup_background_evolution (background.py:140-188)
  B.grhom = 3.33795017e-11 * B.H0 * B.H0;
  B.grhog = 1.49594245e-13 * T4;
  B.grhor = 3.39739477e-14 * T4;
  const double adotrad = sqrt((B.grhog + B.grhor * (B.Neff + B.Nmnu)) / 3.0);
  const double amnu = mnu * K[DEB_TC_C2OK] / B.Tcmb;
  B.fHe = B.YHe / (K[DEB_TC_MHE_MH] * (1.0 - B.YHe));
  double* blob = P.tables + (long)set * P.blob_len;
  // blob layout: header, 7 splines (x, y, S) in the order xe(loga),
  // cs2a(loga), lrhonu(loga), lpnu(loga), a(tau), tau(a), xe(tau), nodes,
  // derived section
  const int sizes[7] = {N, N, NN, NN, N, N, N};
  double* sx[7];
  double* sy[7];
  double* sS[7];
  long p = DEB_HDR_LEN;
  for (int s = 0; s < 7; ++s) {
    sx[s] = blob + p; sy[s] = blob + p + sizes[s]; sS[s] = blob + p + 2 * sizes[s];
    p += 3L * sizes[s];
  }
  // neutrino density and pressure tables (background.py:47-68, 158-167)
  for (int i = lane; i < NN; i += G) {
    const double a = P.a_nu[i];
    double rho = 0.0, pn = 0.0;
    for (int j = 0; j < P.nq_bg; ++j) {
      const double q = P.qw_bg[j], w = P.qw_bg[P.nq_bg + j];
      const double aq = a * amnu / q;
      const double v = 1.0 / sqrt(1.0 + aq * aq);
      rho += w / v;
      pn += w * v / 3.0;
    }
    sx[2][i] = P.la_nu[i]; sy[2][i] = log(rho);
    sx[3][i] = P.la_nu[i]; sy[3][i] = log(pn);
  }
  lane_sync(G);
  for (int l = lane; l < 2; l += G) natural_S(sx[2 + l], sy[2 + l], sS[2 + l], NN, scr + l * 2 * NN, scr + l * 2 * NN + NN);
  lane_sync(G);
  B.lx = sx[2]; B.ly = sy[2]; B.lS = sS[2]; B.nnu = NN;
  // closure (background.py:170-177)
  const double rhonu0 = exp(spl_ab(sx[2], sy[2], sS[2], NN, 0.0));
  const double Omegar = (B.Neff + B.Nmnu * rhonu0) * B.grhor / B.grhom;
  const double Omegag = B.grhog / B.grhom;
  B.ODE = 1.0 - B.Ok - Omegar - Omegag - B.Om;
  const double taumin = P.amin / adotrad;
  // ionisation history on lane 0 (thermodynamics_recfast.py:362-452)
  if (lane == 0) {
    const double H = B.H0 / 100.0, HO = H * K[DEB_TC_BIG_H];
    const double mu_H = 1.0 / (1.0 - B.YHe);
    const double Nnow = 3.0 * HO * HO * B.Ob / (8.0 * K[DEB_TC_PI] * K[DEB_TC_G_N] * mu_H * K[DEB_TC_MH]);
    const double Tc = B.Tcmb;
    int bad = 0;
    double prev[6];
    // step record of this set (a leader) or of the set it follows
    double* rec = (P.leader && P.steps && lead < 0 && !bad_leader) ? P.steps + (long)set * step_stride(P) : nullptr;
    const double* rep = (P.leader && P.steps && lead >= 0) ? P.steps + (long)lead * step_stride(P) : nullptr;
    int pos = 0;
    StepLog slog;
    if (rec) { slog.steps = rec + 3 * N + 1; slog.pos = &pos; slog.cap = P.step_cap; }
    // interval i: the leader's steps when it recorded all of them, adaptive
    // otherwise (the leader did not integrate it, or its record overflowed)
    auto solve = [&](int i, double astart, double aend, double* nw) {
      if (rep) {
        const int o0 = (int)rep[i], o1 = (int)rep[i + 1];
        if (o1 > o0 && o1 <= P.step_cap)
          return solve_ionization(K, B, astart, aend, prev, P.rtol, P.atol, P.max_steps, nw, StepLog(),
                                  rep + 3 * N + 1 + 2 * o0, o1 - o0, rep[2 * N + 1 + i]) ? 0 : (int)DEB_BG_STEPS;
        if (o1 > P.step_cap) bad |= DEB_BG_UNRECORDED;
      }
      StepLog lg = slog;
      if (rec) lg.fin = rec + 2 * N + 1 + i;
      return solve_ionization(K, B, astart, aend, prev, P.rtol, P.atol, P.max_steps, nw, lg) ? 0
                                                                                               : (int)DEB_BG_STEPS;
    };
    for (int i = 0; i < N; ++i) {
      const double astart = P.a_th[i], aend = P.a_th[i + 1];
      if (rec) rec[i] = pos;
      const double zstart = 1.0 / astart - 1.0, zend = 1.0 / aend - 1.0;
      if (i == 0) {
        prev[0] = 1.0; prev[1] = 1.0; prev[2] = Tc * (1.0 + zstart); prev[3] = 0.0; prev[4] = 0.0;
        prev[5] = -Tc * (1.0 + zstart);
      }
      double nw[6];
      // the case of the thermal history (thermodynamics_recfast.py:362-452); a
      // follower takes its leader's, as jax.jacfwd differentiates the branch
      // the nominal values select
      int br = zend > 3500.0 ? 0 : (i > 0 && prev[1] > 0.99) ? 1 : (i > 0 && prev[0] > 0.99) ? 2 : 3;
      if (rep && br != 0) br = (int)rep[N + 1 + i];
      if (rec) rec[N + 1 + i] = br;
      if (br == 0) {
        nw[0] = 1.0; nw[1] = 1.0; nw[2] = Tc * (1.0 + zend); nw[3] = 0.0; nw[4] = 0.0; nw[5] = -Tc * (1.0 + zend);
      } else if (br == 1) {
        const double rhs = exp(1.5 * log(K[DEB_TC_CR] * Tc / (1.0 + zend)) -
                               K[DEB_TC_H_PLANCK] * K[DEB_TC_C] * K[DEB_TC_L_HE1_ION] / K[DEB_TC_KB] / (Tc * (1.0 + zend))) /
                           Nnow * 4.0;
        const double xHe0 = quad_root(rhs - 1.0, (1.0 + B.fHe) * rhs);
        nw[0] = 1.0; nw[1] = (xHe0 - 1.0) / B.fHe; nw[2] = Tc * (1.0 + zend); nw[3] = 0.0; nw[4] = 0.0;
        nw[5] = -Tc * (1.0 + zend);
      } else if (br == 2) {
        const double rhs = exp(1.5 * log(K[DEB_TC_CR] * Tc / (1.0 + zend)) - K[DEB_TC_CB1] / (Tc * (1.0 + zend))) / Nnow;
        const double xH0 = quad_root(rhs, rhs);
        bad |= solve(i, astart, aend, nw);
        nw[0] = xH0;
        nw[3] = 0.0;
      } else {
        bad |= solve(i, astart, aend, nw);
      }
      for (int j = 0; j < 6; ++j) { th[j * N + i] = nw[j]; prev[j] = nw[j]; }
    }
    if (rec) {
      rec[N] = pos;
      if (pos > P.step_cap) bad |= DEB_BG_UNRECORDED;
    }
    if (P.status) P.status[set] = bad | bad_leader;
  }
  lane_sync(G);
  // per sample: x_e, c_s^2 a and the Romberg increment of tau
  // (thermodynamics_recfast.py:455-501)
  for (int i = lane; i < N; i += G) {
    const double a = P.a_th[i + 1];
    const double xeHeII = saha_heii(K, B, a);
    const double x = th[i] + B.fHe * th[N + i] + xeHeII;
    const double mu = 1.0 / (1.0 + (1.0 / K[DEB_TC_MHE_MH] - 1.0) * B.YHe + (1.0 - B.YHe) * x);
    const double Tm = th[2 * N + i], dTmda = th[5 * N + i];
    const double daTmda = Tm + a * dTmda;
    const double cs2 = K[DEB_TC_KB] / K[DEB_TC_MH] / (K[DEB_TC_C] * K[DEB_TC_C]) / mu * Tm * (4.0 - daTmda / Tm) / 3.0;
    xe[i] = x;
    sy[1][i] = a * cs2;
    tau[i] = i > 0 ? romberg_dtauda(B, P.a_th[i], a, 6) : 0.0;
  }
  lane_sync(G);
  if (lane == 0) {   // running sum in sample order, as the reference's scan
    double t = taumin;
    tau[0] = t;
    for (int i = 1; i < N; ++i) { t += tau[i]; tau[i] = t; }
  }
  lane_sync(G);
  for (int i = lane; i < N; i += G) {
    const double a = P.a_th[i + 1], la = P.la_th[i];
    sx[0][i] = la; sy[0][i] = xe[i];
    sx[1][i] = la;
    sx[4][i] = tau[i]; sy[4][i] = a;
    sx[5][i] = a; sy[5][i] = tau[i];
    sx[6][i] = tau[i]; sy[6][i] = xe[i];
  }
  lane_sync(G);
  for (int l = lane; l < 5; l += G) {
    const int s = l < 2 ? l : l + 2;   // splines 0, 1, 4, 5, 6
    natural_S(sx[s], sy[s], sS[s], N, scr + l * 2 * N, scr + l * 2 * N + N);
  }
  lane_sync(G);
  // header (tables.py layout)
  if (lane == 0) {
    const double hdr[19] = {B.Om, B.Ob, B.ODE, B.Ok, B.grhom, B.grhog, B.grhor, B.Neff, B.Nmnu, amnu, B.w0, B.wa,
                            pr[DEB_BG_CS2DE], B.YHe, B.H0, taumin, pr[DEB_BG_AS], pr[DEB_BG_NS], pr[DEB_BG_KP]};
    for (int i = 0; i < 19; ++i) blob[i] = hdr[i];
    blob[19] = P.nqmax;
    for (int s = 0; s < 7; ++s) blob[20 + s] = sizes[s];
    blob[27] = P.blob_len;
    blob[28] = DEB_TABLE_MAGIC;
    blob[30] = 0.0;
    blob[31] = 0.0;
  }
  // momentum nodes
  for (int i = lane; i < 2 * P.nqmax; i += G) blob[p + i] = P.qw[i];
  p += 2L * P.nqmax;
  if (lane == 0) blob[29] = (double)p;
  lane_sync(G);
  // derived section: polynomial coefficients and FP32 knots of each spline
  for (int s = 0; s < 7; ++s) put_derived(blob, p, sx[s], sy[s], sS[s], sizes[s], lane, G);
}

}  // namespace debt
