// adjoint_harness.cpp -- TEST-ONLY host build of the kernel's adjoint logic
// (disco-eb_gb300/csrc/deb_adjoint.cuh), one item at a time, so the tests
// can check every piece -- the bilinear form, J^T x, W^-T, the step and the
// whole solve backwards -- against dense matrices, the oracle and finite
// differences without a GPU.  It is never part of the library.
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "../../disco-eb_gb300/csrc/deb_adjoint.cuh"

using namespace deb;

namespace {
const Grp<1> GP{0};

struct Box {
  Dims D;
  Cosmo c;
  ModeConst m;
  Tab T;
  Rodas R;
  std::vector<double> buf, av, seg, sc;
  AWS<1> A;
};

bool setup(Box& x, const double* blob, int blob_len, const int* dims, double k, int seg_cap = 1) {
  x.D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  if (!load_cosmo(blob, blob_len, x.c)) return false;
  mode_const(x.c, k, x.m);
  fill_tables(x.T);
  fill_rodas(x.R);
  const int n = x.D.n;
  x.buf.assign(slot_len(x.D) * 32, 0.0);
  x.av.assign((size_t)NAV * n * 32, 0.0);
  x.seg.assign((size_t)seg_cap * n * 32, 0.0);
  x.sc.assign(SC_LEN, 0.0);
  WS<1>& w = x.A.w;
  w.p = x.buf.data(); w.n = n; w.misc0 = V_K0 * n;
  w.kp = w.p + hot_len(x.D) * 32;
  w.dp = nullptr;
  x.A.av = x.av.data(); x.A.seg = x.seg.data(); x.A.seg_cap = seg_cap; x.A.sc = x.sc.data(); x.A.n = n;
  for (int i = 0; i < x.D.nq; ++i) {
    const double q = x.c.q[i];
    w.m(M_Q + Q_DLF * x.D.nq + i) = -q / (1.0 + std::exp(-q));
    w.m(M_Q + Q_AMQ * x.D.nq + i) = x.m.amnu / q;
  }
  return true;
}
void put(const Box& x, VecRef v, const double* src) { for (int j = 0; j < x.D.n; ++j) v[j] = src[j]; }
void get(const Box& x, VecRef v, double* dst) { for (int j = 0; j < x.D.n; ++j) dst[j] = v[j]; }
}  // namespace

extern "C" {

int h_adj_ok() { return host_linv().ok; }

// r^T f(tau, y) through the bilinear form: out = [phi, x^T f, d phi/da,
// x^T df/da, d phi/dtau]
int h_adj_phi(const double* blob, int blob_len, const int* dims, double k, double tau, const double* xv,
              const double* y, double* out) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  const int n = b.D.n;
  const VecRef X = b.A.vec(A_RB), Y = b.A.vec(A_TMP);
  put(b, X, xv);
  put(b, Y, y);
  const double a = y[0], mu0 = a * b.m.amnu;
  bform<1>(GP, b.c, b.m, b.D, b.T, b.A.w, X, Y, mu0, true, b.sc.data() + SC_B, false);
  const double* B = b.sc.data() + SC_B;
  out[0] = phi<double>(coef<double>(b.c, b.m, b.D, a, tau, mu0), B, b.m.k);
  out[2] = phi<Jet<double>>(coef<Jet<double>>(b.c, b.m, b.D, Jet<double>(a, 1.0), Jet<double>(tau), mu0), B, b.m.k).d;
  out[4] = phi<Jet<double>>(coef<Jet<double>>(b.c, b.m, b.D, Jet<double>(a), Jet<double>(tau, 1.0), mu0), B, b.m.k).d;
  for (int j = 0; j < n; ++j) b.A.w.v(V_Y, j) = y[j];
  rhs<Dual, 1>(GP, b.c, b.m, b.D, b.T, tau, b.A.w, V_Y, V_K0, V_JC0);
  double s = 0.0, sa = 0.0;
  for (int j = 0; j < n; ++j) { s += xv[j] * b.A.w.v(V_K0, j); sa += xv[j] * b.A.w.v(V_JC0, j); }
  out[1] = s;
  out[3] = sa;
  return 0;
}

// z = J(tau, y)^T x (der = 0) or (dJ/da)^T x on indices >= 1 (der = 1)
int h_adj_jt(const double* blob, int blob_len, const int* dims, double k, double tau, const double* xv,
             const double* y, double* z, int der) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  if (!host_linv().ok) return -3;
  const int n = b.D.n;
  const VecRef X = b.A.vec(A_RB), Y = b.A.vec(A_TMP), Z = b.A.vec(A_UB);
  put(b, X, xv);
  put(b, Y, y);
  for (int j = 0; j < n; ++j) Z[j] = 0.0;
  const double a = y[0], mu0 = a * b.m.amnu;
  if (der) {
    const Coef<Jet<double>> C = coef<Jet<double>>(b.c, b.m, b.D, Jet<double>(a, 1.0), Jet<double>(tau), mu0);
    apply_jt<Jet<double>, 1>(GP, b.c, b.m, b.D, b.T, b.A.w, C, Jet<double>(a, 1.0), X, Z);
  } else {
    const Coef<double> C = coef<double>(b.c, b.m, b.D, a, tau, mu0);
    apply_jt<double, 1>(GP, b.c, b.m, b.D, b.T, b.A.w, C, a, X, Z);
    bform<1>(GP, b.c, b.m, b.D, b.T, b.A.w, X, Y, mu0, true, b.sc.data() + SC_B, false);
    Z[0] = phi<Jet<double>>(coef<Jet<double>>(b.c, b.m, b.D, Jet<double>(a, 1.0), Jet<double>(tau), mu0),
                            b.sc.data() + SC_B, b.m.k).d;
  }
  get(b, Z, z);
  return 0;
}

// z = W^-T rhs with W = I/(gamma dt) - J(tau, y), factored as the forward step does
int h_adj_solve_wt(const double* blob, int blob_len, const int* dims, double k, double tau, const double* y, double dt,
                   const double* rhsv, double* z) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  const int n = b.D.n;
  for (int j = 0; j < n; ++j) b.A.w.v(V_Y, j) = y[j];
  Bg<double> g;
  rhs<Dual, 1>(GP, b.c, b.m, b.D, b.T, tau, b.A.w, V_Y, V_K0, V_JC0, &g);
  const double d = 1.0 / (dt * b.R.gamma);
  factor_W<1>(GP, b.c, b.m, b.D, b.T, b.A.w, d, tau, g);
  const VecRef yh = b.A.vec(A_YH), ye = b.A.vec(A_YE), r = b.A.vec(A_RB);
  prep_wt<1>(GP, b.D, b.A.w, yh, ye);
  put(b, r, rhsv);
  solve_Wt<1>(GP, b.D, b.A.w, r, yh, ye, g.wQ);
  get(b, r, z);
  return 0;
}

// the block solve alone: z = M^-1 b (trans = 0) or M^-T b (trans = 1) on indices >= 2
int h_adj_solve_m(const double* blob, int blob_len, const int* dims, double k, double tau, const double* y, double dt,
                  const double* rhsv, double* z, int trans) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  const int n = b.D.n;
  for (int j = 0; j < n; ++j) b.A.w.v(V_Y, j) = y[j];
  Bg<double> g;
  rhs<Dual, 1>(GP, b.c, b.m, b.D, b.T, tau, b.A.w, V_Y, V_K0, V_JC0, &g);
  const double d = 1.0 / (dt * b.R.gamma);
  factor_W<1>(GP, b.c, b.m, b.D, b.T, b.A.w, d, tau, g);
  const VecRef r = b.A.vec(A_RB);
  put(b, r, rhsv);
  if (trans) {
    solve_Mt<1>(GP, b.D, b.A.w, r);
  } else {
    for (int j = 0; j < n; ++j) b.A.w.v(V_K0, j) = rhsv[j];
    solve_M<1>(GP, b.m, b.D, b.A.w, d, g.aH, V_K0);
    for (int j = 0; j < n; ++j) r[j] = b.A.w.v(V_K0, j);
  }
  get(b, r, z);
  return 0;
}

// the output fields of the state y as the forward kernel converts them
// (deb::outputs) and as the adjoint writes them (outputs_s of 13 scalars)
int h_adj_outputs_pair(const double* blob, int blob_len, const int* dims, double k, const double* y, double* r_kernel,
                       double* r_s) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  const Dims& D = b.D;
  const int n = D.n, nq = D.nq;
  for (int j = 0; j < n; ++j) b.A.w.v(V_Y, j) = y[j];
  outputs<1>(b.c, b.m, D, b.A.w, V_Y, r_kernel, 1);
  double drho = 0.0, fnu = 0.0;
  for (int i = 0; i < nq; ++i) {
    const double aq = y[0] * b.m.amnu / b.c.q[i];
    drho += b.c.w[i] * y[D.iq0 + i] * std::sqrt(1.0 + aq * aq);
    fnu += b.c.w[i] * y[D.iq0 + nq + i];
  }
  const double s[13] = {y[2], y[3], y[4], y[5], y[6], y[7], y[8], y[D.ir], y[D.ir + 1], y[n - 2], y[n - 1], drho, fnu};
  outputs_s<double>(b.c, b.m, y[0], s, r_s);
  return 0;
}

// the 20 output fields from the 13 state scalars (a-jet: d/da into dr)
int h_adj_outputs(const double* blob, int blob_len, const int* dims, double k, double a, const double* s, double* r,
                  double* dr) {
  Box b;
  if (!setup(b, blob, blob_len, dims, k)) return -2;
  outputs_s<double>(b.c, b.m, a, s, r);
  Jet<double> rj[20];
  outputs_s<Jet<double>>(b.c, b.m, Jet<double>(a, 1.0), s, rj);
  for (int i = 0; i < 20; ++i) dr[i] = rj[i].d;
  return 0;
}

// One Rosenbrock step from (t0, y0) over dt on tables[0]: y1.  With lam
// (dL/dy1) given, also the step adjoint: ybar0, [tbar0, dtbar], thbar[npar]
// (tables: nominal then 2 npar perturbed blobs).
int h_step_adj(const double* tables, int npar, int blob_len, const int* dims, double k, double t0, double dt,
               const double* y0, const double* eps, const double* lamv, double* y1, double* ybar0, double* tb,
               double* thbar) {
  Box b;
  if (!setup(b, tables, blob_len, dims, k)) return -2;
  const int n = b.D.n;
  // the momentum-bin constants of the nominal tables (as initial_conditions leaves them)
  for (int j = 0; j < n; ++j) b.A.w.v(V_Y, j) = y0[j];
  Ctl ctl;
  ctl.dense = 0; ctl.nout = 1; ctl.replay = 1; ctl.record = 0; ctl.step_ts = 0; ctl.return_full = 0;
  Run r;
  r.t0 = t0; r.t1 = t0 + dt; r.vy = V_Y; r.vu = V_U;
  bool bad;
  Bg<double> g0;
  step_attempt<1>(GP, b.c, b.m, b.D, b.T, b.R, ctl, b.A.w, r, bad, &g0);
  for (int j = 0; j < n; ++j) y1[j] = b.A.w.v(V_U, j);
  if (!lamv) return 0;
  AdjItem it;
  it.blob0 = tables; it.blobs = tables + blob_len; it.blob_len = blob_len; it.npar = npar; it.eps = eps;
  it.k = k;
  put(b, b.A.vec(A_LAM), lamv);
  for (int i = 0; i < 16; ++i) b.sc[SC_TH + i] = 0.0;
  double tb0, dtb;
  step_adjoint<1>(GP, it, b.c, b.m, b.D, b.T, b.R, b.A, V_U, t0, dt, g0, tb0, dtb);
  get(b, b.A.vec(A_LAM), ybar0);
  tb[0] = tb0; tb[1] = dtb;
  for (int p = 0; p < npar; ++p) thbar[p] = b.sc[SC_TH + p];
  return 0;
}

// One mode end to end: the recorded nominal solve with checkpoints (the
// forward kernel's record path), then the adjoint item for the cotangent gy
// [nout][20].  tables: nominal blob then 2 npar perturbed blobs; tau_out:
// [1 + 2 npar][nout].  Outputs: gth[npar], y_out[nout][20] of the nominal
// solve, nrec and the checkpoint stride; returns the adjoint's status.
int h_adjoint(const double* tables, int npar, int blob_len, double k, const double* tau_out, int nout, const int* dims,
              const double* cfg, int max_steps, int ck_cap, const double* eps, const double* gy, double* gth,
              double* y_out, int* info, double* dbg) {
  const Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  const int n = D.n;
  Ctl ctl;
  ctl.rtol = cfg[0]; ctl.atol = cfg[1];
  ctl.b1 = (cfg[3] + cfg[2] + cfg[4]) / cfg[7]; ctl.b2 = -(cfg[2] + 2.0 * cfg[4]) / cfg[7]; ctl.b3 = cfg[4] / cfg[7];
  ctl.fmax = cfg[5]; ctl.fmin = cfg[6]; ctl.safety = cfg[8]; ctl.hist_on_reject = (int)cfg[9];
  ctl.max_steps = max_steps; ctl.dense = 0; ctl.return_full = 0; ctl.nout = nout;
  ctl.record = 1; ctl.replay = 0; ctl.step_ts = (int)cfg[10];
  std::vector<double> rec(max_steps + 1), ck((size_t)ck_cap * n);
  Box f;
  if (!setup(f, tables, blob_len, dims, k)) return -2;
  for (int i = 0; i < nout * 20; ++i) y_out[i] = std::numeric_limits<double>::quiet_NaN();
  Run r;
  r.rec = rec.data(); r.rec_cap = max_steps; r.nrec = 0;
  r.ck = ck.data(); r.ck_cap = ck_cap;
  mode_begin<1>(GP, f.c, f.m, f.D, ctl, f.A.w, tau_out, r);
  while (mode_step<1>(GP, f.c, f.m, f.D, f.T, f.R, ctl, f.A.w, tau_out, y_out, 1, r)) {}
  info[0] = r.status; info[1] = r.acc; info[2] = r.ck_stride; info[3] = r.rej;
  if (r.status != ST_OK) return -4;
  // ck is laid out [slot][n] (stride 1 per element here, as on the GPU)
  Box b;
  if (!setup(b, tables, blob_len, dims, k, r.ck_stride)) return -2;
  AdjItem it;
  it.blob0 = tables; it.blobs = tables + blob_len; it.blob_len = blob_len; it.npar = npar; it.eps = eps;
  it.tau0 = tau_out; it.taus = tau_out + nout; it.rec = rec.data(); it.nrec = r.acc; it.ck = ck.data();
  it.ck_stride = r.ck_stride; it.gy = gy; it.k = k;
  const int st = adjoint_item<1>(GP, it, b.D, b.T, b.R, nout, b.A, gth);
  if (dbg) {   // dL/dy0, dL/dtau_start (through the scaled step times), dL/dtau_out[o], record
    get(b, b.A.vec(A_LAM), dbg);
    dbg[n] = b.sc[SC_SCAL + SS_STS];
    for (int o = 0; o < nout; ++o) dbg[n + 1 + o] = b.sc[SC_TO + o];
    for (int j = 0; j <= r.acc; ++j) dbg[n + 1 + nout + j] = rec[j];
  }
  return st;
}

}  // extern "C"
