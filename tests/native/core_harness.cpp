// core_harness.cpp -- TEST-ONLY host build of the kernel's per-mode logic.
//
// Compiles disco-eb_gb300/csrc/deb_core.cuh (the code the CUDA kernel runs,
// one thread per mode) for the CPU with a stride-1 workspace, so the tests
// can compare the kernel's structured factorization, RHS and step control
// against the oracle without a GPU.  It is never part of the library.
#include <cstring>
#include <vector>
#include <limits>
#include "../../disco-eb_gb300/csrc/deb_core.cuh"

using namespace deb;

namespace {
struct Ctx {
  Dims D; Cosmo c; ModeConst m; Tab T; Rodas R; std::vector<double> buf, dbuf; WS<1> w;
};
const Grp<1> GP{0};
bool setup(Ctx& x, const double* blob, int blob_len, const int* dims, double k, bool dense) {
  x.D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  if (!load_cosmo(blob, blob_len, x.c)) return false;
  mode_const(x.c, k, x.m);
  fill_tables(x.T); fill_rodas(x.R);
  // the one-thread-per-mode layout interleaves 32 modes; lane 0 is used here
  x.buf.assign(slot_len(x.D) * 32, 0.0);
  x.dbuf.assign(dense ? dense_len(x.D) * 32 : 1, 0.0);
  x.w.p = x.buf.data(); x.w.n = x.D.n; x.w.misc0 = V_K0 * x.D.n;
  x.w.kp = x.w.p + hot_len(x.D) * 32;
  x.w.dp = x.dbuf.data();
  for (int i = 0; i < x.D.nq; ++i) {
    double q = x.c.q[i];
    x.w.m(M_Q + Q_DLF * x.D.nq + i) = -q / (1.0 + std::exp(-q));
    x.w.m(M_Q + Q_AMQ * x.D.nq + i) = x.m.amnu / q;
  }
  return true;
}
}  // namespace

extern "C" {

// f(tau, y) and d f / d a
int h_rhs(const double* blob, int blob_len, const int* dims, double k, double tau, const double* y, double* f, double* jc0) {
  Ctx x; if (!setup(x, blob, blob_len, dims, k, false)) return -2;
  for (int j = 0; j < x.D.n; ++j) x.w.v(V_Y, j) = y[j];
  rhs<Dual, 1>(GP, x.c, x.m, x.D, x.T, tau, x.w, V_Y, (V_K0 + 1), V_JC0);
  for (int j = 0; j < x.D.n; ++j) { f[j] = x.w.v((V_K0 + 1), j); jc0[j] = x.w.v(V_JC0, j); }
  rhs<double, 1>(GP, x.c, x.m, x.D, x.T, tau, x.w, V_Y, V_U, -1);
  for (int j = 0; j < x.D.n; ++j) if (x.w.v(V_U, j) != f[j] && !(f[j] != f[j])) return -10;
  return 0;
}

// x = W^{-1} b with W = I/(gamma dt) - J(tau, y), structured (dense=0) or dense LU (dense=1)
int h_solve_W(const double* blob, int blob_len, const int* dims, double k, double tau, const double* y, double dt,
              const double* b, double* xout, int dense) {
  Ctx x; if (!setup(x, blob, blob_len, dims, k, dense != 0)) return -2;
  const int n = x.D.n;
  for (int j = 0; j < n; ++j) x.w.v(V_Y, j) = y[j];
  rhs<Dual, 1>(GP, x.c, x.m, x.D, x.T, tau, x.w, V_Y, (V_K0 + 1), V_JC0);
  Bg<double> g; background<double>(x.c, x.m, y[0], g);
  const double d = 1.0 / (dt * x.R.gamma);
  factor_W<1>(GP, x.c, x.m, x.D, x.T, x.w, d, tau, g);
  for (int j = 0; j < n; ++j) x.w.v(V_K0, j) = b[j];
  if (dense) {
    dense_factor<1>(GP, x.m, x.D, x.T, x.w, d, tau, g);
    dense_solve<1>(GP, x.D, x.w, V_K0);
  } else {
    solve_W<1>(GP, x.m, x.D, x.w, g.aH, V_K0);
  }
  for (int j = 0; j < n; ++j) xout[j] = x.w.v(V_K0, j);
  return 0;
}

int h_start(const double* blob, int blob_len, const int* dims, double k, double* tau_start, double* y0) {
  Ctx x; if (!setup(x, blob, blob_len, dims, k, false)) return -2;
  *tau_start = start_time(x.c, x.m);
  initial_conditions<1>(GP, x.c, x.m, x.D, 0.99 * *tau_start, x.w, V_Y);
  for (int j = 0; j < x.D.n; ++j) y0[j] = x.w.v(V_Y, j);
  return 0;
}

// spline evaluation as the kernel does it (FP32 search + FP64 fix-up, polynomial form)
int h_spline(const double* blob, int blob_len, int which, const double* x, int nx, double* out, int* idx) {
  Cosmo c; if (!load_cosmo(blob, blob_len, c)) return -2;
  if (which < 0 || which >= NSPL) return -3;
  for (int i = 0; i < nx; ++i) { out[i] = spl_eval(c.sp[which], x[i]); idx[i] = spl_locate(c.sp[which], x[i]); }
  return 0;
}

// record / replay, mirroring the kernel's work items (item = set * nmode + mode)
int h_solve_rr(const double* tables, int ncosmo, int nset, int blob_len, const double* kmodes, const int* cosmo,
               int nmode, const double* tau_out, int nout, const int* dims, const double* cfg, int max_steps,
               double* rec, int rec_len, int* nrec, int record, int replay, double* y_out, int* stats) {
  const Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  Ctl ctl;
  ctl.rtol = cfg[0]; ctl.atol = cfg[1];
  ctl.b1 = (cfg[3] + cfg[2] + cfg[4]) / cfg[7]; ctl.b2 = -(cfg[2] + 2.0 * cfg[4]) / cfg[7]; ctl.b3 = cfg[4] / cfg[7];
  ctl.fmax = cfg[5]; ctl.fmin = cfg[6]; ctl.safety = cfg[8]; ctl.hist_on_reject = (int)cfg[9];
  ctl.max_steps = max_steps; ctl.dense = 0; ctl.return_full = 0; ctl.nout = nout;
  ctl.record = record; ctl.replay = replay; ctl.step_ts = (int)cfg[10];
  for (int it = 0; it < nmode * nset; ++it) {
    const int mi = it % nmode, set = it / nmode;
    const int ci = (cosmo ? cosmo[mi] : 0) * nset + set;
    Ctx x; if (!setup(x, tables + (long)ci * blob_len, blob_len, dims, kmodes[mi], false)) return -2;
    double* dst = y_out + (long)it * nout * 20;
    for (int i = 0; i < nout * 20; ++i) dst[i] = std::numeric_limits<double>::quiet_NaN();
    Run r;
    r.rec = rec + (long)mi * rec_len; r.rec_cap = rec_len - 1; r.nrec = replay ? nrec[mi] : 0;
    mode_begin<1>(GP, x.c, x.m, x.D, ctl, x.w, tau_out + (long)ci * nout, r);
    while (mode_step<1>(GP, x.c, x.m, x.D, x.T, x.R, ctl, x.w, tau_out + (long)ci * nout, dst, 1, r)) {}
    stats[3 * it] = r.status; stats[3 * it + 1] = r.acc; stats[3 * it + 2] = r.rej;
    if (record) nrec[mi] = r.status == ST_OK ? r.acc : 0;
  }
  return 0;
}

// full per-mode solve with the kernel's driver, sequential over modes
int h_solve(const double* tables, int ncosmo, int blob_len, const double* kmodes, const int* cosmo, int nmode,
            const double* tau_out, int nout, const int* dims, const double* cfg, int max_steps, int return_full,
            int dense, double* y_out, int* stats) {
  const Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  Ctl ctl;
  ctl.rtol = cfg[0]; ctl.atol = cfg[1];
  ctl.b1 = (cfg[3] + cfg[2] + cfg[4]) / cfg[7]; ctl.b2 = -(cfg[2] + 2.0 * cfg[4]) / cfg[7]; ctl.b3 = cfg[4] / cfg[7];
  ctl.fmax = cfg[5]; ctl.fmin = cfg[6]; ctl.safety = cfg[8]; ctl.hist_on_reject = (int)cfg[9];
  ctl.max_steps = max_steps; ctl.dense = dense; ctl.return_full = return_full; ctl.nout = nout;
  ctl.record = 0; ctl.replay = 0; ctl.step_ts = (int)cfg[10];
  const int osz = return_full ? D.n : 20;
  for (int mi = 0; mi < nmode; ++mi) {
    const int ci = cosmo ? cosmo[mi] : 0;
    Ctx x; if (!setup(x, tables + (long)ci * blob_len, blob_len, dims, kmodes[mi], dense != 0)) return -2;
    double* dst = y_out + (long)mi * nout * osz;
    for (int i = 0; i < nout * osz; ++i) dst[i] = std::numeric_limits<double>::quiet_NaN();
    Run r;
    r.rec = nullptr; r.rec_cap = 0; r.nrec = 0;
    mode_begin<1>(GP, x.c, x.m, x.D, ctl, x.w, tau_out + (long)ci * nout, r);
    while (mode_step<1>(GP, x.c, x.m, x.D, x.T, x.R, ctl, x.w, tau_out + (long)ci * nout, dst, 1, r)) {}
    stats[3 * mi] = r.status; stats[3 * mi + 1] = r.acc; stats[3 * mi + 2] = r.rej;
  }
  return 0;
}

// groups of batch_size consecutive modes sharing one step sequence (the
// kernel's group driver); nmode must be a multiple of batch_size
int h_solve_grouped(const double* tables, int ncosmo, int blob_len, const double* kmodes, const int* cosmo, int nmode,
                    const double* tau_out, int nout, const int* dims, const double* cfg, int max_steps, int batch_size,
                    double* y_out, int* stats) {
  if (batch_size < 1 || batch_size > 32 || nmode % batch_size) return -1;
  Ctl ctl;
  ctl.rtol = cfg[0]; ctl.atol = cfg[1];
  ctl.b1 = (cfg[3] + cfg[2] + cfg[4]) / cfg[7]; ctl.b2 = -(cfg[2] + 2.0 * cfg[4]) / cfg[7]; ctl.b3 = cfg[4] / cfg[7];
  ctl.fmax = cfg[5]; ctl.fmin = cfg[6]; ctl.safety = cfg[8]; ctl.hist_on_reject = (int)cfg[9];
  ctl.max_steps = max_steps; ctl.dense = 0; ctl.return_full = 0; ctl.nout = nout;
  ctl.record = 0; ctl.replay = 0; ctl.step_ts = (int)cfg[10];
  const int B = batch_size;
  Tab T; Rodas R; fill_tables(T); fill_rodas(R);
  const Dims D = make_dims(dims[0], dims[1], dims[2], dims[3], dims[4]);
  for (int m0 = 0; m0 < nmode; m0 += B) {
    std::vector<Ctx> xs(B);
    const int ci = cosmo ? cosmo[m0] : 0;
    for (int b = 0; b < B; ++b) {
      if ((cosmo ? cosmo[m0 + b] : 0) != ci) return -3;
      if (!setup(xs[b], tables + (long)ci * blob_len, blob_len, dims, kmodes[m0 + b], false)) return -2;
      double* dst = y_out + (long)(m0 + b) * nout * 20;
      for (int i = 0; i < nout * 20; ++i) dst[i] = std::numeric_limits<double>::quiet_NaN();
    }
    auto ctx = [&](int b) {
      ModeCtx<1> x{xs[b].c, xs[b].m, xs[b].w, tau_out + (long)ci * nout, y_out + (long)(m0 + b) * nout * 20};
      return x;
    };
    Run r;
    r.rec = nullptr; r.rec_cap = 0; r.nrec = 0;
    group_solve<1>(GP, D, T, R, ctl, B, ctx, 1, r);
    for (int b = 0; b < B; ++b) { stats[3 * (m0 + b)] = r.status; stats[3 * (m0 + b) + 1] = r.acc; stats[3 * (m0 + b) + 2] = r.rej; }
  }
  return 0;
}

}  // extern "C"
