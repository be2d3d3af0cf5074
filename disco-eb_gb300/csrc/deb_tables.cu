// deb_tables.cu -- the perturbation path's input tables produced on the GPU:
// background densities, the RECFAST thermal history and the seven natural
// cubic splines, packed into the table blob of include/discoeb_gb300.h.
//
// One block of one warp per parameter set (deb_tables_core.cuh holds the
// per-set work).  The ionisation history is a sequential adaptive
// integration over the sampling intervals and runs on lane 0; everything
// indexed by a sample (neutrino momentum sums, HeII Saha fractions, sound
// speeds, the Romberg integrals of d tau / d a, the spline coefficients) is
// spread over the lanes.

#include <cuda_runtime.h>

#include <thread>
#include <vector>

#include "deb_tables_core.cuh"

namespace {

using debt::TParams;

__global__ void __launch_bounds__(32) tables_kernel(TParams P) {
  extern __shared__ double sh[];
  debt::produce_set(P, blockIdx.x, threadIdx.x, 32, sh);
}

// tau(a) of each set at the output scale factors: the tau_of_a spline of
// the blob in the A/B form (perturbations.py:975 via tables.tau_of_a)
__global__ void tau_out_kernel(const double* tables, int nset, int blob_len, const double* aexp, int nout, double* tau) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nset * nout) return;
  const int s = t / nout, o = t - s * nout;
  const double* b = tables + (long)s * blob_len;
  long p = DEB_HDR_LEN;
  for (int q = 0; q < 5; ++q) p += 3L * (long)b[20 + q];
  const int n = (int)b[25];
  tau[t] = debt::spl_ab(b + p, b + p + n, b + p + 2 * n, n, aexp[o]);
}

}  // namespace

extern "C" {

int deb_tau_of_a(const double* d_tables, int nset, int blob_len, const double* d_aexp, int nout, double* d_tau,
                 void* stream) {
  if (!d_tables || !d_aexp || !d_tau || nset < 0 || nout < 0 || blob_len <= DEB_HDR_LEN) return DEB_ERR_INVALID;
  const int tot = nset * nout;
  if (tot == 0) return DEB_OK;
  tau_out_kernel<<<(tot + 127) / 128, 128, 0, (cudaStream_t)stream>>>(d_tables, nset, blob_len, d_aexp, nout, d_tau);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

int deb_tables_blob_len(int num_thermo, int num_nu, int nqmax) {
  if (num_thermo < 4 || num_nu < 4 || nqmax < 1) return DEB_ERR_INVALID;
  const int sizes[7] = {num_thermo, num_thermo, num_nu, num_nu, num_thermo, num_thermo, num_thermo};
  long L = DEB_HDR_LEN + 2L * nqmax;
  for (int s = 0; s < 7; ++s) L += 3L * sizes[s] + 4L * (sizes[s] - 1) + (sizes[s] + 1) / 2;
  return (int)L;
}

}  // extern "C"

namespace {

// The producer's arguments, checked; the same for the device and the host entry.
int make_params(const deb_bg_cfg* cfg, const double* params, int nset, const double* consts, const double* grid,
                double* tables, int blob_len, int* status, TParams& P) {
  if (!cfg || !params || !consts || !grid || !tables || nset < 0) return DEB_ERR_INVALID;
  const int N = cfg->num_thermo, NN = cfg->num_nu;
  if (cfg->nq_bg < 1 || cfg->max_steps < 1 || !(cfg->amin > 0.0)) return DEB_ERR_INVALID;
  const int L = deb_tables_blob_len(N, NN, cfg->nqmax);
  if (L < 0 || blob_len != L) return DEB_ERR_INVALID;
  P = TParams{};
  P.params = params; P.nset = nset; P.consts = consts;
  // grid: a_nu [NN], log a_nu [NN], (q, w) background [2 nq_bg], (q, w) perturbations [2 nqmax],
  // a_thermo [N + 1], log a_thermo[1:] [N]
  const double* g = grid;
  P.a_nu = g; g += NN;
  P.la_nu = g; g += NN;
  P.qw_bg = g; g += 2 * cfg->nq_bg;
  P.qw = g; g += 2 * cfg->nqmax;
  P.a_th = g; g += N + 1;
  P.la_th = g;
  P.num_nu = NN; P.num_thermo = N; P.nq_bg = cfg->nq_bg; P.nqmax = cfg->nqmax; P.max_steps = cfg->max_steps;
  P.amin = cfg->amin; P.rtol = cfg->rtol; P.atol = cfg->atol;
  P.tables = tables; P.blob_len = blob_len; P.status = status;
  return DEB_OK;
}

// produce_set of every set on nthreads host threads (<= 0: one per hardware thread)
void host_sets(const TParams& P, int nthreads) {
  const int nset = P.nset;
  if (nset == 0) return;
  int nt = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > nset) nt = nset;
  const size_t nsh = (size_t)debt::tables_smem_doubles(P.num_thermo, P.num_nu);
  auto work = [&](int t) {
    std::vector<double> sh(nsh);
    for (int s = t; s < nset; s += nt) debt::produce_set(P, s, 0, 1, sh.data());
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

int deb_evolve_background(const deb_bg_cfg* cfg, const double* d_params, int nset, const double* d_consts,
                          const double* d_grid, double* d_tables, int blob_len, int* d_status, void* stream) {
  TParams P;
  const int rc = make_params(cfg, d_params, nset, d_consts, d_grid, d_tables, blob_len, d_status, P);
  if (rc) return rc;
  if (nset == 0) return DEB_OK;
  const size_t smem = (size_t)debt::tables_smem_doubles(P.num_thermo, P.num_nu) * sizeof(double);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(tables_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return DEB_ERR_INVALID;
  }
  tables_kernel<<<nset, 32, smem, (cudaStream_t)stream>>>(P);
  if (cudaGetLastError() != cudaSuccess) return DEB_ERR_CUDA;
  return DEB_OK;
}

int deb_evolve_background_host(const deb_bg_cfg* cfg, const double* params, int nset, const double* consts,
                               const double* grid, double* tables, int blob_len, int* status, int nthreads) {
  TParams P;
  const int rc = make_params(cfg, params, nset, consts, grid, tables, blob_len, status, P);
  if (rc) return rc;
  host_sets(P, nthreads);
  return DEB_OK;
}

int deb_evolve_background_frozen(const deb_bg_cfg* cfg, const double* d_params, int nset, const int* d_leader,
                                 const double* d_consts, const double* d_grid, double* d_steps, int step_cap,
                                 double* d_tables, int blob_len, int* d_status, void* stream) {
  TParams P;
  const int rc = make_params(cfg, d_params, nset, d_consts, d_grid, d_tables, blob_len, d_status, P);
  if (rc) return rc;
  if (!d_leader || !d_steps || step_cap < 1) return DEB_ERR_INVALID;
  if (nset == 0) return DEB_OK;
  P.leader = d_leader; P.steps = d_steps; P.step_cap = step_cap;
  const size_t smem = (size_t)debt::tables_smem_doubles(P.num_thermo, P.num_nu) * sizeof(double);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(tables_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return DEB_ERR_INVALID;
  }
  for (int phase = 1; phase <= 2; ++phase) {
    P.phase = phase;
    tables_kernel<<<nset, 32, smem, (cudaStream_t)stream>>>(P);
    if (cudaGetLastError() != cudaSuccess) return DEB_ERR_CUDA;
  }
  return DEB_OK;
}

int deb_evolve_background_frozen_host(const deb_bg_cfg* cfg, const double* params, int nset, const int* leader,
                                      const double* consts, const double* grid, double* steps, int step_cap,
                                      double* tables, int blob_len, int* status, int nthreads) {
  TParams P;
  const int rc = make_params(cfg, params, nset, consts, grid, tables, blob_len, status, P);
  if (rc) return rc;
  if (!leader || (steps && step_cap < 1)) return DEB_ERR_INVALID;
  if (nset == 0) return DEB_OK;
  std::vector<double> own;
  if (!steps) {
    step_cap = 16 * P.num_thermo;
    own.resize((size_t)nset * (size_t)(3 * P.num_thermo + 1 + 2 * step_cap));
    steps = own.data();
  }
  P.leader = leader; P.steps = steps; P.step_cap = step_cap;
  for (int phase = 1; phase <= 2; ++phase) {
    P.phase = phase;
    host_sets(P, nthreads);
  }
  return DEB_OK;
}

}  // extern "C"
