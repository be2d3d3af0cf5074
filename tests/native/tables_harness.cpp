// Host build of the GPU table producer's per-set code (test-only): every
// parameter set runs produce_set with one lane, so the C++ restatement can be
// checked against the Python host producer without a GPU.
#include <vector>

#include "../../disco-eb_gb300/csrc/deb_tables_core.cuh"

extern "C" int h_tables(const double* params, int nset, const double* consts, const double* grid, int num_thermo,
                        int num_nu, int nq_bg, int nqmax, int max_steps, double amin, double rtol, double atol,
                        double* tables, int blob_len, int* status) {
  debt::TParams P{};
  P.params = params; P.nset = nset; P.consts = consts;
  const double* g = grid;
  P.a_nu = g; g += num_nu;
  P.la_nu = g; g += num_nu;
  P.qw_bg = g; g += 2 * nq_bg;
  P.qw = g; g += 2 * nqmax;
  P.a_th = g; g += num_thermo + 1;
  P.la_th = g;
  P.num_nu = num_nu; P.num_thermo = num_thermo; P.nq_bg = nq_bg; P.nqmax = nqmax; P.max_steps = max_steps;
  P.amin = amin; P.rtol = rtol; P.atol = atol;
  P.tables = tables; P.blob_len = blob_len; P.status = status;
  std::vector<double> sh((size_t)debt::tables_smem_doubles(num_thermo, num_nu));
  for (int s = 0; s < nset; ++s) debt::produce_set(P, s, 0, 1, sh.data());
  return 0;
}
