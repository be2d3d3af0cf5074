// deb_adjoint.cu -- the discrete-adjoint kernel and its C ABI
// (deb_plan_create_adjoint, deb_adjoint in include/discoeb_gb300.h).
//
// One warp per work item (cotangent seed, k-mode), pulled from a device
// queue in order of recorded step counts, longest first.  A warp integrates
// its mode backwards segment by segment: it recomputes the segment's states
// from the checkpoint the recorded forward solve stored, then steps back
// through them (deb_adjoint.cuh).  The forward slot, the adjoint vectors and
// the segment states live in global memory (L2-resident for the warps in
// flight); the bilinear forms, coefficient tables and scalar accumulators in
// shared memory.  Replaces the reference's jax.jacfwd through diffrax
// (perturbations.py:765) by one reverse sweep per mode.

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "deb_adjoint.cuh"
#include "deb_internal.h"
#include "discoeb_gb300.h"

namespace {

__constant__ deb::Tab c_tab;
__constant__ deb::Rodas c_rodas;

struct AParams {
  const double* tables;      // [ncosmo, blob_len]
  const double* tables_pm;   // [ncosmo * 2 npar, blob_len]
  int ncosmo, npar, blob_len;
  const double* eps;         // [ncosmo, npar]
  const double* k;
  const int* cosmo;
  int nmode, nseed, nout;
  const double* tau_out;     // [ncosmo, nout]
  const double* tau_pm;      // [ncosmo * 2 npar, nout]
  const double* rec;
  int rec_len;
  const int* nrec;
  const double* ckpt;
  int ck_cap;
  const long long* ckoff;    // null: mode m's slots from m * ck_cap
  const int* ckstride;
  const double* gy;          // [nseed, nmode, nout, 20]
  double* gth;               // [nseed, nmode, npar]
  int* status;               // [nseed * nmode]
  double* ws;
  long wslot;
  int seg_cap;
  int* queue;
  const int* order;          // modes, most recorded steps first
  deb::Dims D;
  int shared_vectors;        // the NSHV hottest adjoint vectors in shared memory
};

// Warps per SM the register allocation must leave room for: a build-time
// option, 1 by default (255 registers).  Caps for 12 or 16 warps per SM were
// measured slower at nvar 1098 (spills), and the plan runs fewer warps than
// the registers allow anyway (the L2 fit).
#ifndef DEB_ADJ_MIN_WARPS_PER_SM
#define DEB_ADJ_MIN_WARPS_PER_SM 1
#endif

__global__ void __launch_bounds__(32, DEB_ADJ_MIN_WARPS_PER_SM) adjoint_kernel(AParams P) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const deb::Grp<32> gp{lane};
  const int n = P.D.n;
  deb::AWS<32> A;
  A.w.p = P.ws + (long)blockIdx.x * P.wslot;
  A.w.n = n;
  A.w.misc0 = deb::V_K0 * n;
  A.w.kp = A.w.p + deb::hot_len(P.D);
  A.w.dp = nullptr;
  A.av = A.w.p + deb::slot_len(P.D);
  A.seg = A.av + (long)deb::NAV * n;
  A.seg_cap = P.seg_cap;
  A.sc = smem;
  A.n = n;
  A.shv = P.shared_vectors ? smem + deb::SC_LEN : nullptr;
  const long items = (long)P.nmode * P.nseed;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(P.queue, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= items) break;
    const int j = q / P.nseed, seed = q - j * P.nseed;
    const int m = P.order ? P.order[j] : j;
    if (m < 0 || m >= P.nmode) continue;
    const long item = (long)seed * P.nmode + m;
    double* gth = P.gth + item * P.npar;
    const int ci = P.cosmo ? P.cosmo[m] : 0;
    const double km = P.k[m];
    int st = deb::ST_BAD_INPUT;
    if (ci >= 0 && ci < P.ncosmo && km > 0.0 && isfinite(km)) {
      deb::AdjItem it;
      it.blob0 = P.tables + (long)ci * P.blob_len;
      it.blobs = P.tables_pm + (long)ci * 2 * P.npar * P.blob_len;
      it.blob_len = P.blob_len;
      it.npar = P.npar;
      it.eps = P.eps + (long)ci * P.npar;
      it.tau0 = P.tau_out + (long)ci * P.nout;
      it.taus = P.tau_pm + (long)ci * 2 * P.npar * P.nout;
      it.rec = P.rec + (long)m * P.rec_len;
      it.nrec = P.nrec[m];
      it.ck = P.ckpt + (P.ckoff ? (long)P.ckoff[m] : (long)m * P.ck_cap) * n;
      it.ck_stride = it.nrec >= 1 ? P.ckstride[m] : 1;
      it.gy = P.gy + item * P.nout * deb::NFIELD;
      it.k = km;
      if (it.nrec >= 1 && it.nrec <= P.rec_len - 1)
        st = deb::adjoint_item<32>(gp, it, P.D, c_tab, c_rodas, P.nout, A, gth);
    }
    if (lane == 0) {
      P.status[item] = st;
      if (st != deb::ST_OK)
        for (int p = 0; p < P.npar; ++p) gth[p] = __longlong_as_double(0x7ff8000000000000LL);
    }
    __syncwarp();
  }
}

// order[rank(i)] = i by key descending (ties by index), as the replay orders its work
__global__ void rank_desc_adj_kernel(const int* key, int n, int* order) {
  __shared__ int tile[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ki = i < n ? key[i] : 0;
  int r = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int j = base + (int)threadIdx.x;
    tile[threadIdx.x] = j < n ? key[j] : 0;
    __syncthreads();
    const int lim = n - base < (int)blockDim.x ? n - base : (int)blockDim.x;
    for (int t = 0; t < lim; ++t) {
      const int kj = tile[t];
      r += (kj > ki) || (kj == ki && base + t < i);
    }
    __syncthreads();
  }
  if (i < n) order[r] = i;
}

std::mutex g_adj_mu;
unsigned long long g_adj_ctx[64] = {0};

// constant tables of this translation unit, once per context
int adj_upload_constants() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  unsigned long long ctx = deb_internal::current_ctx_id();
  if (ctx == 0) {
    if (cudaFree(nullptr) != cudaSuccess) return DEB_ERR_CUDA;
    ctx = deb_internal::current_ctx_id();
  }
  std::lock_guard<std::mutex> lock(g_adj_mu);
  if (dev >= 0 && dev < 64 && ctx != 0 && g_adj_ctx[dev] == ctx) return DEB_OK;
  deb::Tab T;
  deb::Rodas R;
  deb::fill_tables(T);
  deb::fill_rodas(R);
  const deb::LeadInv& L = deb::host_linv();
  if (!L.ok) return DEB_ERR_INVALID;
  if (cudaMemcpyToSymbol(c_tab, &T, sizeof(T)) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaMemcpyToSymbol(c_rodas, &R, sizeof(R)) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaMemcpyToSymbol(deb::c_linv, &L, sizeof(L)) != cudaSuccess) return DEB_ERR_CUDA;
  if (dev >= 0 && dev < 64) g_adj_ctx[dev] = ctx;
  return DEB_OK;
}

constexpr size_t kAdjSmem = deb::SC_LEN * sizeof(double);
// with the hottest adjoint vectors in shared memory as well
size_t adj_smem_bytes(const deb::Dims& D, bool shared_vectors) {
  return kAdjSmem + (shared_vectors ? (size_t)deb::NSHV * D.n * sizeof(double) : 0);
}

// the kernel's dynamic shared-memory limit, raised to at least bytes in the
// current context (never lowered, so plans of other sizes keep working)
std::mutex g_adj_smem_mu;
unsigned long long g_adj_smem_ctx[64] = {0};
size_t g_adj_smem_set[64] = {0};
int adj_raise_smem(size_t bytes) {
  if (bytes <= 48 * 1024) return DEB_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DEB_ERR_CUDA;
  const unsigned long long ctx = deb_internal::current_ctx_id();
  std::lock_guard<std::mutex> lk(g_adj_smem_mu);
  if (ctx != 0 && g_adj_smem_ctx[dev] == ctx && g_adj_smem_set[dev] >= bytes) return DEB_OK;
  const size_t want = (g_adj_smem_ctx[dev] == ctx && g_adj_smem_set[dev] > bytes) ? g_adj_smem_set[dev] : bytes;
  if (cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) != cudaSuccess)
    return DEB_ERR_CUDA;
  g_adj_smem_ctx[dev] = ctx;
  g_adj_smem_set[dev] = want;
  return DEB_OK;
}

}  // namespace

extern "C" {

int deb_plan_create_adjoint(const deb_dims* dims, int max_items, int seg_cap, deb_plan** out) {
  if (!dims || !out || max_items <= 0 || seg_cap < 1) return DEB_ERR_INVALID;
  *out = nullptr;
  // the lead rows' sources must not alias (lmax >= 5), the scratch block
  // holds up to 64 outputs and 64 momentum bins
  if (dims->lmaxg < 5 || dims->lmaxgp < 5 || dims->lmaxr < 5 || dims->lmaxnu < 3 || dims->nqmax < 1 ||
      dims->nqmax > 64 || dims->nout < 1 || dims->nout > 64)
    return DEB_ERR_INVALID;
  if (dims->lmaxg > deb::LMAX_TABLE || dims->lmaxgp > deb::LMAX_TABLE || dims->lmaxr > deb::LMAX_TABLE ||
      dims->lmaxnu > deb::LMAX_TABLE)
    return DEB_ERR_INVALID;
  if (dims->linear_solver != DEB_SOLVE_STRUCTURED || dims->return_full) return DEB_ERR_INVALID;
  int rc = adj_upload_constants();
  if (rc) return rc;
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel, 32, kAdjSmem) != cudaSuccess)
    return DEB_ERR_CUDA;
  if (per_sm < 1) return DEB_ERR_INVALID;
  {
    // the vectors a warp touches every step: its forward slot, the adjoint
    // vectors and one segment state
    const deb::Dims D = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
    const long hot = (deb::slot_len(D) + (long)(deb::NAV + 1) * D.n) * (long)sizeof(double);
    per_sm = deb_internal::l2_warps_per_sm(dev, nsm, hot, per_sm, 1.6);
  }
  // the hottest adjoint vectors in shared memory when that leaves the warps
  // per SM chosen above (the kernel's attribute is only ever raised)
  const deb::Dims Dm = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
  size_t smem = kAdjSmem;
  {
    int optin = 0, per_sm_bytes = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&per_sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const size_t want = adj_smem_bytes(Dm, true);
    if (want <= (size_t)optin && (long)per_sm * (long)(want + 1024) <= (long)per_sm_bytes &&
        adj_raise_smem(want) == DEB_OK)
      smem = want;
  }
  deb_plan* p = new deb_plan();
  p->adj_smem = (long)smem;
  p->adj_shared = smem > kAdjSmem ? 1 : 0;
  p->D = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
  p->nout = dims->nout;
  p->exec_mode = DEB_EXEC_WARP;
  p->max_modes = max_items;
  p->nsm = nsm;
  p->slot_len = deb::slot_len(p->D);
  p->adj = 1;
  p->adj_seg_cap = seg_cap;
  p->adj_wslot = p->slot_len + (long)(deb::NAV + seg_cap) * p->D.n;
  // warps in flight: what the SMs hold, capped by the items and by 32 GiB
  long warps = (long)nsm * per_sm;
  const long mem_cap = (32L << 30) / (p->adj_wslot * 8);
  if (warps > mem_cap) warps = mem_cap;
  if (warps > max_items) warps = max_items;
  if (warps < 1) { delete p; return DEB_ERR_NOMEM; }
  p->adj_warps = (int)warps;
  p->ws_bytes = (size_t)warps * p->adj_wslot * sizeof(double);
  if (cudaMalloc(&p->adj_ws, p->ws_bytes) != cudaSuccess) { delete p; return DEB_ERR_NOMEM; }
  if (cudaMalloc(&p->queue, sizeof(int) * 4) != cudaSuccess) { cudaFree(p->adj_ws); delete p; return DEB_ERR_NOMEM; }
  if (cudaMalloc(&p->order_dev, sizeof(int) * (size_t)max_items) != cudaSuccess) {
    cudaFree(p->adj_ws); cudaFree(p->queue); delete p; return DEB_ERR_NOMEM;
  }
  *out = p;
  return DEB_OK;
}

int deb_adjoint(deb_plan* p, const double* d_tables, const double* d_tables_pm, int ncosmo, int npar, int blob_len,
                const double* d_eps, const double* d_k, const int* d_cosmo_of_mode, int nmode,
                const double* d_tau_out, const double* d_tau_out_pm, const double* d_record, int rec_len,
                const int* d_nrec, const double* d_ckpt, int ck_cap, const long long* d_ckoff, const int* d_ckstride,
                const double* d_gy, int nseed, double* d_gtheta, int* d_status, void* stream) {
  if (!p || !p->adj || ncosmo <= 0 || npar < 1 || npar > 12 || nmode < 0 || nseed < 1 || blob_len <= deb::HDR_LEN)
    return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_tables_pm || !d_eps || !d_k || !d_tau_out || !d_tau_out_pm || !d_record || !d_nrec || !d_ckpt ||
      !d_ckstride || !d_gy || !d_gtheta || !d_status || rec_len < 2 || (!d_ckoff && ck_cap < 2))
    return DEB_ERR_INVALID;
  if ((long)nmode * nseed > p->max_modes || nmode > p->max_modes) return DEB_ERR_CAPACITY;
  int rc = adj_upload_constants();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  AParams P{};
  P.tables = d_tables; P.tables_pm = d_tables_pm; P.ncosmo = ncosmo; P.npar = npar; P.blob_len = blob_len;
  P.eps = d_eps; P.k = d_k; P.cosmo = d_cosmo_of_mode; P.nmode = nmode; P.nseed = nseed; P.nout = p->nout;
  P.tau_out = d_tau_out; P.tau_pm = d_tau_out_pm; P.rec = d_record; P.rec_len = rec_len; P.nrec = d_nrec;
  P.ckpt = d_ckpt; P.ck_cap = ck_cap; P.ckoff = d_ckoff; P.ckstride = d_ckstride; P.gy = d_gy; P.gth = d_gtheta; P.status = d_status;
  P.ws = p->adj_ws; P.wslot = p->adj_wslot; P.seg_cap = p->adj_seg_cap; P.queue = p->queue; P.order = p->order_dev;
  P.D = p->D;
  P.shared_vectors = p->adj_smem > (long)kAdjSmem;
  if (P.shared_vectors && adj_raise_smem((size_t)p->adj_smem) != DEB_OK) return DEB_ERR_CUDA;
  if (cudaMemsetAsync(p->queue, 0, sizeof(int), s) != cudaSuccess) return DEB_ERR_CUDA;
  rank_desc_adj_kernel<<<(nmode + 255) / 256, 256, 0, s>>>(d_nrec, nmode, p->order_dev);
  const long items = (long)nmode * nseed;
  const int blocks = (int)(items < p->adj_warps ? items : p->adj_warps);
  adjoint_kernel<<<blocks, 32, (size_t)p->adj_smem, s>>>(P);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

}  // extern "C"
