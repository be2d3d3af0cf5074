// deb_solver.cu -- CUDA kernels and the C ABI of include/discoeb_gb300.h.
//
// Execution model: one persistent grid sized to the device (blocks of 128
// threads, a few blocks per SM); every thread owns one workspace slot and
// pulls k-modes from a device-side queue (one atomicAdd per mode).  A mode is
// integrated to completion by its thread, then the thread takes the next
// queued mode, so modes with very different step counts (and modes of
// different cosmologies) share the launch without lock-step waste.  Each
// warp keeps its 32 slots interleaved in global memory (element e of lane l
// at base + 32 e + l), so every vector access of the warp is one coalesced
// 256-byte transaction.
//
// Replaces jax.vmap(evolve_one_mode) of perturbations.py:980-987 (and the
// lock-step while_loop it compiles to) for one GPU.

#include <cuda_runtime.h>

#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <mutex>

#include "deb_core.cuh"
#include "deb_internal.h"
#include "discoeb_gb300.h"

namespace {

constexpr int kBlock = 128;
// one-warp blocks resident per SM: the warp kernel is compiled with up to 255
// registers per thread (launch bound 32), 8 such warps fill the register file
constexpr int kMaxWarpBlocksPerSM = 8;

__constant__ deb::Tab c_tab;
__constant__ deb::Rodas c_rodas;

struct KParams {
  const double* tables;
  int ncosmo, blob_len;
  const double* k;
  const int* cosmo;
  int nmode;
  const double* tau_out;
  double* y_out;
  int* status;
  int* steps;
  double* ws;         // lane mode: interleaved slots; warp mode: slots unless smem == 1
  double* kws;        // warp mode with smem == 1 and stage vectors outside shared memory: [warps, 8 n]
  long hot_len;       // warp mode: doubles of the slot in shared memory
  double* dws;        // dense matrices (dense path only)
  long slot_len, dense_len;
  int smem;           // warp mode: slots live in dynamic shared memory
  int* queue;
  // record / replay of the accepted step times (frozen-step tangents)
  double* rec;        // [nmode, rec_len]
  int rec_len;
  int* nrec;          // [nmode]
  int nset;           // replay: table sets per cosmology; output item = set * nmode + mode
  // queue order: queue position q takes mode order[q] (forward) or mode
  // order[q / nset], set q % nset (replay); null = index order
  const int* order;
  // record with checkpoints: ckpt [nmode, ck_cap, n] or, with ckoff, mode m's
  // ckcap[m] slots from slot ckoff[m] of one pool; ckstride [nmode]
  double* ckpt;
  int ck_cap;
  int* ckstride;
  const long long* ckoff;
  const int* ckcaps;
  deb::Ctl ctl;
  deb::Dims D;
};

// Map queue position q to (mode m, table set, output item oi = set * nmode
// + m), validate it and load its cosmology; fills NaN outputs and the run's
// record pointers.  Same on every lane.  Returns false for an item to skip.
__device__ bool prepare_mode(const KParams& P, int q, deb::Cosmo& c, deb::ModeConst& mc, const double*& tau_out,
                             double*& yout, deb::Run& run, int& oi, int lane, int G) {
  const int osz = P.ctl.return_full ? P.D.n : DEB_NOUT_FIELDS;
  int m, set;
  if (P.ctl.replay) {
    if (P.order) { const int j = q / P.nset; set = q - j * P.nset; m = P.order[j]; }
    else { m = q % P.nmode; set = q / P.nmode; }
  } else {
    set = 0;
    m = P.order ? P.order[q] : q;
  }
  if (m < 0 || m >= P.nmode) return false;   // not a permutation: nothing to do for this position
  const int w = set * P.nmode + m;
  oi = w;
  const int ci = P.cosmo ? P.cosmo[m] : 0;
  const double k = P.k[m];
  double* dst = P.y_out + (long)w * P.ctl.nout * osz;
  for (int i = lane; i < P.ctl.nout * osz; i += G) dst[i] = __longlong_as_double(0x7ff8000000000000LL);
  bool ok = ci >= 0 && ci < P.ncosmo && k > 0.0 && isfinite(k);
  const int ti = ci * P.nset + set;
  if (ok) ok = deb::load_cosmo(P.tables + (long)ti * P.blob_len, P.blob_len, c) && c.nq == P.D.nq;
  run.rec = P.rec ? P.rec + (long)m * P.rec_len : nullptr;
  run.rec_cap = P.rec_len - 1;
  // an odd or too small per-mode capacity would break the thinning's pairing
  // of slots: it is taken down to even, at least 2
  const long ck_slot = P.ckoff ? (long)P.ckoff[m] : (long)m * P.ck_cap;
  const int ck_cap = P.ckoff ? ((P.ckcaps[m] & ~1) < 2 ? 2 : (P.ckcaps[m] & ~1)) : P.ck_cap;
  run.ck = (P.ctl.record && P.ckpt) ? P.ckpt + ck_slot * P.D.n : nullptr;
  run.ck_cap = ck_cap;
  run.ck_stride = 1;
  run.nrec = (P.ctl.replay && P.nrec) ? P.nrec[m] : 0;
  if (ok && P.ctl.replay) ok = run.nrec >= 1 && run.nrec <= run.rec_cap;
  if (!ok) {
    if (lane == 0) {
      P.status[w] = deb::ST_BAD_INPUT;
      if (P.steps) { P.steps[2 * w] = 0; P.steps[2 * w + 1] = 0; }
      if (P.ctl.record && P.nrec) P.nrec[m] = 0;
    }
    return false;
  }
  deb::mode_const(c, k, mc);
  tau_out = P.tau_out + (long)ti * P.ctl.nout;
  yout = dst;
  return true;
}

// One thread per mode: 32 modes per warp, slots interleaved in global memory.
__global__ void __launch_bounds__(kBlock) forward_lane_kernel(KParams P) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const long warp = tid >> 5;
  deb::WS<1> w;
  w.p = P.ws + warp * 32 * P.slot_len + lane;
  w.n = P.D.n;
  w.misc0 = deb::V_K0 * P.D.n;
  w.kp = w.p + (long)deb::hot_len(P.D) * 32;
  w.dp = P.dws ? P.dws + warp * 32 * P.dense_len + lane : nullptr;
  const deb::Grp<1> gp{0};
  int mode = -1;   // output item of the current mode
  deb::Cosmo c;
  deb::ModeConst mc;
  deb::Run run;
  const double* tau_out = nullptr;
  double* yout = nullptr;
  auto fetch = [&]() -> bool {
    for (;;) {
      const int q = atomicAdd(P.queue, 1);
      if (q >= P.nmode * P.nset) return false;
      if (!prepare_mode(P, q, c, mc, tau_out, yout, run, mode, 0, 1)) continue;
      deb::mode_begin<1>(gp, c, mc, P.D, P.ctl, w, tau_out, run);
      return true;
    }
  };
  bool active = fetch();
  while (__any_sync(0xffffffffu, active)) {
    if (active) {
      const bool more = deb::mode_step<1>(gp, c, mc, P.D, c_tab, c_rodas, P.ctl, w, tau_out, yout, 1, run);
      if (!more) {
        P.status[mode] = run.status;
        if (P.steps) { P.steps[2 * mode] = run.acc; P.steps[2 * mode + 1] = run.rej; }
        if (P.ctl.record && P.nrec) P.nrec[mode] = run.status == deb::ST_OK ? run.acc : 0;   // record: set 0, item = mode
        if (P.ctl.record && P.ckstride) P.ckstride[mode] = run.ck_stride;
        active = fetch();
      }
    }
  }
}

// One warp per mode: the mode's vectors and MISC block in shared memory.
// Warps per SM the record kernel's registers must leave room for: a
// build-time option, 1 by default (~245 registers, 8 warps per SM); 12 or 16
// were measured no faster at nvar 1098.
#ifndef DEB_FWD_MIN_WARPS_PER_SM
#define DEB_FWD_MIN_WARPS_PER_SM 1
#endif

__global__ void __launch_bounds__(32, DEB_FWD_MIN_WARPS_PER_SM) forward_warp_kernel(KParams P) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const long gwarp = blockIdx.x;
  deb::WS<32> w;
  w.p = P.smem ? smem : P.ws + gwarp * P.slot_len;
  w.n = P.D.n;
  w.misc0 = deb::V_K0 * P.D.n;
  // stage vectors after MISC in the same slot, or in their own global region
  w.kp = (P.smem && P.kws) ? P.kws + gwarp * deb::stage_len(P.D) : w.p + deb::hot_len(P.D);
  w.dp = P.dws ? P.dws + gwarp * P.dense_len : nullptr;
  const deb::Grp<32> gp{lane};
  deb::Cosmo c;
  deb::ModeConst mc;
  deb::Run run;
  const double* tau_out = nullptr;
  double* yout = nullptr;
  for (;;) {
    int q = 0, m = 0;
    if (lane == 0) q = atomicAdd(P.queue, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= P.nmode * P.nset) break;
    if (!prepare_mode(P, q, c, mc, tau_out, yout, run, m, lane, 32)) continue;
    deb::mode_begin<32>(gp, c, mc, P.D, P.ctl, w, tau_out, run);
    while (deb::mode_step<32>(gp, c, mc, P.D, c_tab, c_rodas, P.ctl, w, tau_out, yout, 1, run)) {}
    if (lane == 0) {
      P.status[m] = run.status;
      if (P.steps) { P.steps[2 * m] = run.acc; P.steps[2 * m + 1] = run.rej; }
      if (P.ctl.record && P.nrec) P.nrec[m] = run.status == deb::ST_OK ? run.acc : 0;
      if (P.ctl.record && P.ckstride) P.ckstride[m] = run.ck_stride;
    }
    __syncwarp();
  }
}

// Groups of B consecutive modes sharing one step sequence (the reference's
// batched variant): one warp per group, taken from the queue; the group's B
// slots live in global memory and the warp steps its modes one after the
// other inside each shared step (deb::group_solve).  A group whose modes are
// not all valid or not all of one cosmology is marked BAD_INPUT.
__global__ void __launch_bounds__(32) forward_group_kernel(KParams P, int B) {
  const int lane = threadIdx.x & 31;
  const long gwarp = blockIdx.x;
  const deb::Grp<32> gp{lane};
  const int osz = P.ctl.return_full ? P.D.n : DEB_NOUT_FIELDS;
  const int ngroup = P.nmode / B;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(P.queue, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= ngroup) break;
    const int m0 = q * B;
    const int ci = P.cosmo ? P.cosmo[m0] : 0;
    bool ok = ci >= 0 && ci < P.ncosmo;
    for (int b = 0; b < B; ++b) {
      const int m = m0 + b;
      const double k = P.k[m];
      ok = ok && (P.cosmo ? P.cosmo[m] : 0) == ci && k > 0.0 && isfinite(k);
      double* dst = P.y_out + (long)m * P.ctl.nout * osz;
      for (int i = lane; i < P.ctl.nout * osz; i += 32) dst[i] = __longlong_as_double(0x7ff8000000000000LL);
    }
    deb::Cosmo c0;
    if (ok) ok = deb::load_cosmo(P.tables + (long)ci * P.blob_len, P.blob_len, c0) && c0.nq == P.D.nq;
    deb::Run run;
    run.rec = nullptr; run.rec_cap = 0; run.nrec = 0; run.acc = 0; run.rej = 0; run.status = deb::ST_BAD_INPUT;
    if (ok) {
      const double* tau_out = P.tau_out + (long)ci * P.ctl.nout;
      auto ctx = [&](int b) {
        deb::ModeCtx<32> x;
        x.c = c0;
        deb::mode_const(c0, P.k[m0 + b], x.m);
        x.w.p = P.ws + (gwarp * B + b) * P.slot_len;
        x.w.n = P.D.n;
        x.w.misc0 = deb::V_K0 * P.D.n;
        x.w.kp = x.w.p + deb::hot_len(P.D);
        x.w.dp = nullptr;
        x.tau_out = tau_out;
        x.yout = P.y_out + (long)(m0 + b) * P.ctl.nout * osz;
        return x;
      };
      deb::group_solve<32>(gp, P.D, c_tab, c_rodas, P.ctl, B, ctx, 1, run);
    }
    if (lane == 0)
      for (int b = 0; b < B; ++b) {
        const int m = m0 + b;
        P.status[m] = run.status;
        if (P.steps) { P.steps[2 * m] = run.acc; P.steps[2 * m + 1] = run.rej; }
      }
    __syncwarp();
  }
}

__global__ void power_kernel(const double* tables, int ncosmo, int blob_len, const double* k, const int* cosmo, int nmode,
                             int nout, const double* y, int stride, int idx, double* P) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nmode * nout) return;
  const int m = (int)(t / nout);
  const int ci = cosmo ? cosmo[m] : 0;
  if (ci < 0 || ci >= ncosmo) { P[t] = __longlong_as_double(0x7ff8000000000000LL); return; }
  const double* b = tables + (long)ci * blob_len;
  const double As = b[deb::H_AS], ns = b[deb::H_NS], kp = b[deb::H_KP];
  const double km = k[m];
  const double v = y[t * stride + idx];
  // get_power, perturbations.py:1123
  P[t] = 2.0 * M_PI * M_PI * As * pow(km / kp, ns - 1.0) * pow(km, -3.0) * v * v;
}

// order[rank(i)] = i with modes ranked by key descending, ties by index:
// the replay hands the modes with the most recorded steps out first, so the
// launch does not end on a long mode started last.  O(n^2) compares through
// shared-memory tiles; n is a few ten thousand at most.
__global__ void rank_desc_kernel(const int* key, int n, int* order) {
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

// Independent FMA chains: 8 per thread, long enough to be issue-bound.
__global__ void fp64_peak_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// Per-device state that lives in a CUDA context (constant tables, kernel
// attributes) is remembered together with the id of the context it was set
// in: after cudaDeviceReset (or with another context current) the id
// differs and the state is set again.  Guarded by g_state_mu.
std::mutex g_state_mu;
unsigned long long g_consts_ctx[64] = {0};
unsigned long long g_attr_ctx[64] = {0};
// largest dynamic shared memory size set on forward_warp_kernel, per device
long g_warp_smem_attr[64] = {0};

int upload_constants() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  unsigned long long ctx = deb_internal::current_ctx_id();
  if (ctx == 0) {
    // no context current on this thread yet: let the runtime make the
    // device's primary context current, then ask again
    if (cudaFree(nullptr) != cudaSuccess) return DEB_ERR_CUDA;
    ctx = deb_internal::current_ctx_id();
  }
  std::lock_guard<std::mutex> lock(g_state_mu);
  if (dev >= 0 && dev < 64 && ctx != 0 && g_consts_ctx[dev] == ctx) return DEB_OK;
  deb::Tab T;
  deb::Rodas R;
  deb::fill_tables(T);
  deb::fill_rodas(R);
  if (cudaMemcpyToSymbol(c_tab, &T, sizeof(T)) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaMemcpyToSymbol(c_rodas, &R, sizeof(R)) != cudaSuccess) return DEB_ERR_CUDA;
  if (dev >= 0 && dev < 64) g_consts_ctx[dev] = ctx;
  return DEB_OK;
}

// Raise forward_warp_kernel's dynamic shared memory limit to at least
// `bytes` in the current context (only ever raised, so that plans made
// earlier with a larger slot stay launchable).
int ensure_warp_smem(int dev, long bytes) {
  const unsigned long long ctx = deb_internal::current_ctx_id();
  std::lock_guard<std::mutex> lock(g_state_mu);
  const bool known = dev >= 0 && dev < 64 && ctx != 0 && g_attr_ctx[dev] == ctx;
  if (known && g_warp_smem_attr[dev] >= bytes) return DEB_OK;
  const long want = known && g_warp_smem_attr[dev] > bytes ? g_warp_smem_attr[dev] : bytes;
  if (cudaFuncSetAttribute(forward_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) != cudaSuccess)
    return DEB_ERR_CUDA;
  if (dev >= 0 && dev < 64) { g_attr_ctx[dev] = ctx; g_warp_smem_attr[dev] = want; }
  return DEB_OK;
}

}  // namespace


extern "C" {

int deb_version(void) { return 1; }

const char* deb_error_string(int code) {
  switch (code) {
    case DEB_OK: return "ok";
    case DEB_ERR_INVALID: return "invalid argument";
    case DEB_ERR_TABLES: return "inconsistent table blob";
    case DEB_ERR_CUDA: return "CUDA runtime error";
    case DEB_ERR_NOMEM: return "device allocation failed";
    case DEB_ERR_CAPACITY: return "plan capacity exceeded";
    case DEB_ERR_STATIC_SCRATCH: return "one mode's solver state exceeds the static scratch array (DEB_STATIC_SCRATCH_BYTES)";
    default: return "unknown error";
  }
}

int deb_nvar(const deb_dims* d) {
  if (!d) return DEB_ERR_INVALID;
  return deb::make_dims(d->lmaxg, d->lmaxgp, d->lmaxr, d->lmaxnu, d->nqmax).n;
}

int deb_plan_create(const deb_dims* dims, int max_modes, deb_plan** out) {
  return deb_plan_create_ex(dims, max_modes, nullptr, out);
}

int deb_plan_create_ex(const deb_dims* dims, int max_modes, const deb_launch_cfg* lc, deb_plan** out) {
  if (!dims || !out || max_modes <= 0) return DEB_ERR_INVALID;
  const int stage_where = lc ? lc->stage_vectors : DEB_STAGE_AUTO;
  const int mps_cap = lc ? lc->modes_per_sm : 0;
  if (stage_where < DEB_STAGE_AUTO || stage_where > DEB_STAGE_ALL_GLOBAL || mps_cap < 0) return DEB_ERR_INVALID;
  *out = nullptr;
  if (dims->lmaxg < 3 || dims->lmaxgp < 3 || dims->lmaxr < 3 || dims->lmaxnu < 3 || dims->nqmax < 1 || dims->nout < 1)
    return DEB_ERR_INVALID;
  if (dims->lmaxg > deb::LMAX_TABLE || dims->lmaxgp > deb::LMAX_TABLE || dims->lmaxr > deb::LMAX_TABLE ||
      dims->lmaxnu > deb::LMAX_TABLE)
    return DEB_ERR_INVALID;
  if (dims->linear_solver != DEB_SOLVE_STRUCTURED && dims->linear_solver != DEB_SOLVE_DENSE) return DEB_ERR_INVALID;
  if (dims->exec_mode < DEB_EXEC_AUTO || dims->exec_mode > DEB_EXEC_WARP) return DEB_ERR_INVALID;
  int rc = upload_constants();
  if (rc) return rc;
  int dev = 0, nsm = 0, smem_optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return DEB_ERR_CUDA;
  deb_plan* p = new deb_plan();
  p->D = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
  p->dense = dims->linear_solver == DEB_SOLVE_DENSE;
  p->return_full = dims->return_full;
  p->nout = dims->nout;
  p->max_modes = max_modes;
  p->nsm = nsm;
  p->slot_len = deb::slot_len(p->D);
  p->dense_len = p->dense ? deb::dense_len(p->D) : 0;
  const long per_slot = p->slot_len + p->dense_len;
  // execution mode: lane per mode once the batch fills every SM sub-partition
  // with >= 1 warp of modes, else warp per mode
  int mode = dims->exec_mode;
  if (mode == DEB_EXEC_AUTO) mode = DEB_EXEC_WARP;
  p->exec_mode = mode;
  // slot counts are capped at 16 GiB of workspace
  const long mem_cap = (16L << 30) / (per_slot * 8);
  long nslots;
  if (mode == DEB_EXEC_LANE) {
    long cap = (long)nsm * 4 * kBlock;
    if (cap > mem_cap) cap = (mem_cap / 32) * 32;
    if (cap < 32) cap = 32;
    long want = ((long)max_modes + 31) / 32 * 32;
    long ns = want < cap ? want : cap;
    p->lane_blocks = (int)((ns + kBlock - 1) / kBlock);
    p->lane_slots = p->lane_blocks * kBlock;
    nslots = p->lane_slots;
  } else {
    // a mode's whole slot in shared memory when 2 modes fit per SM, else only
    // the hot part (vectors before k1 + MISC) with k1..k8 in global memory
    // (L2-resident, lane-strided coalesced access)
    const long full_bytes = p->slot_len * 8, hot_bytes = deb::hot_len(p->D) * 8;
    const long sm_bytes = 228L * 1024;
    long smem_bytes;
    const bool full_fits = sm_bytes / (full_bytes + 1024) >= 2 && full_bytes <= smem_optin;
    bool k_global;
    if (stage_where == DEB_STAGE_SHARED) {
      if (full_bytes > smem_optin) { delete p; return DEB_ERR_INVALID; }
      k_global = false;
    } else if (stage_where == DEB_STAGE_GLOBAL) {
      k_global = true;
    } else {
      k_global = !full_fits;
    }
    smem_bytes = k_global ? hot_bytes : full_bytes;
    p->warp_k_global = k_global ? 1 : 0;
    p->warp_smem = smem_bytes <= smem_optin && stage_where != DEB_STAGE_ALL_GLOBAL;
    if (!p->warp_smem) p->warp_k_global = 0;
    p->warp_block_warps = 1;
    // blocks (= modes in flight) per SM limited by shared memory, by
    // registers (the kernel's own occupancy without shared memory: 8 one-warp
    // blocks at 255 registers per thread) and by the caller's cap
    int per_sm = kMaxWarpBlocksPerSM;
    {
      int occ = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, forward_warp_kernel, 32, 0) == cudaSuccess && occ > 0)
        per_sm = occ;
    }
    if (p->warp_smem) {
      const int by_smem = (int)(sm_bytes / (smem_bytes + 1024));
      if (by_smem < per_sm) per_sm = by_smem;
    }
    if (mps_cap > 0 && mps_cap < per_sm) per_sm = mps_cap;
    if (per_sm < 1) per_sm = 1;
    p->warp_per_sm = per_sm;
    long cap_warps = (long)nsm * per_sm;
    if (cap_warps > mem_cap) cap_warps = mem_cap;
    long want = max_modes;
    long nw = want < cap_warps ? want : cap_warps;
    p->warp_blocks = (int)nw;
    nslots = nw;
    p->warp_smem_bytes = smem_bytes;
    // the attribute belongs to the kernel, not to the plan
    if (p->warp_smem && ensure_warp_smem(dev, smem_bytes) != DEB_OK) {
      delete p;
      return DEB_ERR_CUDA;
    }
  }
  const bool need_ws = mode == DEB_EXEC_LANE || !p->warp_smem;
  p->ws_bytes = (size_t)nslots * (need_ws ? p->slot_len : 0) * sizeof(double) + (size_t)nslots * p->dense_len * sizeof(double);
  p->ws = nullptr;
  p->dws = nullptr;
  p->kws = nullptr;
  if (need_ws && cudaMalloc(&p->ws, (size_t)nslots * p->slot_len * sizeof(double)) != cudaSuccess) { delete p; return DEB_ERR_NOMEM; }
  if (mode == DEB_EXEC_WARP && p->warp_k_global) {
    if (cudaMalloc(&p->kws, (size_t)nslots * deb::stage_len(p->D) * sizeof(double)) != cudaSuccess) {
      cudaFree(p->ws); delete p; return DEB_ERR_NOMEM;
    }
    p->ws_bytes += (size_t)nslots * deb::stage_len(p->D) * sizeof(double);
  }
  if (p->dense && cudaMalloc(&p->dws, (size_t)nslots * p->dense_len * sizeof(double)) != cudaSuccess) {
    cudaFree(p->ws); delete p; return DEB_ERR_NOMEM;
  }
  if (cudaMalloc(&p->queue, sizeof(int) * 4) != cudaSuccess) { cudaFree(p->ws); cudaFree(p->dws); cudaFree(p->kws); delete p; return DEB_ERR_NOMEM; }
  if (cudaMalloc(&p->order_dev, sizeof(int) * (size_t)max_modes) != cudaSuccess) {
    cudaFree(p->ws); cudaFree(p->dws); cudaFree(p->kws); cudaFree(p->queue); delete p; return DEB_ERR_NOMEM;
  }
  p->user_order = nullptr;
  p->user_order_n = 0;
  *out = p;
  return DEB_OK;
}

int deb_plan_workspace_bytes(const deb_plan* p, size_t* bytes) {
  if (!p || !bytes) return DEB_ERR_INVALID;
  *bytes = p->ws_bytes;
  return DEB_OK;
}

int deb_plan_create_grouped(const deb_dims* dims, int max_modes, int batch_size, deb_plan** out) {
  if (!dims || !out || max_modes <= 0 || batch_size < 1 || batch_size > 32) return DEB_ERR_INVALID;
  *out = nullptr;
  if (dims->linear_solver != DEB_SOLVE_STRUCTURED || dims->return_full) return DEB_ERR_INVALID;
  if (dims->lmaxg < 3 || dims->lmaxgp < 3 || dims->lmaxr < 3 || dims->lmaxnu < 3 || dims->nqmax < 1 || dims->nout < 1)
    return DEB_ERR_INVALID;
  if (dims->lmaxg > deb::LMAX_TABLE || dims->lmaxgp > deb::LMAX_TABLE || dims->lmaxr > deb::LMAX_TABLE ||
      dims->lmaxnu > deb::LMAX_TABLE)
    return DEB_ERR_INVALID;
  int rc = upload_constants();
  if (rc) return rc;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEB_ERR_CUDA;
  deb_plan* p = new deb_plan();
  p->D = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
  p->dense = 0;
  p->return_full = 0;
  p->nout = dims->nout;
  p->exec_mode = DEB_EXEC_WARP;
  p->max_modes = max_modes;
  p->nsm = nsm;
  p->slot_len = deb::slot_len(p->D);
  p->dense_len = 0;
  p->group_size = batch_size;
  const long groups = ((long)max_modes + batch_size - 1) / batch_size;
  long warps = (long)nsm * kMaxWarpBlocksPerSM;
  const long mem_cap = (16L << 30) / (p->slot_len * 8 * batch_size);
  if (warps > mem_cap) warps = mem_cap;
  if (warps > groups) warps = groups;
  if (warps < 1) { delete p; return DEB_ERR_NOMEM; }
  p->group_warps = (int)warps;
  p->ws_bytes = (size_t)warps * batch_size * p->slot_len * sizeof(double);
  if (cudaMalloc(&p->ws, p->ws_bytes) != cudaSuccess) { delete p; return DEB_ERR_NOMEM; }
  if (cudaMalloc(&p->queue, sizeof(int) * 4) != cudaSuccess) { cudaFree(p->ws); delete p; return DEB_ERR_NOMEM; }
  if (cudaMalloc(&p->order_dev, sizeof(int)) != cudaSuccess) {
    cudaFree(p->ws); cudaFree(p->queue); delete p; return DEB_ERR_NOMEM;
  }
  *out = p;
  return DEB_OK;
}

int deb_plan_launch_info(const deb_plan* p, deb_launch_cfg* cfg, int* modes_in_flight) {
  if (!p || !cfg || !modes_in_flight) return DEB_ERR_INVALID;
  if (p->adj) {
    // adjoint plan: warps (items) in flight and per SM; "shared" when its
    // hottest vectors live in shared memory
    cfg->stage_vectors = p->adj_shared ? DEB_STAGE_SHARED : DEB_STAGE_ALL_GLOBAL;
    cfg->modes_per_sm = p->nsm > 0 ? (p->adj_warps + p->nsm - 1) / p->nsm : 0;
    *modes_in_flight = p->adj_warps;
  } else if (p->group_size > 0) {
    cfg->stage_vectors = DEB_STAGE_GLOBAL;
    cfg->modes_per_sm = 0;
    *modes_in_flight = p->group_warps * p->group_size;
  } else if (p->exec_mode == DEB_EXEC_LANE) {
    cfg->stage_vectors = DEB_STAGE_GLOBAL;
    cfg->modes_per_sm = 0;
    *modes_in_flight = p->lane_slots;
  } else {
    cfg->stage_vectors = !p->warp_smem ? DEB_STAGE_ALL_GLOBAL : (!p->warp_k_global ? DEB_STAGE_SHARED : DEB_STAGE_GLOBAL);
    cfg->modes_per_sm = p->warp_per_sm;
    *modes_in_flight = p->warp_blocks;
  }
  return DEB_OK;
}

void deb_plan_destroy(deb_plan* p) {
  if (!p) return;
  cudaFree(p->adj_ws);
  cudaFree(p->ws);
  cudaFree(p->dws);
  cudaFree(p->kws);
  cudaFree(p->queue);
  cudaFree(p->order_dev);
  delete p;
}

int deb_plan_set_order(deb_plan* p, const int* d_order, int nmode) {
  if (!p || (d_order && nmode <= 0)) return DEB_ERR_INVALID;
  p->user_order = d_order;
  p->user_order_n = d_order ? nmode : 0;
  return DEB_OK;
}

}  // extern "C"

namespace {

int launch_forward(deb_plan* p, const double* d_tables, int ncosmo, int nset, int blob_len, const double* d_k,
                   const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                   double* d_y_out, int* d_status, int* d_steps, double* d_record, int rec_len, int* d_nrec,
                   int record, int replay, void* stream, double* d_ckpt = nullptr, int ck_cap = 0,
                   int* d_ckstride = nullptr, const long long* d_ckoff = nullptr, const int* d_ckcap = nullptr) {
  if (!p || !cfg || ncosmo <= 0 || nset <= 0 || nmode < 0 || blob_len <= deb::HDR_LEN) return DEB_ERR_INVALID;
  if (p->group_size > 0 || p->adj) return DEB_ERR_INVALID;   // grouped / adjoint plans serve their own calls only
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_k || !d_tau_out || !d_y_out || !d_status) return DEB_ERR_INVALID;
  if ((long)nmode * nset > p->max_modes) return DEB_ERR_CAPACITY;
  if (!(cfg->rtol >= 0.0) || !(cfg->atol >= 0.0) || cfg->max_steps <= 0 || !(cfg->error_order > 0.0)) return DEB_ERR_INVALID;
  if ((record || replay) && (!d_record || !d_nrec || rec_len < 2)) return DEB_ERR_INVALID;
  if (record && rec_len < cfg->max_steps + 1) return DEB_ERR_INVALID;
  if (replay && p->exec_mode != DEB_EXEC_WARP) return DEB_ERR_INVALID;
  if (d_ckpt && (!record || !d_ckstride || (!d_ckoff && (ck_cap < 2 || (ck_cap & 1))))) return DEB_ERR_INVALID;
  if (d_ckoff && !d_ckcap) return DEB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  KParams P{};
  P.tables = d_tables; P.ncosmo = ncosmo; P.blob_len = blob_len; P.k = d_k; P.cosmo = d_cosmo_of_mode;
  P.nmode = nmode; P.tau_out = d_tau_out; P.y_out = d_y_out; P.status = d_status; P.steps = d_steps;
  P.ws = p->ws; P.dws = p->dws; P.slot_len = p->slot_len; P.dense_len = p->dense_len; P.queue = p->queue; P.D = p->D;
  P.smem = p->warp_smem;
  P.kws = p->kws;
  P.rec = d_record; P.rec_len = rec_len; P.nrec = d_nrec; P.nset = nset;
  P.ckpt = d_ckpt; P.ck_cap = ck_cap; P.ckstride = d_ckstride; P.ckoff = d_ckoff; P.ckcaps = d_ckcap;
  P.order = (!replay && p->user_order && p->user_order_n == nmode) ? p->user_order : nullptr;
  P.ctl.rtol = cfg->rtol; P.ctl.atol = cfg->atol;
  P.ctl.b1 = (cfg->icoeff + cfg->pcoeff + cfg->dcoeff) / cfg->error_order;
  P.ctl.b2 = -(cfg->pcoeff + 2.0 * cfg->dcoeff) / cfg->error_order;
  P.ctl.b3 = cfg->dcoeff / cfg->error_order;
  P.ctl.safety = cfg->safety; P.ctl.fmin = cfg->factormin; P.ctl.fmax = cfg->factormax;
  P.ctl.max_steps = cfg->max_steps; P.ctl.hist_on_reject = cfg->hist_on_reject;
  P.ctl.dense = p->dense; P.ctl.return_full = p->return_full; P.ctl.nout = p->nout;
  P.ctl.record = record; P.ctl.replay = replay; P.ctl.step_ts = cfg->step_to_outputs;
  if (cudaMemsetAsync(p->queue, 0, sizeof(int), s) != cudaSuccess) return DEB_ERR_CUDA;
  if (replay) {
    rank_desc_kernel<<<(nmode + 255) / 256, 256, 0, s>>>(d_nrec, nmode, p->order_dev);
    P.order = p->order_dev;
  }
  const long items = (long)nmode * nset;
  if (p->exec_mode == DEB_EXEC_LANE) {
    long need = (items + kBlock - 1) / kBlock;
    const int blocks = (int)(need < p->lane_blocks ? need : p->lane_blocks);
    forward_lane_kernel<<<blocks, kBlock, 0, s>>>(P);
  } else {
    const int wpb = p->warp_block_warps;
    long need = (items + wpb - 1) / wpb;
    const int blocks = (int)(need < p->warp_blocks ? need : p->warp_blocks);
    const size_t smem = p->warp_smem ? (size_t)p->warp_smem_bytes * wpb : 0;
    forward_warp_kernel<<<blocks, 32 * wpb, smem, s>>>(P);
  }
  if (cudaGetLastError() != cudaSuccess) return DEB_ERR_CUDA;
  return DEB_OK;
}

}  // namespace

extern "C" {

int deb_forward(deb_plan* p, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                double* d_y_out, int* d_status, int* d_steps, void* stream) {
  return launch_forward(p, d_tables, ncosmo, 1, blob_len, d_k, d_cosmo_of_mode, nmode, d_tau_out, cfg, d_y_out,
                        d_status, d_steps, nullptr, 0, nullptr, 0, 0, stream);
}

int deb_forward_grouped(deb_plan* p, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                        const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                        double* d_y_out, int* d_status, int* d_steps, void* stream) {
  if (!p || !cfg || p->group_size <= 0 || ncosmo <= 0 || nmode < 0 || blob_len <= deb::HDR_LEN) return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_k || !d_tau_out || !d_y_out || !d_status) return DEB_ERR_INVALID;
  if (nmode % p->group_size) return DEB_ERR_INVALID;
  if (nmode > p->max_modes) return DEB_ERR_CAPACITY;
  if (!(cfg->rtol >= 0.0) || !(cfg->atol >= 0.0) || cfg->max_steps <= 0 || !(cfg->error_order > 0.0)) return DEB_ERR_INVALID;
  if (cfg->step_to_outputs) return DEB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  KParams P{};
  P.tables = d_tables; P.ncosmo = ncosmo; P.blob_len = blob_len; P.k = d_k; P.cosmo = d_cosmo_of_mode;
  P.nmode = nmode; P.tau_out = d_tau_out; P.y_out = d_y_out; P.status = d_status; P.steps = d_steps;
  P.ws = p->ws; P.slot_len = p->slot_len; P.queue = p->queue; P.D = p->D; P.nset = 1;
  P.ctl.rtol = cfg->rtol; P.ctl.atol = cfg->atol;
  P.ctl.b1 = (cfg->icoeff + cfg->pcoeff + cfg->dcoeff) / cfg->error_order;
  P.ctl.b2 = -(cfg->pcoeff + 2.0 * cfg->dcoeff) / cfg->error_order;
  P.ctl.b3 = cfg->dcoeff / cfg->error_order;
  P.ctl.safety = cfg->safety; P.ctl.fmin = cfg->factormin; P.ctl.fmax = cfg->factormax;
  P.ctl.max_steps = cfg->max_steps; P.ctl.hist_on_reject = cfg->hist_on_reject;
  P.ctl.dense = 0; P.ctl.return_full = 0; P.ctl.nout = p->nout;
  P.ctl.record = 0; P.ctl.replay = 0; P.ctl.step_ts = 0;
  if (cudaMemsetAsync(p->queue, 0, sizeof(int), s) != cudaSuccess) return DEB_ERR_CUDA;
  const int ngroup = nmode / p->group_size;
  const int blocks = ngroup < p->group_warps ? ngroup : p->group_warps;
  forward_group_kernel<<<blocks, 32, 0, s>>>(P, p->group_size);
  if (cudaGetLastError() != cudaSuccess) return DEB_ERR_CUDA;
  return DEB_OK;
}

int deb_forward_record(deb_plan* p, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                       const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                       double* d_y_out, int* d_status, int* d_steps, double* d_record, int rec_len, int* d_nrec,
                       void* stream) {
  return launch_forward(p, d_tables, ncosmo, 1, blob_len, d_k, d_cosmo_of_mode, nmode, d_tau_out, cfg, d_y_out,
                        d_status, d_steps, d_record, rec_len, d_nrec, 1, 0, stream);
}

int deb_forward_record_ckpt(deb_plan* p, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                            const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                            double* d_y_out, int* d_status, int* d_steps, double* d_record, int rec_len, int* d_nrec,
                            double* d_ckpt, int ck_cap, const long long* d_ckoff, const int* d_ckcap,
                            int* d_ckstride, void* stream) {
  if (!d_ckpt) return DEB_ERR_INVALID;
  return launch_forward(p, d_tables, ncosmo, 1, blob_len, d_k, d_cosmo_of_mode, nmode, d_tau_out, cfg, d_y_out,
                        d_status, d_steps, d_record, rec_len, d_nrec, 1, 0, stream, d_ckpt, ck_cap, d_ckstride,
                        d_ckoff, d_ckcap);
}

int deb_replay(deb_plan* p, const double* d_tables, int ncosmo, int nset, int blob_len, const double* d_k,
               const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
               const double* d_record, int rec_len, const int* d_nrec, double* d_y_out, int* d_status, void* stream) {
  return launch_forward(p, d_tables, ncosmo, nset, blob_len, d_k, d_cosmo_of_mode, nmode, d_tau_out, cfg, d_y_out,
                        d_status, nullptr, const_cast<double*>(d_record), rec_len, const_cast<int*>(d_nrec), 0, 1,
                        stream);
}

int deb_get_power(const double* d_tables, int ncosmo, int blob_len, const double* d_k, const int* d_cosmo_of_mode,
                  int nmode, int nout, const double* d_y, int stride, int idx, double* d_P, void* stream) {
  if (!d_tables || !d_k || !d_y || !d_P || ncosmo <= 0 || nmode < 0 || nout <= 0 || idx < 0 || idx >= stride)
    return DEB_ERR_INVALID;
  if (nmode == 0) return DEB_OK;
  const long tot = (long)nmode * nout;
  const int threads = 256;
  power_kernel<<<(unsigned)((tot + threads - 1) / threads), threads, 0, (cudaStream_t)stream>>>(
      d_tables, ncosmo, blob_len, d_k, d_cosmo_of_mode, nmode, nout, d_y, stride, idx, d_P);
  return cudaGetLastError() == cudaSuccess ? DEB_OK : DEB_ERR_CUDA;
}

// ---------------------------------------------------------------- allocation-free entry point
// Scratch of deb_forward_static: bytes [0, 256) hold the work-queue counter,
// the rest holds one warp-mode slot per mode in flight.
static __device__ __align__(256) double g_static_scratch[DEB_STATIC_SCRATCH_BYTES / sizeof(double)];

int deb_forward_static(const deb_dims* dims, const double* d_tables, int ncosmo, int blob_len, const double* d_k,
                       const int* d_cosmo_of_mode, int nmode, const double* d_tau_out, const deb_solver_cfg* cfg,
                       double* d_y_out, int* d_status, int* d_steps, void* stream) {
  if (!dims || !cfg || ncosmo <= 0 || nmode < 0 || blob_len <= deb::HDR_LEN) return DEB_ERR_INVALID;
  if (dims->lmaxg < 3 || dims->lmaxgp < 3 || dims->lmaxr < 3 || dims->lmaxnu < 3 || dims->nqmax < 1 || dims->nout < 1)
    return DEB_ERR_INVALID;
  if (dims->lmaxg > deb::LMAX_TABLE || dims->lmaxgp > deb::LMAX_TABLE || dims->lmaxr > deb::LMAX_TABLE ||
      dims->lmaxnu > deb::LMAX_TABLE)
    return DEB_ERR_INVALID;
  if (dims->linear_solver != DEB_SOLVE_STRUCTURED) return DEB_ERR_INVALID;
  if (!(cfg->rtol >= 0.0) || !(cfg->atol >= 0.0) || cfg->max_steps <= 0 || !(cfg->error_order > 0.0)) return DEB_ERR_INVALID;
  const deb::Dims D = deb::make_dims(dims->lmaxg, dims->lmaxgp, dims->lmaxr, dims->lmaxnu, dims->nqmax);
  const long slot_len = deb::slot_len(D);
  const long max_slots = (long)(DEB_STATIC_SCRATCH_BYTES - 256) / (slot_len * (long)sizeof(double));
  if (max_slots < 1) return DEB_ERR_STATIC_SCRATCH;
  if (nmode == 0) return DEB_OK;
  if (!d_tables || !d_k || !d_tau_out || !d_y_out || !d_status) return DEB_ERR_INVALID;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DEB_ERR_CUDA;
  int rc = upload_constants();
  if (rc) return rc;
  // the array's device address in the current context, looked up on every
  // call (cheap): a cached pointer would outlive a cudaDeviceReset
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_static_scratch) != cudaSuccess || !ptr) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEB_ERR_CUDA;
  double* base = (double*)ptr;
  cudaStream_t s = (cudaStream_t)stream;
  KParams P{};
  P.tables = d_tables; P.ncosmo = ncosmo; P.blob_len = blob_len; P.k = d_k; P.cosmo = d_cosmo_of_mode;
  P.nmode = nmode; P.tau_out = d_tau_out; P.y_out = d_y_out; P.status = d_status; P.steps = d_steps;
  P.ws = base + 256 / sizeof(double); P.dws = nullptr; P.slot_len = slot_len; P.dense_len = 0;
  P.queue = (int*)base; P.D = D; P.smem = 0;
  P.rec = nullptr; P.rec_len = 0; P.nrec = nullptr; P.nset = 1; P.kws = nullptr;
  P.ctl.rtol = cfg->rtol; P.ctl.atol = cfg->atol;
  P.ctl.b1 = (cfg->icoeff + cfg->pcoeff + cfg->dcoeff) / cfg->error_order;
  P.ctl.b2 = -(cfg->pcoeff + 2.0 * cfg->dcoeff) / cfg->error_order;
  P.ctl.b3 = cfg->dcoeff / cfg->error_order;
  P.ctl.safety = cfg->safety; P.ctl.fmin = cfg->factormin; P.ctl.fmax = cfg->factormax;
  P.ctl.max_steps = cfg->max_steps; P.ctl.hist_on_reject = cfg->hist_on_reject;
  P.ctl.dense = 0; P.ctl.return_full = dims->return_full; P.ctl.nout = dims->nout;
  P.ctl.record = 0; P.ctl.replay = 0; P.ctl.step_ts = cfg->step_to_outputs;
  long warps = (long)nsm * 8;
  if (warps > max_slots) warps = max_slots;
  if (warps > nmode) warps = nmode;
  if (cudaMemsetAsync(P.queue, 0, sizeof(int), s) != cudaSuccess) return DEB_ERR_CUDA;
  forward_warp_kernel<<<(unsigned)warps, 32, 0, s>>>(P);
  if (cudaGetLastError() != cudaSuccess) return DEB_ERR_CUDA;
  return DEB_OK;
}

int deb_measure_fp64_peak(double* flops_per_s, void* stream) {
  if (!flops_per_s) return DEB_ERR_INVALID;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEB_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return DEB_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = nsm * 8, threads = 256, iters = 1 << 14;
  fp64_peak_kernel<<<blocks, threads, 0, s>>>(out, 256, 1.0000001, 1e-9);  // warm-up
  cudaEventRecord(e0, s);
  fp64_peak_kernel<<<blocks, threads, 0, s>>>(out, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return DEB_ERR_CUDA;
  *flops_per_s = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3);
  return DEB_OK;
}

}  // extern "C"
