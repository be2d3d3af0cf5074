// deb_internal.h -- library-internal declarations shared by the CUDA
// translation units (not part of the C ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "deb_core.cuh"

struct deb_plan {
  deb::Dims D;
  int dense, return_full, nout, exec_mode;
  int max_modes, nsm;
  long slot_len, dense_len;
  // lane mode
  int lane_blocks, lane_slots;
  // warp mode
  int warp_block_warps, warp_blocks, warp_smem, warp_k_global, warp_per_sm;
  // grouped plans (deb_plan_create_grouped): modes per group, warps in flight
  int group_size, group_warps;
  long warp_smem_bytes;
  double* kws;      // warp mode: stage vectors in global memory
  double* ws;       // lane slots (or warp slots when shared memory is too small)
  double* dws;      // dense matrices
  int* queue;
  int* order_dev;   // replay order (max_modes ints)
  const int* user_order;   // deb_plan_set_order
  int user_order_n;
  size_t ws_bytes;
  // adjoint plans (deb_plan_create_adjoint): warps in flight, states per
  // segment, per-warp workspace (doubles) and its array
  int adj, adj_warps, adj_seg_cap;
  long adj_wslot;
  long adj_smem;   // dynamic shared memory of the adjoint launch (bytes)
  int adj_shared;  // its hottest vectors in shared memory
  double* adj_ws;
};


namespace deb_internal {

using PFN_ctxGetCurrent = CUresult (*)(CUcontext*);
using PFN_ctxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current thread's CUDA context (never reused within a
// process), 0 if it cannot be determined.  The driver entry points are found
// through the runtime, so the library needs no link to libcuda.
inline unsigned long long current_ctx_id() {
  static PFN_ctxGetCurrent get_cur = nullptr;
  static PFN_ctxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = (PFN_ctxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PFN_ctxGetId)f;
  });
  if (!get_cur || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_cur(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id + 1;   // 0 stays "unknown"
}

// Warps per SM for a kernel whose warps each work on hot_bytes of global
// memory: the warps whose bytes fill `fill` times the SM's share of L2
// (measured at nvar 1098: the adjoint, ~300 KB a warp, is fastest at 4
// warps per SM, fill 1.6; more warps in flight evict each other's vectors,
// fewer hide less latency), at least 2, at most max_per_sm.  (The record,
// 141 KB a mode, gained from 6 modes per SM on 2048 modes but lost on 4096:
// it keeps its register-limited 8.)
inline int l2_warps_per_sm(int dev, int nsm, long hot_bytes, int max_per_sm, double fill) {
  int l2 = 0;
  if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess || l2 <= 0 || nsm <= 0 ||
      hot_bytes <= 0)
    return max_per_sm;
  const double share = (double)l2 / nsm;
  int w = (int)(fill * share / (double)hot_bytes);
  if (w < 2) w = 2;
  return w < max_per_sm ? w : max_per_sm;
}

}  // namespace deb_internal
