// runtime.cu - the C ABI of include/nmc_abi.h.
//
// Replaces the reference's Objective-C host runtime (NMC/NMCCode/MetalMC.m):
// kernel selection (MetalMC.m:115-149), buffer set-up (:179-383), dispatch
// (:385-496) and the host-side tally reduction (:508-824).  Differences by
// design:
//  * one persistent launch simulates any number of photons (the reference
//    dispatches PHOTON_BATCH threads per blocking command buffer);
//  * tallies are device-resident u64 fixed point (no per-thread slabs: the
//    reference's mcxyz Rd2D/DetPhot2D slabs are PHOTON_BATCH*Nx*Ny each);
//  * every call returns a status; waits are bounded by nmc_ext.timeout_s.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "nmc_abi.h"

using nmc::DevSums;

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
};

// Regions of the result staging buffer (floats): the tallies
// nmc_get_compute_results can return, converted on the device.
enum StageRegion { kStJ, kStF, kStF3D, kStSlots, kStRd2D, kStDet, kStSums, kStN };

// A CUDA graph that converts and copies one combination of regions (mask of
// 1 << StageRegion): captured once per handle and combination, replayed by
// every nmc_get_compute_results.
struct ReduceGraph {
  unsigned mask;
  cudaGraphExec_t exec;
};

struct nmc_handle {
  int sim = 0;
  int device = 0;
  nmc_ext ext{};
  nmc_run_params rp{};
  nmc_tissue_params tp{};
  bool prepared = false;
  uint32_t tiss_used = 0;  // bit t: tissue t occurs in the map
  uint64_t tiss_count[NMC_NTISS] = {};  // voxels of each tissue id in the map
  std::string err;
  int32_t run = 1;
  cudaStream_t stream = nullptr;
  int nsm = 0;
  DevSums* d_sums = nullptr;
  uint8_t* d_V = nullptr;
  unsigned long long* d_F3D = nullptr;
  unsigned long long* d_Rd2D = nullptr;
  unsigned int* d_Det = nullptr;
  unsigned long long* d_slots = nullptr;
  unsigned long long* d_J = nullptr;
  unsigned long long* d_F = nullptr;
  size_t nvox = 0, n2d = 0, nslots = 0, nJ = 0, nF = 0;
  // the persisting L2 set-aside this handle raised, and the value it found
  bool l2_raised = false;
  size_t l2_prev = 0;
  // Fixed-point tallies are folded into FP64 carries before they could wrap:
  // a photon adds at most about one weight unit (2^32 fixed-point units) to a
  // bin, so 2^31 photons between folds keep every u64 word below 2^63 and
  // every u32 count below 2^31.  Carries are allocated at the first fold.
  double *c_F3D = nullptr, *c_Rd2D = nullptr, *c_Det = nullptr, *c_slots = nullptr, *c_J = nullptr,
         *c_F = nullptr, *c_rdr = nullptr;
  uint64_t since_fold = 0, fold_every = 1ull << 31;
  // Grow-only device scratch of the synchronous calls (sweeps, adjoint
  // backward).  Each of them waits for the handle's earlier work before it
  // writes here and for its own before it returns.
  char* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  float* d_stage = nullptr;  // conversion buffer for results (floats)
  float* h_stage = nullptr;  // pinned host copy
  size_t stage_elems = 0;
  size_t st_off[kStN] = {}, st_len[kStN] = {};
  std::vector<ReduceGraph> graphs;
  std::vector<EventPair> pending;
  std::vector<EventPair> pool;
  double kernel_ms = 0.0;
  uint32_t launches = 0;
  uint32_t seen_flags = 0;
  nmc::XyzParams xp{};
  nmc::SubParams sp{};
  // per-voxel media, radial tally, adjoint
  bool voxel_mode = false;
  float4* d_vox = nullptr;
  int rd_bins = 0;
  float rd_dr = 0.f;
  unsigned long long* d_rdr = nullptr;
  nmc::AdjEvent* d_ev = nullptr;
  unsigned long long* d_evcount = nullptr;
  uint64_t ev_cap = 0, ev_limit = 0, adj_first = 0, adj_n = 0;  // allocated / requested events
  bool adj_ready = false;
  // the record pass's deposit list (adjoint of a fluence loss without a score replay)
  uint2* d_dl = nullptr;
  unsigned int* d_dlfill = nullptr;
  unsigned long long* d_dlnext = nullptr;
  unsigned int dl_chunks = 0;  // allocated chunks
  unsigned int dl_req = 0;     // chunks the last record pass could use
  unsigned int dl_used = 0;    // chunks the last record pass filled
  bool dl_ok = false;          // the last record pass's list is complete
};

namespace {

nmc_status fail(nmc_handle* h, nmc_status st, const std::string& msg) {
  if (h) h->err = msg;
  return st;
}

nmc_status cuda_fail(nmc_handle* h, cudaError_t e, const char* what) {
  return fail(h, NMC_EDEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

#define NMC_CUDA(h, call)                                 \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

// The handle's device is current for the rest of the entry point.
#define NMC_ON_DEVICE(h)                      \
  nmc::DeviceScope on_device_((h)->device); \
  if (!on_device_.ok) return fail((h), NMC_EDEVICE, "cudaSetDevice failed")

template <class T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

// Marks [base, base + bytes) as persisting in L2 for the handle's stream and
// raises the context's persisting set-aside to cover it (capped by the
// device); the u64 fluence tally then stays in L2 under the atomics instead
// of being written back and re-fetched.  A hint only: a device or driver
// that refuses it leaves the run as it was.
void keep_in_l2(nmc_handle* h, void* base, size_t bytes) {
  if (h->ext.flags & NMC_FLAG_NO_L2_PERSIST) return;
  int max_persist = 0, max_window = 0;
  if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, h->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, h->device) != cudaSuccess ||
      max_persist <= 0 || max_window <= 0) {
    cudaGetLastError();
    return;
  }
  const size_t window = std::min(bytes, (size_t)max_window);
  const size_t want = std::min(window, (size_t)max_persist);
  size_t cur = 0;
  if (cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (cur < want && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) == cudaSuccess) {
    if (!h->l2_raised) h->l2_prev = cur;
    h->l2_raised = true;
    cur = want;
  }
  cudaStreamAttrValue a{};
  a.accessPolicyWindow.base_ptr = base;
  a.accessPolicyWindow.num_bytes = window;
  a.accessPolicyWindow.hitRatio = std::min(1.0f, (float)cur / (float)window);
  a.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  a.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &a);
  cudaGetLastError();
}

// Clears the stream's window (before the tally it covers is freed).
void release_l2_window(nmc_handle* h) {
  if (!h->stream) return;
  cudaStreamAttrValue a{};
  a.accessPolicyWindow.num_bytes = 0;
  cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &a);
  cudaGetLastError();
}

// Everything a prepared handle may have grown beyond its map, its tallies
// and their staging: per-voxel properties, the radial tally, the adjoint's
// lists, FP64 carries, scratch and the captured reduction graphs.
void free_extras(nmc_handle* h) {
  dfree(h->d_vox);
  dfree(h->d_rdr);
  dfree(h->d_ev);
  dfree(h->d_evcount);
  dfree(h->d_dl);
  dfree(h->d_dlfill);
  dfree(h->d_dlnext);
  h->dl_chunks = 0;
  h->dl_ok = false;
  dfree(h->c_F3D);
  dfree(h->c_Rd2D);
  dfree(h->c_Det);
  dfree(h->c_slots);
  dfree(h->c_J);
  dfree(h->c_F);
  dfree(h->c_rdr);
  dfree(h->d_scratch);
  h->scratch_bytes = 0;
  h->since_fold = 0;
  for (ReduceGraph& g : h->graphs) cudaGraphExecDestroy(g.exec);
  h->graphs.clear();
  h->voxel_mode = false;
  h->rd_bins = 0;
  h->ev_cap = 0;
  h->adj_ready = false;
}

void free_buffers(nmc_handle* h) {
  release_l2_window(h);
  free_extras(h);
  dfree(h->d_V);
  dfree(h->d_F3D);
  dfree(h->d_Rd2D);
  dfree(h->d_Det);
  dfree(h->d_slots);
  dfree(h->d_J);
  dfree(h->d_F);
  dfree(h->d_stage);
  if (h->h_stage) cudaFreeHost(h->h_stage);
  h->h_stage = nullptr;
  h->nvox = h->n2d = h->nslots = h->nJ = h->nF = h->stage_elems = 0;
}

bool finite_nonneg(float v) { return std::isfinite(v) && v >= 0.f; }

// The handle's scratch with at least `bytes`: reused across calls, so a sweep
// pays no cudaMalloc, and no cudaFree (which waits for the whole device)
// holds up other handles' streams.
nmc_status scratch(nmc_handle* h, size_t bytes, char** out) {
  if (bytes > h->scratch_bytes) {
    dfree(h->d_scratch);
    h->scratch_bytes = 0;
    NMC_CUDA(h, cudaMalloc((void**)&h->d_scratch, bytes));
    h->scratch_bytes = bytes;
  }
  *out = h->d_scratch;
  return NMC_OK;
}

nmc_status build_xyz(nmc_handle* h) {
  nmc::XyzParams& p = h->xp;
  p = nmc::XyzParams{};
  nmc::fill_xyz(p, h->rp, h->tp, h->ext, h->sim);
  p.V = h->d_V;
  p.F3D = h->d_F3D;
  p.Rd2D = h->d_Rd2D;
  p.Det2D = h->d_Det;
  p.rd_slots = h->d_slots;
  p.nslots = h->nslots;
  p.sums = h->d_sums;
  p.vox = h->d_vox;
  p.rd_r = h->d_rdr;
  p.rd_bins = h->rd_bins;
  p.rd_idr = h->rd_bins > 0 ? (float)(1.0 / h->rd_dr) : 0.f;
  return NMC_OK;
}

nmc_status build_sub(nmc_handle* h) {
  nmc::SubParams& p = h->sp;
  p = nmc::SubParams{};
  nmc::fill_sub(p, h->rp, h->tp, h->ext);
  p.J = h->d_J;
  p.F = h->d_F;
  p.sums = h->d_sums;
  return NMC_OK;
}

// The optical properties of every tissue in `mask` (bit t = tissue t) must be
// usable: finite mua >= 0, finite mus > 0, finite g.  `set` >= 0 names the
// sweep set in the message.
nmc_status check_tissues(nmc_handle* h, const nmc_tissue_params* tp, uint32_t mask, int set) {
  for (int t = 0; t < NMC_NTISS; ++t) {
    if (!(mask >> t & 1u)) continue;
    if (!nmc::tissue_usable(*tp, t)) {
      char msg[128];
      if (set >= 0)
        std::snprintf(msg, sizeof msg, "sweep set %d, tissue %d needs finite mua >= 0, mus > 0 and phase terms",
                      set, t);
      else
        std::snprintf(msg, sizeof msg, "tissue %d needs finite mua >= 0, mus > 0 and phase terms", t);
      return fail(h, NMC_EINVAL, msg);
    }
  }
  return NMC_OK;
}

nmc_status validate(nmc_handle* h, const nmc_run_params* rp, const nmc_tissue_params* tp,
                    const uint8_t* v) {
  const nmc_ext& e = h->ext;
  if (e.photons_per_dispatch == 0) return fail(h, NMC_EINVAL, "photons_per_dispatch must be > 0");
  if (e.rng != NMC_RNG_PHILOX && e.rng != NMC_RNG_TAUS_REF) return fail(h, NMC_EINVAL, "unknown rng");
  if (h->sim == NMC_SIM_MCSUB) {
    if (e.sub_bins < 2 || e.sub_bins > 4096) return fail(h, NMC_EINVAL, "sub_bins out of range [2, 4096]");
    if (!(e.sub_dr > 0.f) || !(e.sub_dz > 0.f)) return fail(h, NMC_EINVAL, "sub_dr / sub_dz must be > 0");
    if (e.phase > NMC_PHASE_TWO_TERM) return fail(h, NMC_EINVAL, "unknown phase function");
    const float mua = tp->muav[1], mus = tp->musv[1];
    if (!finite_nonneg(mua) || !finite_nonneg(mus) || !(mua + mus > 0.f))
      return fail(h, NMC_EINVAL, "tissue 1 needs finite mua, mus >= 0 with mua + mus > 0");
    if (!(rp->n1 > 0.f) || !(rp->n2 > 0.f)) return fail(h, NMC_EINVAL, "n1, n2 must be > 0");
    return NMC_OK;
  }
  if (!v) return fail(h, NMC_EINVAL, "voxel kinds need a tissue map");
  if (rp->Nx <= 0 || rp->Ny <= 0 || rp->Nz <= 0) return fail(h, NMC_EINVAL, "Nx, Ny, Nz must be > 0");
  if ((double)rp->Nx * rp->Ny * rp->Nz >= 2147483647.0) return fail(h, NMC_EINVAL, "grid too large (>= 2^31 voxels)");
  if (!(rp->dx > 0.f) || !(rp->dy > 0.f) || !(rp->dz > 0.f) || !std::isfinite(rp->dx) ||
      !std::isfinite(rp->dy) || !std::isfinite(rp->dz))
    return fail(h, NMC_EINVAL, "dx, dy, dz must be finite and > 0");
  if (rp->boundaryflag < 0 || rp->boundaryflag > 2) return fail(h, NMC_EINVAL, "boundaryflag must be 0, 1 or 2");
  if (rp->det_state != 0 && rp->det_state != 1) return fail(h, NMC_EINVAL, "det_state must be 0 or 1");
  if (!(rp->n1 > 0.f) || !(rp->n2 > 0.f)) return fail(h, NMC_EINVAL, "n1, n2 must be > 0");
  uint64_t count[NMC_NTISS] = {};
  const size_t n = (size_t)rp->Nx * rp->Ny * rp->Nz;
  for (size_t k = 0; k < n; ++k) {
    if (v[k] >= NMC_NTISS) {
      char msg[96];
      std::snprintf(msg, sizeof msg, "tissue id %u at voxel %zu exceeds %d", (unsigned)v[k], k, NMC_NTISS - 1);
      return fail(h, NMC_EINVAL, msg);
    }
    ++count[v[k]];
  }
  uint32_t mask = 0;
  for (int t = 0; t < NMC_NTISS; ++t)
    if (count[t]) mask |= 1u << t;
  nmc_status st = check_tissues(h, tp, mask, -1);
  if (st == NMC_OK) {
    h->tiss_used = mask;
    std::copy(count, count + NMC_NTISS, h->tiss_count);
  }
  return st;
}

nmc_status wait_event(nmc_handle* h, cudaEvent_t ev) {
  const auto t0 = std::chrono::steady_clock::now();
  const double limit = h->ext.timeout_s > 0 ? h->ext.timeout_s : 1e30;
  while (true) {
    const cudaError_t q = cudaEventQuery(ev);
    if (q == cudaSuccess) return NMC_OK;
    if (q != cudaErrorNotReady) return cuda_fail(h, q, "kernel execution");
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > limit) return fail(h, NMC_ETIMEOUT, "device work did not finish within timeout_s");
    std::this_thread::sleep_for(std::chrono::microseconds(el < 0.01 ? 20 : 500));
  }
}

// Waits (bounded by timeout_s) for everything queued on the handle's stream.
nmc_status wait_stream(nmc_handle* h) {
  cudaEvent_t ev;
  NMC_CUDA(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, h->stream);
  nmc_status st = e == cudaSuccess ? wait_event(h, ev) : cuda_fail(h, e, "cudaEventRecord");
  cudaEventDestroy(ev);
  return st;
}

EventPair get_pair(nmc_handle* h) {
  if (!h->pool.empty()) {
    EventPair p = h->pool.back();
    h->pool.pop_back();
    return p;
  }
  EventPair p;
  cudaEventCreate(&p.a);
  cudaEventCreate(&p.b);
  return p;
}

// Device buffers of one adjoint pass.
struct AdjArgs {
  int pass;  // 0 record, 1 accumulating replay, 2 score replay
  float* D;
  const float* G;
  const float* GF;
  double* gL;
  double* gM;
  double* gQ;
  bool deposit_list = false;  // record pass: also keep the deposit list
};

nmc_status fold(nmc_handle* h);

nmc_status launch(nmc_handle* h, uint64_t first, uint64_t n, nmc_photon_record* d_recs,
                  float4* d_events, uint32_t k_events, const AdjArgs* adj = nullptr) {
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  if (n == 0) return NMC_OK;
  if (!d_recs && !adj && n > h->fold_every) {  // launches of at most fold_every photons, folded between
    for (uint64_t done = 0; done < n;) {
      const uint64_t m = std::min<uint64_t>(h->fold_every, n - done);
      const nmc_status st = launch(h, first + done, m, nullptr, nullptr, 0, nullptr);
      if (st != NMC_OK) return st;
      done += m;
    }
    return NMC_OK;
  }
  if (h->since_fold + n > h->fold_every) {
    const nmc_status st = fold(h);
    if (st != NMC_OK) return st;
  }
  h->since_fold += n;
  if (adj && !h->voxel_mode) return fail(h, NMC_ESTATE, "the adjoint needs per-voxel properties");
  if (h->voxel_mode && h->sim == NMC_SIM_MCXYZ_TT)
    return fail(h, NMC_EUNSUPPORTED, "per-voxel media use the one-term HG kernel (NMC_SIM_MCXYZ)");
  if (h->voxel_mode && h->ext.rng != NMC_RNG_PHILOX)
    return fail(h, NMC_EUNSUPPORTED, "per-voxel media use the Philox streams");
  NMC_CUDA(h, cudaMemsetAsync(&h->d_sums->work, 0, sizeof(unsigned long long), h->stream));
  const bool trace = d_recs != nullptr;
  nmc::TraceParams tr{d_recs, d_events, d_events ? k_events : 0u};
  int block, per_sm = 0;
  EventPair ev = get_pair(h);
  NMC_CUDA(h, cudaEventRecord(ev.a, h->stream));
  if (h->sim == NMC_SIM_MCSUB) {
    nmc::SubParams p = h->sp;
    p.first = first;
    p.n = n;
    p.trace = tr;
    block = h->ext.block_size > 0 ? h->ext.block_size : 512;
    NMC_CUDA(h, nmc::mcsub_occupancy(p, trace, block, &per_sm));
    if (h->ext.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)h->ext.blocks_per_sm);
    if (per_sm < 1) return fail(h, NMC_EDEVICE, "mcsub kernel does not fit on an SM with this block size");
    uint64_t grid = (uint64_t)h->nsm * per_sm;
    grid = std::min<uint64_t>(grid, (n + block - 1) / block);
    NMC_CUDA(h, nmc::launch_mcsub(p, trace, (int)grid, block, h->stream));
  } else {
    nmc::XyzParams p = h->xp;
    p.first = first;
    p.n = n;
    p.trace = tr;
    if (adj) {
      p.adj_pass = adj->pass;
      p.ev = h->d_ev;
      p.ev_count = h->d_evcount;
      p.ev_cap = (unsigned int)std::min(h->ev_cap, h->ev_limit);
      p.adj_D = adj->D;
      p.adj_Dw = adj->D;
      p.adj_G = adj->G;
      p.adj_GF = adj->GF;
      p.gL = adj->gL;
      p.gM = adj->gM;
      p.gQ = adj->gQ;
      if (adj->pass == 0 && adj->deposit_list) {
        p.dl_pool = h->d_dl;
        p.dl_chunks = h->dl_req;
        p.dl_fill = h->d_dlfill;
        p.dl_next = h->d_dlnext;
      }
    }
    block = h->ext.block_size > 0 ? h->ext.block_size : 256;
    const bool tt = h->sim == NMC_SIM_MCXYZ_TT;
    const int mode = !adj ? nmc::kVoxel : adj->pass == 0 ? nmc::kRecord : adj->pass == 2 ? nmc::kScore : nmc::kAdjoint;
    if (h->voxel_mode)
      NMC_CUDA(h, nmc::mcxyz_voxel_occupancy(mode, trace, block, &per_sm));
    else
      NMC_CUDA(h, nmc::mcxyz_occupancy(tt, trace, block, &per_sm));
    if (h->ext.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)h->ext.blocks_per_sm);
    if (per_sm < 1) return fail(h, NMC_EDEVICE, "mcxyz kernel does not fit on an SM with this block size");
    uint64_t grid = (uint64_t)h->nsm * per_sm;
    grid = std::min<uint64_t>(grid, (n + block - 1) / block);
    if (h->voxel_mode)
      NMC_CUDA(h, nmc::launch_mcxyz_voxel(p, mode, trace, (int)grid, block, h->stream));
    else
      NMC_CUDA(h, nmc::launch_mcxyz(p, tt, trace, (int)grid, block, h->stream));
  }
  NMC_CUDA(h, cudaEventRecord(ev.b, h->stream));
  h->pending.push_back(ev);
  ++h->launches;
  return NMC_OK;
}

nmc_status sync_all(nmc_handle* h) {
  if (h->pending.empty()) {
    NMC_CUDA(h, cudaStreamSynchronize(h->stream));
    return NMC_OK;
  }
  nmc_status st = wait_event(h, h->pending.back().b);
  if (st != NMC_OK) return st;
  for (EventPair& p : h->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) h->kernel_ms += ms;
    h->pool.push_back(p);
  }
  h->pending.clear();
  NMC_CUDA(h, cudaStreamSynchronize(h->stream));
  unsigned int flags = 0;
  NMC_CUDA(h, cudaMemcpy(&flags, &h->d_sums->flags, sizeof flags, cudaMemcpyDeviceToHost));
  const unsigned int fresh = flags & ~h->seen_flags;
  h->seen_flags = flags;
  if (fresh & NMC_DEVFLAG_BOUNDS)
    return fail(h, NMC_EDEVICE, "a tally index fell outside its buffer (checked build)");
  if (fresh & NMC_DEVFLAG_REPLAY)
    return fail(h, NMC_EDEVICE, "the adjoint replay did not reproduce the recorded detections");
  if (fresh & NMC_DEVFLAG_STEPCAP)
    return fail(h, NMC_ESTEPCAP, "a photon reached the device step cap and was terminated");
  return NMC_OK;
}

__global__ void unfix_f32(const unsigned long long* __restrict__ s, const double* __restrict__ c,
                          float* __restrict__ d, size_t n, double scale) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    d[k] = (float)((double)s[k] * scale + (c ? c[k] : 0.0));
}
__global__ void u32_to_f32(const unsigned int* __restrict__ s, const double* __restrict__ c,
                           float* __restrict__ d, size_t n) {
  // counts travel as int32 bits (the reference's DetPhot2D is int); saturate
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const double t = (double)s[k] + (c ? c[k] : 0.0);
    d[k] = __uint_as_float((unsigned int)fmin(t, 2147483647.0));
  }
}
// Moves fixed-point tallies into their FP64 carries (exact while a carry
// stays below 2^53 fixed-point units) and clears them.
__global__ void fold_u64(unsigned long long* __restrict__ s, double* __restrict__ c, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long v = s[k];
    if (v) {
      c[k] += (double)v * nmc::kUnfix;
      s[k] = 0ull;
    }
  }
}
__global__ void fold_u32(unsigned int* __restrict__ s, double* __restrict__ c, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const unsigned int v = s[k];
    if (v) {
      c[k] += (double)v;
      s[k] = 0u;
    }
  }
}
__global__ void fold_sums(DevSums* d) {
  d->carry[0] += (double)d->S * nmc::kUnfix;
  d->carry[1] += (double)d->A * nmc::kUnfix;
  d->carry[2] += (double)d->E * nmc::kUnfix;
  d->carry[3] += (double)d->rd * nmc::kUnfix;
  d->S = d->A = d->E = d->rd = 0ull;
}

// The reduction graph for `mask` (regions of StageRegion), captured on first
// use: per region a conversion kernel (u64 fixed point -> float, or u32 count
// bits) into the device staging buffer, then its copy to pinned host memory.
nmc_status reduce_graph(nmc_handle* h, unsigned mask, cudaGraphExec_t* out) {
  for (const ReduceGraph& g : h->graphs)
    if (g.mask == mask) {
      *out = g.exec;
      return NMC_OK;
    }
  const void* src[kStN] = {h->d_J, h->d_F, h->d_F3D, h->d_slots, h->d_Rd2D, h->d_Det, h->d_sums};
  const double* carry[kStN] = {h->c_J, h->c_F, h->c_F3D, h->c_slots, h->c_Rd2D, h->c_Det, nullptr};
  NMC_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < kStN && e == cudaSuccess; ++k) {
    if (!(mask >> k & 1u) || h->st_len[k] == 0) continue;
    const size_t n = h->st_len[k];
    float* dst = h->d_stage + h->st_off[k];
    if (k == kStSums) {
      e = cudaMemcpyAsync(dst, src[k], sizeof(DevSums), cudaMemcpyDeviceToDevice, h->stream);
    } else {
      const int block = 256;
      const int grid = (int)std::min<size_t>((n + block - 1) / block, (size_t)h->nsm * 8);
      if (k == kStDet)
        u32_to_f32<<<grid, block, 0, h->stream>>>((const unsigned int*)src[k], carry[k], dst, n);
      else
        unfix_f32<<<grid, block, 0, h->stream>>>((const unsigned long long*)src[k], carry[k], dst, n,
                                                  nmc::kUnfix);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->h_stage + h->st_off[k], dst, n * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(h, e != cudaSuccess ? e : e2, "capturing the result reduction");
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(h, e, "instantiating the result reduction");
  h->graphs.push_back(ReduceGraph{mask, exec});
  *out = exec;
  return NMC_OK;
}

// Folds every fixed-point tally and the fixed-point totals into their FP64
// carries, in stream order (no host wait).  A carry allocated here changes
// what the reduction graphs read, so they are captured again.
nmc_status fold(nmc_handle* h) {
  struct T {
    void* s;
    double** c;
    size_t n;
    bool u32;
  } t[] = {{h->d_F3D, &h->c_F3D, h->nvox, false}, {h->d_Rd2D, &h->c_Rd2D, h->n2d, false},
           {h->d_Det, &h->c_Det, h->n2d, true},   {h->d_slots, &h->c_slots, h->nslots, false},
           {h->d_J, &h->c_J, h->nJ, false},       {h->d_F, &h->c_F, h->nF, false},
           {h->d_rdr, &h->c_rdr, h->d_rdr ? (size_t)h->rd_bins + 1 : 0, false}};
  bool fresh = false;
  for (T& x : t) {
    if (!x.s || x.n == 0) continue;
    if (!*x.c) {
      NMC_CUDA(h, cudaMalloc((void**)x.c, x.n * sizeof(double)));
      NMC_CUDA(h, cudaMemsetAsync(*x.c, 0, x.n * sizeof(double), h->stream));
      fresh = true;
    }
    const int block = 256;
    const int grid = (int)std::min<size_t>((x.n + block - 1) / block, (size_t)h->nsm * 8);
    if (x.u32)
      fold_u32<<<grid, block, 0, h->stream>>>((unsigned int*)x.s, *x.c, x.n);
    else
      fold_u64<<<grid, block, 0, h->stream>>>((unsigned long long*)x.s, *x.c, x.n);
    NMC_CUDA(h, cudaGetLastError());
  }
  fold_sums<<<1, 1, 0, h->stream>>>(h->d_sums);
  NMC_CUDA(h, cudaGetLastError());
  if (fresh) {
    NMC_CUDA(h, cudaStreamSynchronize(h->stream));
    for (ReduceGraph& g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
  }
  h->since_fold = 0;
  return NMC_OK;
}

}  // namespace

// ------------------------------------------------------------- C entry points
extern "C" {

void nmc_ext_defaults(nmc_ext* e) {
  if (!e) return;
  std::memset(e, 0, sizeof *e);
  e->size = sizeof(nmc_ext);
  e->rng = NMC_RNG_PHILOX;
  e->seed = 0;
  e->phase = NMC_PHASE_HG;
  e->flags = 0;
  e->photons_per_dispatch = NMC_PHOTON_BATCH_DEFAULT;
  e->photons_total = NMC_PHOTON_TOTAL_DEFAULT;
  e->sub_bins = NMC_MCSUB_BINS_DEFAULT;
  e->sub_dr = NMC_MCSUB_DR_DEFAULT;
  e->sub_dz = NMC_MCSUB_DZ_DEFAULT;
  e->sub_mcflag = 0;          // mcflag_mcsub (definitions.h:38)
  e->sub_boundaryflag = 1;    // boundaryflag_mcsub (definitions.h:48)
  e->sub_radius = 0.0f;       // radius_mcsub
  e->sub_waist = 0.10f;       // waist_mcsub
  e->sub_zfocus = 1.0f;       // zfocus_mcsub
  e->sub_xs = e->sub_ys = e->sub_zs = 0.0f;
  e->block_size = 0;
  e->blocks_per_sm = 0;
  e->timeout_s = 600.0;
}

int32_t nmc_abi_version(void) { return NMC_ABI_VERSION; }

nmc_status nmc_create(int32_t sim_type, int32_t device, nmc_handle** out) {
  if (!out) return NMC_EINVAL;
  *out = nullptr;
  if (sim_type == NMC_SIM_POLARIZATION_CBS_ELECTRIC_FIELDS || sim_type == NMC_SIM_RAMAN ||
      sim_type == NMC_SIM_POLARIZATION_MUELLER_STOKES)
    return NMC_EUNSUPPORTED;
  if (sim_type != NMC_SIM_MCSUB && sim_type != NMC_SIM_MCXYZ && sim_type != NMC_SIM_MCXYZ_TT)
    return NMC_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NMC_EDEVICE;
  nmc_handle* h = new (std::nothrow) nmc_handle();
  if (!h) return NMC_ENOMEM;
  h->sim = sim_type;
  h->device = device;
  nmc_ext_defaults(&h->ext);
  nmc::DeviceScope dev(device);
  if (!dev.ok || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaMalloc((void**)&h->d_sums, sizeof(DevSums)) != cudaSuccess ||
      cudaMemset(h->d_sums, 0, sizeof(DevSums)) != cudaSuccess) {
    if (h->d_sums) cudaFree(h->d_sums);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return NMC_EDEVICE;
  }
  *out = h;
  return NMC_OK;
}

nmc_status nmc_set_ext(nmc_handle* h, const nmc_ext* ext) {
  if (!h || !ext) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  if (ext->size != sizeof(nmc_ext)) return fail(h, NMC_EINVAL, "nmc_ext.size does not match this library");
  const bool reprepare = h->prepared;
  h->ext = *ext;
  if (reprepare) {
    if (h->sim == NMC_SIM_MCSUB && (size_t)h->ext.sub_bins + 1 != h->nJ)
      return fail(h, NMC_ESTATE, "sub_bins changed: call nmc_prepare again");
    if (h->sim != NMC_SIM_MCSUB && h->ext.photons_per_dispatch != h->nslots)
      return fail(h, NMC_ESTATE, "photons_per_dispatch changed: call nmc_prepare again");
    return h->sim == NMC_SIM_MCSUB ? build_sub(h) : build_xyz(h);
  }
  return NMC_OK;
}

nmc_status nmc_prepare(nmc_handle* h, const nmc_run_params* rp, const nmc_tissue_params* tp,
                       const uint8_t* v) {
  if (!h || !rp || !tp) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  nmc_status st = validate(h, rp, tp, v);
  if (st != NMC_OK) return st;
  st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  // A voxel handle prepared again for a grid of the same size keeps its map,
  // tally and staging buffers (no cudaFree, which waits for the whole
  // device, and no pinned re-allocation); the rest is released as below.
  if (h->prepared && h->sim != NMC_SIM_MCSUB && h->nvox == (size_t)rp->Nx * rp->Ny * rp->Nz &&
      h->n2d == (size_t)rp->Nx * rp->Ny && h->nslots == h->ext.photons_per_dispatch) {
    free_extras(h);
    h->prepared = false;
    h->rp = *rp;
    h->tp = *tp;
    NMC_CUDA(h, cudaMemcpyAsync(h->d_V, v, h->nvox, cudaMemcpyHostToDevice, h->stream));
    h->prepared = true;
    st = nmc_reset(h);
    if (st != NMC_OK) return st;
    return build_xyz(h);
  }
  free_buffers(h);
  h->prepared = false;
  h->rp = *rp;
  h->tp = *tp;
  if (h->sim == NMC_SIM_MCSUB) {
    h->nJ = (size_t)h->ext.sub_bins + 1;
    h->nF = h->nJ * h->nJ;
    NMC_CUDA(h, cudaMalloc((void**)&h->d_J, h->nJ * 8));
    NMC_CUDA(h, cudaMalloc((void**)&h->d_F, h->nF * 8));
  } else {
    h->nvox = (size_t)rp->Nx * rp->Ny * rp->Nz;
    h->n2d = (size_t)rp->Nx * rp->Ny;
    h->nslots = h->ext.photons_per_dispatch;
    NMC_CUDA(h, cudaMalloc((void**)&h->d_V, h->nvox));
    NMC_CUDA(h, cudaMemcpyAsync(h->d_V, v, h->nvox, cudaMemcpyHostToDevice, h->stream));
    NMC_CUDA(h, cudaMalloc((void**)&h->d_F3D, h->nvox * 8));
    keep_in_l2(h, h->d_F3D, h->nvox * 8);
    NMC_CUDA(h, cudaMalloc((void**)&h->d_Rd2D, h->n2d * 8));
    NMC_CUDA(h, cudaMalloc((void**)&h->d_Det, h->n2d * 4));
    NMC_CUDA(h, cudaMalloc((void**)&h->d_slots, h->nslots * 8));
  }
  // one region per tally, 256-byte aligned
  const size_t lens[kStN] = {h->nJ, h->nF, h->nvox, h->nslots, h->n2d,
                             h->sim == NMC_SIM_MCXYZ ? h->n2d : 0, (sizeof(DevSums) + 3) / 4};
  size_t stage = 0;
  for (int k = 0; k < kStN; ++k) {
    h->st_off[k] = stage;
    h->st_len[k] = lens[k];
    stage += (lens[k] + 63) & ~(size_t)63;
  }
  h->stage_elems = stage;
  NMC_CUDA(h, cudaMalloc((void**)&h->d_stage, stage * sizeof(float)));
  NMC_CUDA(h, cudaMallocHost((void**)&h->h_stage, stage * sizeof(float)));
  h->prepared = true;
  st = nmc_reset(h);
  if (st != NMC_OK) return st;
  return h->sim == NMC_SIM_MCSUB ? build_sub(h) : build_xyz(h);
}

nmc_status nmc_set_tissue_params(nmc_handle* h, const nmc_tissue_params* tp) {
  if (!h || !tp) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_status st;
  if (h->sim == NMC_SIM_MCSUB) {
    const float mua = tp->muav[1], mus = tp->musv[1];
    if (!finite_nonneg(mua) || !finite_nonneg(mus) || !(mua + mus > 0.f))
      return fail(h, NMC_EINVAL, "tissue 1 needs finite mua, mus >= 0 with mua + mus > 0");
  } else if ((st = check_tissues(h, tp, h->tiss_used, -1)) != NMC_OK) {
    return st;
  }
  st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  h->tp = *tp;
  return h->sim == NMC_SIM_MCSUB ? build_sub(h) : build_xyz(h);
}

nmc_status nmc_reset(nmc_handle* h) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  NMC_CUDA(h, cudaMemsetAsync(h->d_sums, 0, sizeof(DevSums), h->stream));
  if (h->d_J) NMC_CUDA(h, cudaMemsetAsync(h->d_J, 0, h->nJ * 8, h->stream));
  if (h->d_F) NMC_CUDA(h, cudaMemsetAsync(h->d_F, 0, h->nF * 8, h->stream));
  if (h->d_F3D) NMC_CUDA(h, cudaMemsetAsync(h->d_F3D, 0, h->nvox * 8, h->stream));
  if (h->d_Rd2D) NMC_CUDA(h, cudaMemsetAsync(h->d_Rd2D, 0, h->n2d * 8, h->stream));
  if (h->d_Det) NMC_CUDA(h, cudaMemsetAsync(h->d_Det, 0, h->n2d * 4, h->stream));
  if (h->d_slots) NMC_CUDA(h, cudaMemsetAsync(h->d_slots, 0, h->nslots * 8, h->stream));
  if (h->d_rdr) NMC_CUDA(h, cudaMemsetAsync(h->d_rdr, 0, ((size_t)h->rd_bins + 1) * 8, h->stream));
  const std::pair<double*, size_t> carries[] = {{h->c_F3D, h->nvox}, {h->c_Rd2D, h->n2d}, {h->c_Det, h->n2d},
                                                {h->c_slots, h->nslots}, {h->c_J, h->nJ}, {h->c_F, h->nF},
                                                {h->c_rdr, (size_t)h->rd_bins + 1}};
  for (const auto& c : carries)
    if (c.first) NMC_CUDA(h, cudaMemsetAsync(c.first, 0, c.second * sizeof(double), h->stream));
  h->since_fold = 0;
  h->kernel_ms = 0.0;
  h->launches = 0;
  h->seen_flags = 0;
  return wait_stream(h);
}

nmc_status nmc_set_fold_interval(nmc_handle* h, uint64_t photons) {
  if (!h) return NMC_EINVAL;
  if (photons < 1 || photons > (1ull << 31))
    return fail(h, NMC_EINVAL, "the fold interval must be in [1, 2^31] photons");
  h->fold_every = photons;
  return NMC_OK;
}

nmc_status nmc_set_num_runs_seed(nmc_handle* h, int32_t run, float time_seed) {
  (void)time_seed;  // never read by the reference kernels (kernels.metal:330 is unused)
  if (!h) return NMC_EINVAL;
  if (run < 1) return fail(h, NMC_EINVAL, "run numbers start at 1 (main.m:159)");
  h->run = run;
  return NMC_OK;
}

nmc_status nmc_send_compute_command(nmc_handle* h) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  const uint64_t b = h->ext.photons_per_dispatch;
  return nmc_run(h, (uint64_t)(h->run - 1) * b, b);
}

nmc_status nmc_run_async(nmc_handle* h, uint64_t first, uint64_t n) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  return launch(h, first, n, nullptr, nullptr, 0);
}

nmc_status nmc_synchronize(nmc_handle* h) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  return sync_all(h);
}

nmc_status nmc_run(nmc_handle* h, uint64_t first, uint64_t n) {
  nmc_status st = nmc_run_async(h, first, n);
  if (st != NMC_OK) return st;
  NMC_ON_DEVICE(h);
  return sync_all(h);
}

nmc_status nmc_run_traced(nmc_handle* h, uint64_t first, uint64_t n, nmc_photon_record* recs,
                          float* events, uint32_t k_events) {
  if (!h || !recs) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_photon_record* d_recs = nullptr;
  float4* d_ev = nullptr;
  NMC_CUDA(h, cudaMalloc((void**)&d_recs, n * sizeof(nmc_photon_record)));
  const size_t nev = events ? (size_t)n * k_events : 0;
  if (nev) {
    if (cudaMalloc((void**)&d_ev, nev * sizeof(float4)) != cudaSuccess) {
      cudaFree(d_recs);
      return fail(h, NMC_ENOMEM, "trace event buffer");
    }
    std::vector<float> nanv(nev * 4, NAN);
    cudaMemcpy(d_ev, nanv.data(), nev * sizeof(float4), cudaMemcpyHostToDevice);
  }
  nmc_status st = launch(h, first, n, d_recs, d_ev, nev ? k_events : 0);
  if (st == NMC_OK) st = sync_all(h);
  if (st == NMC_OK || st == NMC_ESTEPCAP) {
    if (cudaMemcpy(recs, d_recs, n * sizeof(nmc_photon_record), cudaMemcpyDeviceToHost) != cudaSuccess)
      st = fail(h, NMC_EDEVICE, "copying trace records");
    if (nev && cudaMemcpy(events, d_ev, nev * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess)
      st = fail(h, NMC_EDEVICE, "copying trace events");
  }
  cudaFree(d_recs);
  if (d_ev) cudaFree(d_ev);
  return st;
}

nmc_status nmc_autotune(nmc_handle* h, uint64_t photons, nmc_tune_result* out) {
  if (!h || !out) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  if (photons == 0) return fail(h, NMC_EINVAL, "photons must be > 0");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  std::memset(out, 0, sizeof *out);
  const nmc_ext saved = h->ext;
  const bool sub = h->sim == NMC_SIM_MCSUB;
  const bool tt = h->sim == NMC_SIM_MCXYZ_TT;
  auto apply = [&](int block, int bps, uint32_t priv, uint32_t per) {
    h->ext = saved;
    h->ext.block_size = block;
    h->ext.blocks_per_sm = bps;
    h->ext.photons_per_fetch = per;
    h->ext.flags = (saved.flags & ~(uint32_t)NMC_FLAG_GLOBAL_TALLIES) | priv;
    return sub ? build_sub(h) : build_xyz(h);
  };
  auto restore = [&](nmc_status s) {
    h->ext = saved;
    const nmc_status b = sub ? build_sub(h) : build_xyz(h);
    return s != NMC_OK ? s : b;
  };
  auto time_run = [&](float* ms) -> nmc_status {
    const double before = h->kernel_ms;
    nmc_status s = launch(h, 0, photons, nullptr, nullptr, 0);
    if (s == NMC_OK) s = sync_all(h);
    if (s != NMC_OK && s != NMC_ESTEPCAP) return s;
    *ms = (float)(h->kernel_ms - before);
    return NMC_OK;
  };
  auto max_resident = [&](int block, int* bps) -> nmc_status {
    cudaError_t e;
    if (sub)
      e = nmc::mcsub_occupancy(h->sp, false, block, bps);
    else if (h->voxel_mode)
      e = nmc::mcxyz_voxel_occupancy(nmc::kVoxel, false, block, bps);
    else
      e = nmc::mcxyz_occupancy(tt, false, block, bps);
    return e == cudaSuccess ? NMC_OK : cuda_fail(h, e, "occupancy query");
  };
  // the defaults, run twice (the first also warms the caches)
  const uint32_t priv0 = saved.flags & NMC_FLAG_GLOBAL_TALLIES;
  float ms = 0.f;
  if ((st = apply(0, 0, priv0, 0)) != NMC_OK || (st = time_run(&ms)) != NMC_OK || (st = time_run(&ms)) != NMC_OK)
    return restore(st);
  out->fallback = nmc_tune_entry{0, 0, priv0, 0, ms};
  out->best = out->fallback;
  const std::vector<int> blocks = sub ? std::vector<int>{128, 256, 512} : std::vector<int>{64, 128, 256};
  std::vector<uint32_t> privs{0u};
  if (sub && !(saved.flags & NMC_FLAG_SKIP_FLUENCE) && nmc::mcsub_smem_bytes(saved.sub_bins) <= 200 * 1024)
    privs.push_back((uint32_t)NMC_FLAG_GLOBAL_TALLIES);
  // block size x resident blocks x privatisation at one photon per fetch,
  // then the best shape with runs of 2, 4 and 8 photons per fetch
  for (int block : blocks) {
    for (uint32_t priv : privs) {
      if ((st = apply(block, 0, priv, 1)) != NMC_OK) return restore(st);
      int maxb = 0;
      if ((st = max_resident(block, &maxb)) != NMC_OK) return restore(st);
      if (maxb < 1) continue;
      std::vector<int> cands{maxb, std::max(1, (3 * maxb) / 4), std::max(1, maxb / 2)};
      std::sort(cands.begin(), cands.end());
      cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
      for (int bps : cands) {
        if (out->n_tried >= (int)(sizeof out->tried / sizeof out->tried[0])) break;
        if ((st = apply(block, bps, priv, 1)) != NMC_OK || (st = time_run(&ms)) != NMC_OK) return restore(st);
        const nmc_tune_entry t{block, bps, priv, 1, ms};
        out->tried[out->n_tried++] = t;
        if (ms < out->best.ms) out->best = t;
      }
    }
  }
  const nmc_tune_entry shape = out->best;
  for (uint32_t per : {2u, 4u, 8u}) {
    if (out->n_tried >= (int)(sizeof out->tried / sizeof out->tried[0])) break;
    if ((st = apply(shape.block_size, shape.blocks_per_sm, shape.flags, per)) != NMC_OK ||
        (st = time_run(&ms)) != NMC_OK)
      return restore(st);
    const nmc_tune_entry t{shape.block_size, shape.blocks_per_sm, shape.flags, per, ms};
    out->tried[out->n_tried++] = t;
    if (ms < out->best.ms) out->best = t;
  }
  h->ext = saved;
  h->ext.block_size = out->best.block_size;
  h->ext.blocks_per_sm = out->best.blocks_per_sm;
  h->ext.photons_per_fetch = out->best.photons_per_fetch;
  h->ext.flags = (saved.flags & ~(uint32_t)NMC_FLAG_GLOBAL_TALLIES) | out->best.flags;
  st = sub ? build_sub(h) : build_xyz(h);
  if (st != NMC_OK) return st;
  return nmc_reset(h);
}

size_t nmc_tally_size(nmc_handle* h, int32_t which) {
  if (!h || !h->prepared) return 0;
  switch (which) {
    case NMC_TALLY_J: return h->nJ;
    case NMC_TALLY_F: return h->nF;
    case NMC_TALLY_F3D: return h->nvox;
    case NMC_TALLY_RD2D: return h->n2d;
    case NMC_TALLY_DETPHOT2D: return h->n2d;
    case NMC_TALLY_RD_SLOTS: return h->nslots;
    case NMC_TALLY_RD_R: return h->rd_bins > 0 ? (size_t)h->rd_bins + 1 : 0;
    default: return 0;
  }
}

nmc_status nmc_get_tally_f64(nmc_handle* h, int32_t which, double* out, size_t n) {
  if (!h || !out) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  const size_t want = nmc_tally_size(h, which);
  if (want == 0 || n != want) return fail(h, NMC_EINVAL, "tally not produced by this kind, or wrong size");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  const double* carry = which == NMC_TALLY_J ? h->c_J
                        : which == NMC_TALLY_F ? h->c_F
                        : which == NMC_TALLY_F3D ? h->c_F3D
                        : which == NMC_TALLY_RD2D ? h->c_Rd2D
                        : which == NMC_TALLY_DETPHOT2D ? h->c_Det
                        : which == NMC_TALLY_RD_R  ? h->c_rdr
                                                   : h->c_slots;
  std::vector<double> c(carry ? n : 0);
  if (carry) NMC_CUDA(h, cudaMemcpy(c.data(), carry, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (which == NMC_TALLY_DETPHOT2D) {
    std::vector<unsigned int> tmp(n);
    NMC_CUDA(h, cudaMemcpy(tmp.data(), h->d_Det, n * 4, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < n; ++k) out[k] = (double)tmp[k] + (carry ? c[k] : 0.0);
    return NMC_OK;
  }
  const unsigned long long* src = which == NMC_TALLY_J ? h->d_J
                                  : which == NMC_TALLY_F ? h->d_F
                                  : which == NMC_TALLY_F3D ? h->d_F3D
                                  : which == NMC_TALLY_RD2D ? h->d_Rd2D
                                  : which == NMC_TALLY_RD_R  ? h->d_rdr
                                                             : h->d_slots;
  std::vector<unsigned long long> tmp(n);
  NMC_CUDA(h, cudaMemcpy(tmp.data(), src, n * 8, cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < n; ++k) out[k] = (double)tmp[k] * nmc::kUnfix + (carry ? c[k] : 0.0);
  return NMC_OK;
}

nmc_status nmc_get_compute_results(nmc_handle* h, float* J, float* F, float* F3D, float* SAE,
                                   float* Rd, float* Rd2D, int32_t* DetPhot2D, float* PolXX,
                                   float* PolXY, float* PolYX, float* PolYY, float* Phase0,
                                   float* Phase1, float* Phase2, float* Phase3, float* PolVsScatt) {
  (void)PolXX, (void)PolXY, (void)PolYX, (void)PolYY, (void)Phase0, (void)Phase1, (void)Phase2,
      (void)Phase3, (void)PolVsScatt;
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  float* dst[kStN] = {nullptr};
  if (h->sim == NMC_SIM_MCSUB) {
    dst[kStJ] = J;
    dst[kStF] = F;
    dst[kStSums] = SAE;
  } else {
    dst[kStF3D] = F3D;
    dst[kStSlots] = Rd;
    dst[kStRd2D] = Rd2D;
    if (h->sim == NMC_SIM_MCXYZ) dst[kStDet] = reinterpret_cast<float*>(DetPhot2D);
  }
  unsigned mask = 0;
  for (int k = 0; k < kStN; ++k)
    if (dst[k] && h->st_len[k]) mask |= 1u << k;
  if (!mask) return NMC_OK;
  cudaGraphExec_t exec = nullptr;
  if ((st = reduce_graph(h, mask, &exec)) != NMC_OK) return st;
  NMC_CUDA(h, cudaGraphLaunch(exec, h->stream));
  if ((st = wait_stream(h)) != NMC_OK) return st;
  for (int k = 0; k < kStN; ++k) {
    if (!(mask >> k & 1u)) continue;
    const float* src = h->h_stage + h->st_off[k];
    const size_t n = h->st_len[k];
    if (k == kStSums) {
      DevSums s;
      std::memcpy(&s, src, sizeof s);
      SAE[0] += (float)(s.S * nmc::kUnfix + s.carry[0]);
      SAE[1] += (float)(s.A * nmc::kUnfix + s.carry[1]);
      SAE[2] += (float)(s.E * nmc::kUnfix + s.carry[2]);
    } else if (k == kStDet) {
      const unsigned int* c = reinterpret_cast<const unsigned int*>(src);
      for (size_t i = 0; i < n; ++i) DetPhot2D[i] += (int32_t)c[i];
    } else {
      float* d = dst[k];
      for (size_t i = 0; i < n; ++i) d[i] += src[i];
    }
  }
  return NMC_OK;
}

nmc_status nmc_get_summary(nmc_handle* h, nmc_summary* out) {
  if (!h || !out) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  std::memset(out, 0, sizeof *out);
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  DevSums s;
  NMC_CUDA(h, cudaMemcpy(&s, h->d_sums, sizeof s, cudaMemcpyDeviceToHost));
  out->photons = s.photons;
  out->substeps = s.substeps;
  out->scatters = s.scatters;
  out->S = s.S * nmc::kUnfix + s.carry[0];
  out->A = s.A * nmc::kUnfix + s.carry[1];
  out->E = s.E * nmc::kUnfix + s.carry[2];
  out->rd_sum = s.rd * nmc::kUnfix + s.carry[3];
  out->rd_sumsq = s.rd_sumsq;
  out->kernel_ms = h->kernel_ms;
  out->launches = h->launches;
  out->device_flags = s.flags;
  return NMC_OK;
}

nmc_status nmc_run_sweep(nmc_handle* h, const nmc_sweep_set* sets, int32_t n_sets, double* out,
                         double* J) {
  if (!h || !sets || !out) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (h->sim != NMC_SIM_MCSUB) return fail(h, NMC_EINVAL, "sweeps run on an NMC_SIM_MCSUB handle");
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  if (n_sets < 1 || n_sets > 1024) return fail(h, NMC_EINVAL, "n_sets must be in [1, 1024]");
  if (h->ext.rng != NMC_RNG_PHILOX) return fail(h, NMC_EINVAL, "sweeps use the Philox streams");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  const int bins = h->ext.sub_bins, nJ = bins + 1;
  std::vector<nmc::SweepSetDev> hs(n_sets);
  std::vector<unsigned long long> prefix(n_sets + 1, 0ull);
  // queue order: decreasing estimated cost per photon, mu_t / mu_a (the
  // interactions before the weight decays); results do not depend on it
  std::vector<uint32_t> order(n_sets);
  for (int s = 0; s < n_sets; ++s) order[s] = (uint32_t)s;
  auto est = [&](uint32_t s) {  // invalid sets are rejected below; keep the ordering strict
    const double a = sets[s].mua, b = sets[s].mus, e = (a + b) / std::max(a, 1e-6);
    return std::isfinite(e) ? e : 0.0;
  };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return est(a) > est(b); });
  for (int k = 0; k < n_sets; ++k) {
    const int s = (int)order[k];
    const nmc_sweep_set& q = sets[s];
    const float vals[] = {q.mua, q.mus, q.g, q.gf, q.af, q.gb, q.ab, q.cc, q.n1, q.n2};
    for (float v : vals)
      if (!std::isfinite(v)) return fail(h, NMC_EINVAL, "sweep set with a non-finite parameter");
    if (q.mua < 0.f || q.mus < 0.f || !(q.mua + q.mus > 0.f) || !(q.n1 > 0.f) || !(q.n2 > 0.f))
      return fail(h, NMC_EINVAL, "sweep set needs mua, mus >= 0, mua + mus > 0 and n1, n2 > 0");
    if (q.photons > (1ull << 31))  // per-set fixed-point sums stay below 2^63
      return fail(h, NMC_EINVAL, "at most 2^31 photons per sweep set and call");
    nmc_tissue_params tp{};
    tp.muav[1] = q.mua;
    tp.musv[1] = q.mus;
    tp.gv[1] = q.g;
    tp.gf[1] = q.gf;
    tp.af[1] = q.af;
    tp.gb[1] = q.gb;
    tp.ab[1] = q.ab;
    tp.CC[1] = q.cc;
    nmc::SweepSetDev& d = hs[k];
    d = nmc::SweepSetDev{};
    d.id = (unsigned int)s;
    d.mut = q.mua + q.mus;
    d.albedo = q.mus / d.mut;
    d.n1 = q.n1;
    d.n2 = q.n2;
    float t = q.n1 / q.n2;  // kernels.metal:118-120
    t = (1.f - t) / (1.f + t);
    d.rsp = t * t;
    d.first = q.first_photon;
    d.ph = nmc::phase_const(tp, 1);
    prefix[k + 1] = prefix[k] + q.photons;
  }
  nmc::SweepParams p{};
  p.nsets = n_sets;
  p.total = prefix[n_sets];
  p.bins = bins;
  p.idr = (float)(1.0 / h->ext.sub_dr);
  p.mcflag = h->ext.sub_mcflag;
  p.boundaryflag = h->ext.sub_boundaryflag;
  p.radius = h->ext.sub_radius;
  p.waist = h->ext.sub_waist;
  p.zfocus = h->ext.sub_zfocus;
  p.xs = h->ext.sub_xs;
  p.ys = h->ext.sub_ys;
  p.zs = h->ext.sub_zs;
  p.k0 = (uint32_t)h->ext.seed;
  p.k1 = (uint32_t)(h->ext.seed >> 32);
  p.phase_kind = h->sp.phase_kind;
  p.fast = h->sp.fast_math;
  p.step_cap = h->sp.step_cap;
  p.flags = &h->d_sums->flags;
  // device buffers for this sweep: sets, prefix, per-set sums, counter, J
  char* base = nullptr;
  const size_t b_sets = sizeof(nmc::SweepSetDev) * n_sets, b_pre = 8 * (n_sets + 1),
               b_sums = 8 * 5 * (size_t)n_sets, b_e2 = 8 * (size_t)n_sets, b_work = 8,
               b_J = J ? 8 * (size_t)nJ * n_sets : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t total_b = al(b_sets) + al(b_pre) + al(b_sums) + al(b_e2) + al(b_work) + al(b_J);
  if ((st = scratch(h, total_b, &base)) != NMC_OK) return st;
  char* cur = base;
  auto take = [&](size_t b) {
    char* r = cur;
    cur += al(b);
    return r;
  };
  p.sets = (const nmc::SweepSetDev*)take(b_sets);
  p.prefix = (const unsigned long long*)take(b_pre);
  p.sums = (unsigned long long*)take(b_sums);
  p.e2 = (double*)take(b_e2);
  p.work = (unsigned long long*)take(b_work);
  p.J = J ? (unsigned long long*)take(b_J) : nullptr;
  if (cudaMemcpyAsync((void*)p.sets, hs.data(), b_sets, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void*)p.prefix, prefix.data(), b_pre, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      // sums, e2, counter and J are contiguous: clear them together
      cudaMemsetAsync(p.sums, 0, al(b_sums) + al(b_e2) + al(b_work) + al(b_J), h->stream) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep buffer set-up");
  const int block = h->ext.block_size > 0 ? h->ext.block_size : 256;
  int per_sm = 0;
  if (nmc::sweep_occupancy(p, block, &per_sm) != cudaSuccess || per_sm < 1)
    return fail(h, NMC_EDEVICE, "sweep kernel does not fit on an SM");
  if (h->ext.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)h->ext.blocks_per_sm);
  uint64_t grid = (uint64_t)h->nsm * per_sm;
  grid = std::max<uint64_t>(1, std::min<uint64_t>(grid, (p.total + block - 1) / block));
  EventPair ev = get_pair(h);
  cudaEventRecord(ev.a, h->stream);
  if (p.total > 0 && nmc::launch_sweep(p, (int)grid, block, h->stream) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep launch");
  cudaEventRecord(ev.b, h->stream);
  h->pending.push_back(ev);
  ++h->launches;
  st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  std::vector<unsigned long long> sums(5 * (size_t)n_sets);
  std::vector<double> e2(n_sets);
  if (cudaMemcpy(sums.data(), p.sums, b_sums, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(e2.data(), p.e2, b_e2, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep results");
  if (J) {
    std::vector<unsigned long long> hj((size_t)nJ * n_sets);
    if (cudaMemcpy(hj.data(), p.J, b_J, cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(h, NMC_EDEVICE, "sweep J");
    for (size_t k = 0; k < hj.size(); ++k) J[k] = (double)hj[k] * nmc::kUnfix;
  }
  for (int s = 0; s < n_sets; ++s) {
    double* o = out + (size_t)s * NMC_SWEEP_FIELDS;
    const unsigned long long* u = &sums[5 * (size_t)s];
    const double n = (double)u[0];
    o[NMC_SWEEP_PHOTONS] = n;
    o[NMC_SWEEP_HOPS] = (double)u[1];
    o[NMC_SWEEP_S] = (double)u[2] * nmc::kUnfix;
    o[NMC_SWEEP_A] = (double)u[3] * nmc::kUnfix;
    o[NMC_SWEEP_E] = (double)u[4] * nmc::kUnfix;
    o[NMC_SWEEP_E2] = e2[s];
    const double me = n > 0 ? o[NMC_SWEEP_E] / n : 0.0;
    o[NMC_SWEEP_RD] = n > 0 ? (o[NMC_SWEEP_S] + o[NMC_SWEEP_E]) / n : 0.0;
    o[NMC_SWEEP_RD_SE] = n > 1 ? std::sqrt(std::max(0.0, e2[s] / n - me * me) / n) : 0.0;
  }
  return st;
}

nmc_status nmc_run_sweep_tissues(nmc_handle* h, const nmc_tissue_params* tables, const uint64_t* photons,
                                 const uint64_t* first_photon, int32_t n_sets, double* out) {
  if (!h || !tables || !photons || !out) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (h->sim != NMC_SIM_MCXYZ && h->sim != NMC_SIM_MCXYZ_TT)
    return fail(h, NMC_EINVAL, "tissue sweeps run on an NMC_SIM_MCXYZ or NMC_SIM_MCXYZ_TT handle");
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  if (n_sets < 1 || n_sets > 65536) return fail(h, NMC_EINVAL, "n_sets must be in [1, 65536]");
  if (h->ext.rng != NMC_RNG_PHILOX) return fail(h, NMC_EINVAL, "sweeps use the Philox streams");
  if (h->voxel_mode) return fail(h, NMC_ESTATE, "tissue sweeps read the tissue map, not per-voxel properties");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  const size_t nt = (size_t)n_sets * NMC_NTISS;
  std::vector<float4> core(nt);
  std::vector<nmc::PhaseConst> phase(nt);
  std::vector<unsigned long long> prefix(n_sets + 1, 0ull), first(n_sets, 0ull);
  // The work queue hands out the sets in decreasing order of an estimated
  // cost per photon, so that the long-lived photons of the costliest sets
  // start first and the launch does not end waiting on them.  Estimate:
  // sub-steps along a photon's path grow with (mus + 1/d) / mua in the
  // tissues it crosses, weighted by each tissue's share of the map.  The
  // order changes no result: a photon's stream is a function of its set and
  // its index within the set, and the tallies are integer sums.
  std::vector<double> cost(n_sets, 0.0);
  const double inv_d = 1.0 / std::min(h->rp.dx, std::min(h->rp.dy, h->rp.dz));
  for (int s = 0; s < n_sets; ++s) {
    if ((st = check_tissues(h, &tables[s], h->tiss_used, s)) != NMC_OK) return st;
    if (photons[s] > (1ull << 31))  // per-set fixed-point sums stay below 2^63
      return fail(h, NMC_EINVAL, "at most 2^31 photons per sweep set and call");
    nmc::XyzParams tmp{};
    nmc::fill_xyz(tmp, h->rp, tables[s], h->ext, h->sim);
    for (int t = 0; t < NMC_NTISS; ++t) {
      core[(size_t)s * NMC_NTISS + t] = tmp.core[t];
      phase[(size_t)s * NMC_NTISS + t] = tmp.phase[t];
      if (h->tiss_count[t])
        cost[s] += (double)h->tiss_count[t] * ((double)tables[s].musv[t] + inv_d) /
                   std::max((double)tables[s].muav[t], 1e-6);
    }
  }
  std::vector<uint32_t> order(n_sets);
  for (int s = 0; s < n_sets; ++s) order[s] = (uint32_t)s;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  for (int k = 0; k < n_sets; ++k) {  // queue slot k runs set order[k]
    if (first_photon) first[k] = first_photon[order[k]];
    prefix[k + 1] = prefix[k] + photons[order[k]];
  }
  nmc::XyzParams p = h->xp;
  const size_t b_core = sizeof(float4) * nt, b_ph = sizeof(nmc::PhaseConst) * nt, b_pre = 8 * (n_sets + 1),
               b_first = 8 * (size_t)n_sets, b_sums = sizeof(nmc::XyzSweepSums) * n_sets,
               b_order = 4 * (size_t)n_sets;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* base = nullptr;
  {
    const nmc_status sc =
        scratch(h, al(b_core) + al(b_ph) + al(b_pre) + al(b_first) + al(b_sums) + al(b_order), &base);
    if (sc != NMC_OK) return sc;
  }
  char* cur = base;
  auto take = [&](size_t b) {
    char* r = cur;
    cur += al(b);
    return r;
  };
  p.sw_core = (const float4*)take(b_core);
  p.sw_phase = (const nmc::PhaseConst*)take(b_ph);
  p.sw_prefix = (const unsigned long long*)take(b_pre);
  p.sw_first = (const unsigned long long*)take(b_first);
  p.sw_sums = (nmc::XyzSweepSums*)take(b_sums);
  p.sw_order = (const unsigned int*)take(b_order);
  p.sw_nsets = n_sets;
  p.first = 0;
  p.n = prefix[n_sets];
  p.trace = nmc::TraceParams{nullptr, nullptr, 0u};
  if (cudaMemcpyAsync((void*)p.sw_core, core.data(), b_core, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void*)p.sw_phase, phase.data(), b_ph, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void*)p.sw_prefix, prefix.data(), b_pre, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void*)p.sw_first, first.data(), b_first, cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync((void*)p.sw_order, order.data(), b_order, cudaMemcpyHostToDevice, h->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(p.sw_sums, 0, b_sums, h->stream) != cudaSuccess ||
      cudaMemsetAsync(&h->d_sums->work, 0, sizeof(unsigned long long), h->stream) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep buffer set-up");
  const bool tt = h->sim == NMC_SIM_MCXYZ_TT;
  const int block = h->ext.block_size > 0 ? h->ext.block_size : 256;
  int per_sm = 0;
  if (nmc::mcxyz_sweep_occupancy(tt, block, &per_sm) != cudaSuccess || per_sm < 1)
    return fail(h, NMC_EDEVICE, "sweep kernel does not fit on an SM");
  if (h->ext.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)h->ext.blocks_per_sm);
  uint64_t grid = (uint64_t)h->nsm * per_sm;
  grid = std::max<uint64_t>(1, std::min<uint64_t>(grid, (p.n + block - 1) / block));
  EventPair ev = get_pair(h);
  cudaEventRecord(ev.a, h->stream);
  if (p.n > 0 && nmc::launch_mcxyz_sweep(p, tt, (int)grid, block, h->stream) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep launch");
  cudaEventRecord(ev.b, h->stream);
  h->pending.push_back(ev);
  ++h->launches;
  st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  std::vector<nmc::XyzSweepSums> sums(n_sets);
  if (cudaMemcpy(sums.data(), p.sw_sums, b_sums, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "sweep results");
  for (int s = 0; s < n_sets; ++s) {
    double* o = out + (size_t)s * NMC_SWEEP_FIELDS;
    const nmc::XyzSweepSums& u = sums[s];
    const double n = (double)u.photons;
    o[NMC_SWEEP_PHOTONS] = n;
    o[NMC_SWEEP_HOPS] = (double)u.substeps;
    o[NMC_SWEEP_S] = 0.0;
    o[NMC_SWEEP_A] = (double)u.A * nmc::kUnfix;
    o[NMC_SWEEP_E] = (double)u.rd * nmc::kUnfix;
    o[NMC_SWEEP_E2] = u.rd2;
    const double me = n > 0 ? o[NMC_SWEEP_E] / n : 0.0;
    o[NMC_SWEEP_RD] = me;
    o[NMC_SWEEP_RD_SE] = n > 1 ? std::sqrt(std::max(0.0, u.rd2 / n - me * me) / n) : 0.0;
  }
  return st;
}

nmc_status nmc_set_voxel_props(nmc_handle* h, const float* mua, const float* mus, const float* g) {
  if (!h || !mua || !mus) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (h->sim != NMC_SIM_MCXYZ) return fail(h, NMC_EINVAL, "per-voxel media need an NMC_SIM_MCXYZ handle");
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  std::vector<float4> v(h->nvox);
  const float g1 = h->tp.gv[1];
  for (size_t k = 0; k < h->nvox; ++k) {
    const float a = mua[k], s = mus[k], gg = g ? g[k] : g1;
    if (!std::isfinite(a) || a < 0.f || !std::isfinite(s) || !(s > 0.f) || !std::isfinite(gg) || !(gg > -1.f) ||
        !(gg < 1.f)) {
      char msg[128];
      std::snprintf(msg, sizeof msg, "voxel %zu: need mua >= 0, mus > 0, -1 < g < 1 (got %g, %g, %g)", k, a, s, gg);
      return fail(h, NMC_EINVAL, msg);
    }
    v[k] = make_float4(a, s, (float)(1.0 / s), gg);
  }
  if (!h->d_vox) NMC_CUDA(h, cudaMalloc((void**)&h->d_vox, h->nvox * sizeof(float4)));
  NMC_CUDA(h, cudaMemcpy(h->d_vox, v.data(), h->nvox * sizeof(float4), cudaMemcpyHostToDevice));
  h->voxel_mode = true;
  h->adj_ready = false;
  return build_xyz(h);
}

nmc_status nmc_set_radial_tally(nmc_handle* h, int32_t bins, float dr) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  if (h->sim == NMC_SIM_MCSUB) return fail(h, NMC_EINVAL, "the radial tally is for voxel kinds (mcsub has J)");
  if (!h->prepared) return fail(h, NMC_ESTATE, "nmc_prepare has not been called");
  if (bins < 1 || bins > 65536 || !(dr > 0.f) || !std::isfinite(dr))
    return fail(h, NMC_EINVAL, "radial tally needs 1 <= bins <= 65536 and dr > 0");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  dfree(h->d_rdr);
  dfree(h->c_rdr);
  NMC_CUDA(h, cudaMalloc((void**)&h->d_rdr, ((size_t)bins + 1) * 8));
  NMC_CUDA(h, cudaMemset(h->d_rdr, 0, ((size_t)bins + 1) * 8));
  h->rd_bins = bins;
  h->rd_dr = dr;
  return build_xyz(h);
}

nmc_status nmc_adjoint_forward_ex(nmc_handle* h, uint64_t first, uint64_t n, uint64_t event_capacity,
                                  uint64_t deposit_capacity) {
  if (!h) return NMC_EINVAL;
  NMC_ON_DEVICE(h);
  if (!h->prepared || !h->voxel_mode) return fail(h, NMC_ESTATE, "the adjoint needs nmc_set_voxel_props");
  if (h->rd_bins < 1) return fail(h, NMC_ESTATE, "the adjoint differentiates the radial tally: nmc_set_radial_tally");
  if (n >= 0xFFFFFFFFull || event_capacity == 0 || event_capacity >= 0xFFFFFFFFull)
    return fail(h, NMC_EINVAL, "adjoint runs need n < 2^32 photons and 0 < event_capacity < 2^32");
  // every thread of the launch holds one chunk at a time: the pool adds one
  // chunk per thread to the records asked for, so the capacity counts records
  uint64_t chunks = 0;
  if (deposit_capacity > 0) {
    const int block = h->ext.block_size > 0 ? h->ext.block_size : 256;
    int per_sm = 0;
    NMC_CUDA(h, nmc::mcxyz_voxel_occupancy(nmc::kRecord, false, block, &per_sm));
    const uint64_t threads = (uint64_t)h->nsm * (uint64_t)std::max(per_sm, 1) * (uint64_t)block;
    chunks = (deposit_capacity + nmc::kDepChunk - 1) / nmc::kDepChunk + threads;
  }
  if (chunks >= 0xFFFFFFF0ull) return fail(h, NMC_EINVAL, "deposit_capacity too large");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  if (h->ev_cap < event_capacity) {
    dfree(h->d_ev);
    NMC_CUDA(h, cudaMalloc((void**)&h->d_ev, event_capacity * sizeof(nmc::AdjEvent)));
    h->ev_cap = event_capacity;
  }
  h->ev_limit = event_capacity;
  if (!h->d_evcount) NMC_CUDA(h, cudaMalloc((void**)&h->d_evcount, sizeof(unsigned long long)));
  NMC_CUDA(h, cudaMemsetAsync(h->d_evcount, 0, sizeof(unsigned long long), h->stream));
  h->dl_ok = false;
  bool list = chunks > 0;
  if (list && chunks > h->dl_chunks) {  // grow-only, like the event list
    dfree(h->d_dl);
    dfree(h->d_dlfill);
    h->dl_chunks = 0;
    // the list only saves time: without the memory the run keeps none
    if (cudaMalloc((void**)&h->d_dl, chunks * nmc::kDepChunk * sizeof(uint2)) != cudaSuccess ||
        cudaMalloc((void**)&h->d_dlfill, chunks * sizeof(unsigned int)) != cudaSuccess) {
      (void)cudaGetLastError();
      dfree(h->d_dl);
      dfree(h->d_dlfill);
      list = false;
    } else {
      h->dl_chunks = (unsigned int)chunks;
    }
  }
  h->dl_req = list ? (unsigned int)chunks : 0;
  if (list && !h->d_dlnext) NMC_CUDA(h, cudaMalloc((void**)&h->d_dlnext, sizeof(unsigned long long)));
  if (list) NMC_CUDA(h, cudaMemsetAsync(h->d_dlnext, 0, sizeof(unsigned long long), h->stream));
  AdjArgs a{0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  a.deposit_list = list;
  st = launch(h, first, n, nullptr, nullptr, 0, &a);
  if (st == NMC_OK) st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  unsigned long long cnt = 0;
  NMC_CUDA(h, cudaMemcpy(&cnt, h->d_evcount, sizeof cnt, cudaMemcpyDeviceToHost));
  if (cnt > h->ev_limit) {
    h->adj_ready = false;
    char msg[128];
    std::snprintf(msg, sizeof msg, "%llu detection events exceed event_capacity %llu", cnt,
                  (unsigned long long)h->ev_limit);
    return fail(h, NMC_EINVAL, msg);
  }
  if (list) {  // a list that ran out of chunks is dropped: the backward replays the scores instead
    unsigned long long used = 0;
    NMC_CUDA(h, cudaMemcpy(&used, h->d_dlnext, sizeof used, cudaMemcpyDeviceToHost));
    h->dl_ok = used <= h->dl_req;
    h->dl_used = (unsigned int)std::min<unsigned long long>(used, h->dl_req);
  }
  h->adj_first = first;
  h->adj_n = n;
  h->adj_ready = true;
  return st;
}

nmc_status nmc_adjoint_forward(nmc_handle* h, uint64_t first, uint64_t n, uint64_t event_capacity) {
  return nmc_adjoint_forward_ex(h, first, n, event_capacity, 0);
}

int32_t nmc_adjoint_deposit_list_complete(nmc_handle* h) { return h && h->adj_ready && h->dl_ok ? 1 : 0; }

nmc_status nmc_adjoint_backward_ex(nmc_handle* h, const float* grad_rd_r, const float* grad_absorbed,
                                   double* grad_mua, double* grad_mus, double* grad_g) {
  if (!h || (!grad_rd_r && !grad_absorbed)) return fail(h, NMC_EINVAL, "null argument");
  NMC_ON_DEVICE(h);
  if (!h->adj_ready) return fail(h, NMC_ESTATE, "nmc_adjoint_forward has not completed");
  nmc_status st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  unsigned long long cnt = 0;
  NMC_CUDA(h, cudaMemcpy(&cnt, h->d_evcount, sizeof cnt, cudaMemcpyDeviceToHost));
  const size_t nb = (size_t)h->rd_bins + 1, nv = h->nvox;
  const size_t bD = h->adj_n * 4, bG = nb * 4, bF = grad_absorbed ? nv * 4 : 0, bg = nv * 8;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* base = nullptr;
  if ((st = scratch(h, al(bD) + al(bG) + al(bF) + 3 * al(bg), &base)) != NMC_OK) return st;
  float* D = (float*)base;
  float* G = (float*)(base + al(bD));
  float* GF = grad_absorbed ? (float*)(base + al(bD) + al(bG)) : nullptr;
  double* gL = (double*)(base + al(bD) + al(bG) + al(bF));
  double* gM = (double*)((char*)gL + al(bg));
  double* gQ = (double*)((char*)gM + al(bg));
  bool ok = cudaMemsetAsync(gL, 0, 3 * al(bg), h->stream) == cudaSuccess;
  ok = ok && (grad_rd_r ? cudaMemcpyAsync(G, grad_rd_r, bG, cudaMemcpyHostToDevice, h->stream)
                        : cudaMemsetAsync(G, 0, bG, h->stream)) == cudaSuccess;
  if (GF) ok = ok && cudaMemcpyAsync(GF, grad_absorbed, bF, cudaMemcpyHostToDevice, h->stream) == cudaSuccess;
  if (!ok) return fail(h, NMC_EDEVICE, "adjoint set-up");
  if (GF && h->dl_ok) {
    // deposits score too: each photon's total score from the events and
    // the record pass's deposit list
    if (cudaMemsetAsync(D, 0, bD, h->stream) != cudaSuccess ||
        nmc::launch_adjoint_scores(h->d_ev, (unsigned int)cnt, G, D, h->stream) != cudaSuccess ||
        nmc::launch_deposit_scores(h->d_dl, h->d_dlfill, h->dl_used, GF, D, h->adj_n, h->stream) != cudaSuccess)
      return fail(h, NMC_EDEVICE, "adjoint scores");
  } else if (GF) {
    // deposits score too: a first replay gives every photon its total score
    AdjArgs a{2, D, G, GF, nullptr, nullptr, nullptr};
    st = launch(h, h->adj_first, h->adj_n, nullptr, nullptr, 0, &a);
    if (st != NMC_OK) return st;
  } else {
    // detection scores only: from the events the record pass kept
    if (cudaMemsetAsync(D, 0, bD, h->stream) != cudaSuccess ||
        nmc::launch_adjoint_scores(h->d_ev, (unsigned int)cnt, G, D, h->stream) != cudaSuccess)
      return fail(h, NMC_EDEVICE, "adjoint scores");
  }
  AdjArgs a{1, D, G, GF, gL, gM, gQ};
  st = launch(h, h->adj_first, h->adj_n, nullptr, nullptr, 0, &a);
  if (st == NMC_OK) st = sync_all(h);
  if (st != NMC_OK && st != NMC_ESTEPCAP) return st;
  std::vector<double> L(nv), M(nv), Q(nv);
  if (cudaMemcpy(L.data(), gL, bg, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(M.data(), gM, bg, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(Q.data(), gQ, bg, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(h, NMC_EDEVICE, "adjoint results");
  for (size_t k = 0; k < nv; ++k) {
    if (grad_mua) grad_mua[k] = -L[k];
    if (grad_mus) grad_mus[k] = M[k];
    if (grad_g) grad_g[k] = Q[k];
  }
  return st;
}

nmc_status nmc_adjoint_backward(nmc_handle* h, const float* grad_rd_r, double* grad_mua, double* grad_mus,
                                double* grad_g) {
  if (!h || !grad_rd_r) return fail(h, NMC_EINVAL, "null argument");
  return nmc_adjoint_backward_ex(h, grad_rd_r, nullptr, grad_mua, grad_mus, grad_g);
}

void* nmc_stream(nmc_handle* h) { return h ? (void*)h->stream : nullptr; }

const char* nmc_last_error(const nmc_handle* h) { return h ? h->err.c_str() : "null handle"; }

void nmc_destroy(nmc_handle* h) {
  if (!h) return;
  nmc::DeviceScope dev(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_buffers(h);
  if (h->d_sums) cudaFree(h->d_sums);
  for (EventPair& p : h->pool) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (EventPair& p : h->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->l2_raised) cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, h->l2_prev);
  delete h;
}

}  // extern "C"
