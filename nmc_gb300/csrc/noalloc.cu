// noalloc.cu - voxel transport for callers that cannot allocate device memory.
//
// Some hosts own every byte of device memory themselves: an application
// that sub-allocates from its own memory pool, a plugin process inside a
// larger runtime with a fixed memory budget, or a real-time loop where an
// allocation's latency or failure is not allowed.  Such a caller hands over
// its own device buffers for the inputs and outputs and cannot let the
// library call cudaMalloc.  nmc_mcxyz_run_noalloc serves it: the working
// memory the transport needs beyond the caller's buffers (the u64
// fixed-point tallies, the photon counter and the totals) is one file-scope
// __device__ array of fixed size, so the call allocates nothing.
//
// Costs of that choice, all documented in nmc_abi.h:
//  * the array (about 17 MB) exists on every GPU that loads this library,
//    for as long as the process lives;
//  * grids are limited to NMC_NOALLOC_MAX_VOXELS voxels and
//    NMC_NOALLOC_MAX_MAP columns (Nx*Ny);
//  * every call uses the same array: the call clears what must start at
//    zero, and calls whose GPU work overlaps (e.g. on two streams) race.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "nmc_abi.h"

namespace {

constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  unsigned long long F3D[NMC_NOALLOC_MAX_VOXELS];
  unsigned long long Rd2D[NMC_NOALLOC_MAX_MAP];
  unsigned int Det[NMC_NOALLOC_MAX_MAP];
  unsigned long long slot[1];
  nmc::DevSums sums;
  unsigned int tissue_mask;
  unsigned int pad;
};

static __device__ __align__(256) NoAllocScratch g_scratch;

// Device address of g_scratch, looked up once per device (host code may not
// use the symbol's name as an address).
NoAllocScratch* g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

nmc_status scratch_on(int dev, NoAllocScratch** out) {
  if (dev < 0 || dev >= kMaxDevices) return NMC_EDEVICE;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return NMC_EDEVICE;
    g_scratch_addr[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_addr[dev];
  return NMC_OK;
}

// Bit t set for every tissue id t present in the map (ids >= 31 set bit 31).
__global__ void tissue_mask_kernel(const uint8_t* __restrict__ v, size_t n, unsigned int* mask) {
  unsigned int m = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const unsigned int t = v[k];
    m |= t < 31 ? (1u << t) : 0x80000000u;
  }
  m = __reduce_or_sync(0xFFFFFFFFu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicOr(mask, m);
}

__global__ void finish_kernel(const NoAllocScratch* __restrict__ s, size_t nvox, size_t n2d, float* F3D,
                              float* Rd2D, uint32_t* Det, double* totals) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (size_t k = t0; k < nvox; k += stride) F3D[k] = (float)((double)s->F3D[k] * nmc::kUnfix);
  for (size_t k = t0; k < n2d; k += stride) {
    if (Rd2D) Rd2D[k] = (float)((double)s->Rd2D[k] * nmc::kUnfix);
    if (Det) Det[k] = s->Det[k];
  }
  if (t0 == 0 && totals) {
    totals[0] = (double)s->sums.photons;
    totals[1] = (double)s->sums.substeps;
    totals[2] = (double)s->sums.scatters;
    totals[3] = (double)s->sums.A * nmc::kUnfix;
    totals[4] = (double)s->sums.rd * nmc::kUnfix;
    totals[5] = s->sums.rd_sumsq;
    totals[6] = (double)s->sums.flags;
    totals[7] = 0.0;
  }
}

}  // namespace

extern "C" nmc_status nmc_mcxyz_run_noalloc(const nmc_run_params* rp, const nmc_tissue_params* tp,
                                            const nmc_ext* ext, const uint8_t* d_v, uint64_t first_photon,
                                            uint64_t n_photons, float* d_F3D, float* d_Rd2D,
                                            uint32_t* d_DetPhot2D, double* d_totals, void* stream) {
  if (!rp || !tp || !ext || !d_v || !d_F3D) return NMC_EINVAL;
  // The u64 fixed-point sums and u32 counts of one call are never folded
  // (nmc_run folds every 2^31 photons), so one call takes at most 2^31.
  if (n_photons > NMC_NOALLOC_MAX_PHOTONS || first_photon > UINT64_MAX - n_photons) return NMC_EINVAL;
  if (ext->size != sizeof(nmc_ext) || ext->photons_per_dispatch == 0) return NMC_EINVAL;
  if (ext->block_size < 0 || ext->block_size > 1024 || ext->blocks_per_sm < 0) return NMC_EINVAL;
  if (ext->rng != NMC_RNG_PHILOX && ext->rng != NMC_RNG_TAUS_REF) return NMC_EINVAL;
  if (rp->mckernelflag != NMC_SIM_MCXYZ && rp->mckernelflag != NMC_SIM_MCXYZ_TT) return NMC_EINVAL;
  if (rp->Nx <= 0 || rp->Ny <= 0 || rp->Nz <= 0) return NMC_EINVAL;
  const size_t nvox = (size_t)rp->Nx * rp->Ny * rp->Nz, n2d = (size_t)rp->Nx * rp->Ny;
  if (nvox > NMC_NOALLOC_MAX_VOXELS || n2d > NMC_NOALLOC_MAX_MAP) return NMC_EINVAL;  // grid too large
  if (!(rp->dx > 0.f) || !(rp->dy > 0.f) || !(rp->dz > 0.f) || !std::isfinite(rp->dx) ||
      !std::isfinite(rp->dy) || !std::isfinite(rp->dz))
    return NMC_EINVAL;
  if (rp->boundaryflag < 0 || rp->boundaryflag > 2 || (rp->det_state != 0 && rp->det_state != 1))
    return NMC_EINVAL;
  if (!(rp->n1 > 0.f) || !(rp->n2 > 0.f)) return NMC_EINVAL;

  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NMC_EDEVICE;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return NMC_EDEVICE;
  NoAllocScratch* S = nullptr;
  nmc_status st = scratch_on(dev, &S);
  if (st != NMC_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // tissue ids must index the 19-entry table and name usable tissues
  unsigned int mask = 0;
  if (cudaMemsetAsync(&S->tissue_mask, 0, sizeof(unsigned int), s) != cudaSuccess) return NMC_EDEVICE;
  tissue_mask_kernel<<<nsm * 4, 256, 0, s>>>(d_v, nvox, &S->tissue_mask);
  if (cudaMemcpyAsync(&mask, &S->tissue_mask, sizeof mask, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return NMC_EDEVICE;
  for (int t = 0; t < 32; ++t) {
    if (!(mask & (1u << t))) continue;
    if (t >= NMC_NTISS || !nmc::tissue_usable(*tp, t)) return NMC_EINVAL;
  }

  // the working memory starts at zero on every call
  if (cudaMemsetAsync(S->F3D, 0, nvox * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(S->Rd2D, 0, n2d * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(S->Det, 0, n2d * sizeof(unsigned int), s) != cudaSuccess ||
      cudaMemsetAsync(S->slot, 0, sizeof S->slot, s) != cudaSuccess ||
      cudaMemsetAsync(&S->sums, 0, sizeof(nmc::DevSums), s) != cudaSuccess)
    return NMC_EDEVICE;

  if (n_photons > 0) {
    nmc::XyzParams p{};
    nmc::fill_xyz(p, *rp, *tp, *ext, rp->mckernelflag);
    p.V = d_v;
    p.F3D = S->F3D;
    p.Rd2D = S->Rd2D;
    p.Det2D = S->Det;
    p.rd_slots = S->slot;
    p.nslots = 1;
    p.sums = &S->sums;
    p.first = first_photon;
    p.n = n_photons;
    p.trace = nmc::TraceParams{nullptr, nullptr, 0};
    const bool tt = rp->mckernelflag == NMC_SIM_MCXYZ_TT;
    // the launch shape nmc_run takes from the same nmc_ext
    const int block = ext->block_size > 0 ? ext->block_size : 256;
    int per_sm = 0;
    if (nmc::mcxyz_occupancy(tt, false, block, &per_sm) != cudaSuccess) return NMC_EDEVICE;
    if (ext->blocks_per_sm > 0) per_sm = std::min(per_sm, (int)ext->blocks_per_sm);
    if (per_sm < 1) return NMC_EDEVICE;
    uint64_t grid = (uint64_t)nsm * per_sm;
    if (grid > (n_photons + block - 1) / block) grid = (n_photons + block - 1) / block;
    if (nmc::launch_mcxyz(p, tt, false, (int)grid, block, s) != cudaSuccess) return NMC_EDEVICE;
  }
  finish_kernel<<<nsm * 4, 256, 0, s>>>(S, nvox, n2d, d_F3D, d_Rd2D, d_DetPhot2D, d_totals);
  return cudaGetLastError() == cudaSuccess ? NMC_OK : NMC_EDEVICE;
}
