// mcxyz_voxel.cu - the voxel transport kernel for media with per-voxel
// optical properties (no reference counterpart: the reference indexes at most
// 18 tissue types through a uint8 map, definitions.h:57), forward and
// perturbation Monte Carlo adjoint.  The kernel itself is in mcxyz_kernel.cuh.
#include "mcxyz_kernel.cuh"

namespace nmc {
namespace {

const void* pick_voxel(int mode, bool trace, bool fast) {
  if (mode == kAdjoint)
    return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, true, kAdjoint>
                : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, false, kAdjoint>;
  if (mode == kRecord)
    return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, true, kRecord>
                : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, false, kRecord>;
  if (mode == kScore)
    return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, true, kScore>
                : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, false, kScore>;
  if (trace)
    return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, true, true, kVoxel>
                : (const void*)mcxyz_kernel<false, PhiloxRng<false>, true, false, kVoxel>;
  return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, true, kVoxel>
              : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, false, kVoxel>;
}

__global__ void adjoint_scores_kernel(const AdjEvent* __restrict__ ev, unsigned int n, const float* __restrict__ G,
                                      float* __restrict__ D) {
  for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const AdjEvent e = ev[k];
    const float v = G[e.bin] * e.w;
    if (v != 0.f) atomicAdd(D + e.photon, v);
  }
}

// One thread per chunk of the deposit list: each photon's run of records
// (from its header to the next header or the chunk's end) adds its
// sum GF[voxel] * deposit to D[photon] with one atomic.  A chunk is 2 KB
// (256 records, 16-byte aligned) read two records at a time.
__global__ void deposit_scores_kernel(const uint2* __restrict__ pool, const unsigned int* __restrict__ fill,
                                      unsigned int n_chunks, const float* __restrict__ GF, float* __restrict__ D,
                                      unsigned long long n_photons) {
  static_assert(kDepChunk % 2 == 0, "records are read in pairs");
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_chunks; c += gridDim.x * blockDim.x) {
    const uint4* r = reinterpret_cast<const uint4*>(pool + (size_t)c * kDepChunk);
    const unsigned int n = min(fill[c], kDepChunk);
    unsigned int p = 0xFFFFFFFFu;
    float sum = 0.f;
    auto take = [&](unsigned int a, unsigned int b) {
      if (a == 0xFFFFFFFFu) {
        if (p < n_photons && sum != 0.f) atomicAdd(D + p, sum);
        p = b;
        sum = 0.f;
      } else {
        sum = fmaf(__ldg(GF + a), __uint_as_float(b), sum);
      }
    };
#pragma unroll 4
    for (unsigned int k = 0; k < n / 2; ++k) {
      const uint4 x = __ldg(r + k);
      take(x.x, x.y);
      take(x.z, x.w);
    }
    if (n & 1u) {
      const uint2 x = pool[(size_t)c * kDepChunk + n - 1];
      take(x.x, x.y);
    }
    if (p < n_photons && sum != 0.f) atomicAdd(D + p, sum);
  }
}

}  // namespace

cudaError_t launch_deposit_scores(const uint2* pool, const unsigned int* fill, unsigned int n_chunks,
                                  const float* GF, float* D, unsigned long long n_photons, cudaStream_t stream) {
  if (n_chunks == 0) return cudaSuccess;
  const int block = 256;
  const unsigned int grid = (n_chunks + block - 1) / block < 8192u ? (n_chunks + block - 1) / block : 8192u;
  deposit_scores_kernel<<<grid, block, 0, stream>>>(pool, fill, n_chunks, GF, D, n_photons);
  return cudaGetLastError();
}

cudaError_t launch_mcxyz_voxel(const XyzParams& p, int mode, bool trace, int grid, int block,
                               cudaStream_t stream) {
  const void* f = pick_voxel(mode, trace, p.fast_math != 0);
  void* args[] = {(void*)&p};
  return cudaLaunchKernel(f, dim3(grid), dim3(block), args, 0, stream);
}

cudaError_t mcxyz_voxel_occupancy(int mode, bool trace, int block, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pick_voxel(mode, trace, true), block, 0);
}

cudaError_t launch_adjoint_scores(const AdjEvent* ev, unsigned int n_ev, const float* G, float* D,
                                  cudaStream_t stream) {
  if (n_ev == 0) return cudaSuccess;
  const int block = 256;
  const unsigned int grid = (n_ev + block - 1) / block < 4096u ? (n_ev + block - 1) / block : 4096u;
  adjoint_scores_kernel<<<grid, block, 0, stream>>>(ev, n_ev, G, D);
  return cudaGetLastError();
}

}  // namespace nmc
