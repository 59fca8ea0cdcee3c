// mcxyz.cu - the voxel transport kernel for tissue-map media (the
// reference's MCXYZKernel / MCXYZKernelTT model, kernels.metal:321-1118):
// instantiations and launchers.  The kernel itself is in mcxyz_kernel.cuh.
#include "mcxyz_kernel.cuh"

namespace nmc {
namespace {

template <bool TT, bool TRACE, bool FAST>
const void* kernel_for(uint32_t rng_kind) {
  if (rng_kind == NMC_RNG_TAUS_REF) return (const void*)mcxyz_kernel<TT, TausRng, TRACE, FAST, kTissue>;
  return (const void*)mcxyz_kernel<TT, PhiloxRng<TT>, TRACE, FAST, kTissue>;
}

const void* pick(bool tt, bool trace, bool fast, uint32_t rng_kind) {
  if (tt) {
    if (trace) return fast ? kernel_for<true, true, true>(rng_kind) : kernel_for<true, true, false>(rng_kind);
    return fast ? kernel_for<true, false, true>(rng_kind) : kernel_for<true, false, false>(rng_kind);
  }
  if (trace) return fast ? kernel_for<false, true, true>(rng_kind) : kernel_for<false, true, false>(rng_kind);
  return fast ? kernel_for<false, false, true>(rng_kind) : kernel_for<false, false, false>(rng_kind);
}

}  // namespace

cudaError_t launch_mcxyz(const XyzParams& p, bool two_term, bool trace, int grid, int block,
                         cudaStream_t stream) {
  const void* f = pick(two_term, trace, p.fast_math != 0, p.rng.kind);
  void* args[] = {(void*)&p};
  return cudaLaunchKernel(f, dim3(grid), dim3(block), args, 0, stream);
}

cudaError_t mcxyz_occupancy(bool two_term, bool trace, int block, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pick(two_term, trace, true, 0),
                                                       block, 0);
}

}  // namespace nmc
