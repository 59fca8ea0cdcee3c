// mcxyz_sweep.cu - batched sweep on a voxel tissue map: many tissue tables
// (one per set, e.g. one per wavelength) with uneven photon budgets in one
// persistent launch.  Replaces the reference's one `nmc` process per
// wavelength (NMC-samples/example3.ipynb cell 5 rewrites _H.mci and relaunches
// nmc for each wavelength on the same skin-vessel map).  The kernel itself is
// in mcxyz_kernel.cuh (mode kSweep): the photon queue runs over the
// concatenated budgets, a photon finds its set by binary search over the
// budget prefix sums, and reads that set's table through the read-only path.
#include "mcxyz_kernel.cuh"

namespace nmc {
namespace {

const void* pick_sweep(bool tt, bool fast) {
  if (tt)
    return fast ? (const void*)mcxyz_kernel<true, PhiloxRng<true>, false, true, kSweep>
                : (const void*)mcxyz_kernel<true, PhiloxRng<true>, false, false, kSweep>;
  return fast ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, true, kSweep>
              : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false, false, kSweep>;
}

}  // namespace

cudaError_t launch_mcxyz_sweep(const XyzParams& p, bool two_term, int grid, int block, cudaStream_t stream) {
  const void* f = pick_sweep(two_term, p.fast_math != 0);
  void* args[] = {(void*)&p};
  return cudaLaunchKernel(f, dim3(grid), dim3(block), args, 0, stream);
}

cudaError_t mcxyz_sweep_occupancy(bool two_term, int block, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pick_sweep(two_term, true), block, 0);
}

}  // namespace nmc
