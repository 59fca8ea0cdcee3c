// sweep.cu - many parameter sets of the semi-infinite medium (MCSubKernel,
// kernels.metal:59-319) in one persistent launch.
//
// The reference sweeps wavelengths by rewriting its input files and starting
// one process (one pipeline, ten blocking dispatches) per wavelength
// (NMC-samples/example3.ipynb cell 5).  Here every set's photon budget is a
// slice of one global photon index space: threads take photon indices from
// a warp-aggregated counter (work stealing across sets), find the photon's
// set by binary search over the budgets' prefix sums, and read that set's
// optical constants through the read-only cache.  The host lays the sets
// out in decreasing order of estimated cost per photon, so the photons that
// live longest start first.  Uneven budgets therefore
// cost nothing extra: the GPU stays full until the last photon of the last
// set, and there is one tail for the whole sweep instead of one per set.
// Per-set totals are u64 fixed point in shared memory, folded into global
// memory once per block; the escaping flux J(r) of each set goes straight to
// global u64 atomics (one deposit per escaping photon).
#include <cuda_runtime.h>

#include "engine.h"

namespace nmc {
namespace {

template <int PHASE, bool FAST>
__global__ void __launch_bounds__(256) sweep_kernel(const SweepParams P) {
  using M = Math<FAST>;
  constexpr bool TT = PHASE == kPhaseTT;
  extern __shared__ unsigned long long s_sum[];  // nsets x 5: photons, hops, S, A, E
  double* s_e2 = reinterpret_cast<double*>(s_sum + 5 * P.nsets);
  for (int k = threadIdx.x; k < 6 * P.nsets; k += blockDim.x) s_sum[k] = 0ull;
  __syncthreads();
  const int BINS = P.bins;
  const uint32_t k0 = P.k0;

  PhiloxRng<TT> rng;
  float x = 0.f, y = 0.f, z = 0.f, ux = 0.f, uy = 0.f, uz = 1.f, W = 0.f, step_u = 1.f;
  float rsp = 0.f, Atot = 0.f, E = 0.f;
  uint32_t nsc = 0, nsub = 0, k1 = P.k1;
  int set = 0;
  const SweepSetDev* S = P.sets;
  bool alive = false, have = false;

  while (true) {
    if (!alive) {
      if (have) {
        unsigned long long* b = s_sum + 5 * set;
        atomicAdd(b + 0, 1ull);
        atomicAdd(b + 1, (unsigned long long)nsub);
        atomicAdd(b + 2, to_fix(rsp));
        atomicAdd(b + 3, to_fix(Atot));
        atomicAdd(b + 4, to_fix(E));
        if (E > 0.f) atomicAdd(s_e2 + set, (double)E * (double)E);
      }
      const unsigned long long g = next_photon(P.work);
      if (g >= P.total) break;
      have = true;
      // queue slot of global photon g: prefix[k] <= g < prefix[k + 1]
      int lo = 0, hi = P.nsets;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(P.prefix + mid) <= g) lo = mid; else hi = mid;
      }
      S = P.sets + lo;
      set = (int)__ldg(&S->id);
      k1 = P.k1 + (uint32_t)set;
      rng.init(__ldg(&S->first) + (g - __ldg(P.prefix + lo)));
      // ---- LAUNCH (kernels.metal:106-168) with this set's indices
      const float n1 = __ldg(&S->n1), n2 = __ldg(&S->n2);
      x = y = z = 0.f;
      ux = uy = uz = 0.f;
      rsp = 0.f;
      LaunchDraws d{rng.block(0xFFFFFFFFu, k0, k1), 0};
      if (P.mcflag == 0) {
        x = P.radius * sqrtf(d.next());
        z = P.zs;
        uz = 1.f;
        rsp = __ldg(&S->rsp);
      } else if (P.mcflag == 1) {
        x = P.radius * sqrtf(-logf(d.next()));
        z = P.zs;
        const float xf = P.waist * sqrtf(-logf(d.next()));
        const float temp = sqrtf((x - xf) * (x - xf) + P.zfocus * P.zfocus);
        const float costheta = P.zfocus / temp;
        float uzn = costheta;
        rsp = rfresnel(n2, n1, costheta, &uzn);
        uz = uzn;
        ux = sqrtf(fmaxf(1.f - uz * uz, 0.f));
      } else if (P.mcflag == 2) {
        x = P.xs;
        y = P.ys;
        z = P.zs;
        const float costheta = 1.f - 2.f * d.next();
        const float sintheta = sqrtf(fmaxf(1.f - costheta * costheta, 0.f));
        float sp, cp;
        M::sincos2pi(d.next(), &sp, &cp);
        ux = sintheta * cp;
        uy = sintheta * sp;
        uz = costheta;
      }
      step_u = rng.first_step(k0, k1);
      W = 1.f - rsp;
      Atot = E = 0.f;
      nsc = nsub = 0;
      alive = true;
    }

    const float mut = __ldg(&S->mut);
    // ---- HOP (:183-187)
    const float s = M::div(M::neglog(step_u), mut);
    x = fmaf(s, ux, x);
    y = fmaf(s, uy, y);
    z = fmaf(s, uz, z);
    ++nsub;
    if (P.boundaryflag == 1 && z <= P.zs) {  // ESCAPE (:190-214)
      float uz1;
      if (rng.fres_u(k0, k1) > rfresnel(__ldg(&S->n1), __ldg(&S->n2), -uz, &uz1)) {
        x = fmaf(-s, ux, x);
        y = fmaf(-s, uy, y);
        z = fmaf(-s, uz, z);
        const float s2 = fabsf(z / uz);
        x = fmaf(s2, ux, x);
        y = fmaf(s2, uy, y);
        const float r = sqrtf(x * x + y * y);
        int ir = (int)fminf(r * P.idr, (float)BINS) + 1;
        if (ir > BINS) ir = BINS;
        if (P.J) atomicAdd(P.J + (size_t)set * (BINS + 1) + ir, to_fix(W));
        E += W;
        alive = false;
        continue;
      }
      z = -z;
      uz = -uz;
    }
    // ---- DROP (:224-234): absorbed weight only (no F(r,z) in sweeps)
    const float absorb = W * (1.f - __ldg(&S->albedo));
    W -= absorb;
    Atot += absorb;
    // ---- SPIN (:243-279), ROULETTE (:289-294), next HOP's draw
    const bool need_roul = W < kTHRESHOLD;
    const SpinDraws dr = rng.spin_draws(need_roul, k0, k1);
    float costheta;
    if (PHASE == kPhaseTT)
      costheta = tt_sample<FAST>(S->ph, dr.a, dr.b);
    else if (PHASE == kPhaseIsoRef)
      costheta = 2.f * dr.a - 1.f;
    else
      costheta = hg_sample<FAST>(S->ph, dr.a);
    spin<FAST>(costheta, TT ? dr.c : dr.b, ux, uy, uz);
    ++nsc;
    if (need_roul) {
      if (dr.roul <= kCHANCE)
        W /= kCHANCE;
      else
        alive = false;
    }
    step_u = dr.step;
    if (alive && nsub >= P.step_cap) {
      alive = false;
      atomicOr(P.flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
    }
  }

  __syncthreads();
  for (int k = threadIdx.x; k < 5 * P.nsets; k += blockDim.x)
    if (s_sum[k]) atomicAdd(P.sums + k, s_sum[k]);
  for (int k = threadIdx.x; k < P.nsets; k += blockDim.x)
    if (s_e2[k] != 0.0) atomicAdd(P.e2 + k, s_e2[k]);
}

template <bool FAST>
const void* pick(int phase) {
  if (phase == kPhaseTT) return (const void*)sweep_kernel<kPhaseTT, FAST>;
  if (phase == kPhaseIsoRef) return (const void*)sweep_kernel<kPhaseIsoRef, FAST>;
  return (const void*)sweep_kernel<kPhaseHG, FAST>;
}

}  // namespace

size_t sweep_smem_bytes(int nsets) { return (size_t)nsets * 6 * 8; }

cudaError_t sweep_prepare(const SweepParams& p, const void** f, size_t* sh) {
  *f = p.fast ? pick<true>(p.phase_kind) : pick<false>(p.phase_kind);
  *sh = sweep_smem_bytes(p.nsets);
  if (*sh > 48 * 1024) return cudaFuncSetAttribute(*f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*sh);
  return cudaSuccess;
}

cudaError_t launch_sweep(const SweepParams& p, int grid, int block, cudaStream_t stream) {
  const void* f;
  size_t sh;
  cudaError_t e = sweep_prepare(p, &f, &sh);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&p};
  return cudaLaunchKernel(f, dim3(grid), dim3(block), args, sh, stream);
}

cudaError_t sweep_occupancy(const SweepParams& p, int block, int* blocks_per_sm) {
  const void* f;
  size_t sh;
  cudaError_t e = sweep_prepare(p, &f, &sh);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, sh);
}

}  // namespace nmc
