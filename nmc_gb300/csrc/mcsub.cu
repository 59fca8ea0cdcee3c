// mcsub.cu - semi-infinite medium photon transport (MCSubKernel,
// kernels.metal:59-319) as a persistent CUDA kernel for sm_103a.
//
// One loop trip is one HOP-ESCAPE-DROP-SPIN-ROULETTE cycle of one photon;
// the SPIN draws and the next hop's step come from one Philox block.  The
// cylindrical tallies F(r,z) and J(r) are privatised per block in shared
// memory as 64-bit fixed point held in two 32-bit words (low word atomicAdd,
// carry into the high word when the add wraps), so every deposit is a
// shared-memory atomic and the block's copy is folded into the global u64
// tally once at the end.  Integer sums make the result independent of
// deposit order.
#include <cuda_runtime.h>

#include <type_traits>

#include "engine.h"

namespace nmc {
namespace {

constexpr float kFix31 = 2147483648.0f;  // shared-memory scale 2^31

__device__ __forceinline__ void smem_add(uint32_t* lo, uint32_t* hi, int k, float v) {
  const uint32_t a = __float2uint_rn(v * kFix31);
  const uint32_t old = atomicAdd(lo + k, a);
  if (old + a < old) atomicAdd(hi + k, 1u);
}

template <bool FAST, class D>
__device__ __forceinline__ void launch_photon(const SubParams& P, D& d, float& x, float& y, float& z,
                                              float& ux, float& uy, float& uz, float& rsp) {
  using M = Math<FAST>;
  rsp = 0.f;
  x = y = z = 0.f;
  ux = uy = uz = 0.f;
  if (P.mcflag == 0) {  // kernels.metal:106-121
    const float r = d.next();
    x = P.radius * sqrtf(r);
    z = P.zs;
    uz = 1.f;
    float t = P.n1 / P.n2;
    t = (1.f - t) / (1.f + t);
    rsp = t * t;
  } else if (P.mcflag == 1) {  // :122-147
    float r;
    while ((r = d.next()) <= 0.f) {
    }
    x = P.radius * sqrtf(-logf(r));
    z = P.zs;
    while ((r = d.next()) <= 0.f) {
    }
    const float xf = P.waist * sqrtf(-logf(r));
    const float temp = sqrtf((x - xf) * (x - xf) + P.zfocus * P.zfocus);
    const float costheta = P.zfocus / temp;
    ux = -(x - xf) / temp;
    uz = costheta;
    float uzn = uz;
    rsp = rfresnel(P.n2, P.n1, costheta, &uzn);
    uz = uzn;
    ux = sqrtf(fmaxf(1.f - uz * uz, 0.f));
  } else if (P.mcflag == 2) {  // :148-164
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
}

template <int PHASE, class RNG, bool TRACE, bool SMEM, bool FAST>
__global__ void __launch_bounds__(512) mcsub_kernel(const SubParams P) {
  using M = Math<FAST>;
  constexpr bool TT = PHASE == kPhaseTT;
  extern __shared__ uint32_t smem[];
  __shared__ unsigned long long s_tot[6];  // photons, hops, scatters, S, A, E
  __shared__ double s_rd2;
  const int BINS = P.bins;
  const int nJ = BINS + 1, nF = nJ * nJ;
  uint32_t* Flo = smem;
  uint32_t* Fhi = Flo + nF;
  uint32_t* Jlo = Fhi + nF;
  uint32_t* Jhi = Jlo + nJ;
  if (SMEM)
    for (int k = threadIdx.x; k < 2 * (nF + nJ); k += blockDim.x) smem[k] = 0u;
  if (threadIdx.x < 6) s_tot[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) s_rd2 = 0.0;
  __syncthreads();
  const RoundKeys keys{P.rng.rk};  // Philox round keys of the seed

  RNG rng;
  float x = 0.f, y = 0.f, z = 0.f, ux = 0.f, uy = 0.f, uz = 1.f, W = 0.f, step_u = 1.f;
  float rsp = 0.f, Atot = 0.f, E = 0.f;
  uint32_t nsc = 0, nsub = 0, fate = NMC_FATE_ALIVE, ndet = 0, nev = 0;
  unsigned long long pidx = ~0ull;  // the photon; ~0 before the first (its run of queue indices)
  bool alive = false, have = false;

  while (true) {
    if (!alive) {
      if (have) {
        atomicAdd(&s_tot[0], 1ull);
        atomicAdd(&s_tot[1], (unsigned long long)nsub);
        atomicAdd(&s_tot[2], (unsigned long long)nsc);
        atomicAdd(&s_tot[3], to_fix(rsp));
        atomicAdd(&s_tot[4], to_fix(Atot));
        atomicAdd(&s_tot[5], to_fix(E));
        if (E > 0.f) atomicAdd(&s_rd2, (double)E * (double)E);
        if (TRACE) {
          nmc_photon_record r;
          r.n_scatt = nsc;
          r.n_sub = nsub;
          r.fate = fate;
          r.n_detect = ndet;
          r.w_final = W;
          r.absorbed = Atot;
          r.detected = E;
          r.x = x;
          r.y = y;
          r.z = z;
          P.trace.recs[pidx] = r;
        }
      }
      pidx = next_photon_run(&P.sums->work, P.per_fetch, pidx);
      if (pidx >= P.n) break;
      have = true;
      const unsigned long long pid = P.first + pidx;
      if constexpr (std::is_same<RNG, TausRng>::value) {
        rng.init_photon(pid, P.rng.batch, false, false);
        typename TausRng::Seq d{&rng};
        launch_photon<FAST>(P, d, x, y, z, ux, uy, uz, rsp);
      } else {
        rng.init(pid);
        LaunchDraws d{rng.block(0xFFFFFFFFu, keys), 0};
        launch_photon<FAST>(P, d, x, y, z, ux, uy, uz, rsp);
      }
      step_u = rng.first_step(keys);
      W = 1.f - rsp;  // :166-168
      Atot = 0.f;
      E = 0.f;
      nsc = nsub = 0;
      if (TRACE) {
        fate = NMC_FATE_ALIVE;
        ndet = nev = 0;
      }
      alive = true;
    }

    // ---- HOP (:183-187)
    const float s = M::div(M::neglog(step_u), P.mut);
    x = fmaf(s, ux, x);
    y = fmaf(s, uy, y);
    z = fmaf(s, uz, z);
    ++nsub;
    if (P.boundaryflag == 1 && z <= P.zs) {  // ESCAPE (:190-214)
      float uz1;
      if (rng.fres_u(keys) > rfresnel(P.n1, P.n2, -uz, &uz1)) {
        x = fmaf(-s, ux, x);
        y = fmaf(-s, uy, y);
        z = fmaf(-s, uz, z);
        const float s2 = fabsf(z / uz);
        x = fmaf(s2, ux, x);
        y = fmaf(s2, uy, y);
        const float r = sqrtf(x * x + y * y);
        int ir = (int)fminf(r * P.idr, (float)BINS) + 1;
        if (ir > BINS) ir = BINS;
        if (SMEM)
          smem_add(Jlo, Jhi, ir, W);
        else
          if (idx_ok(ir, (unsigned)BINS + 1u, &P.sums->flags)) atomicAdd(P.J + ir, to_fix(W));
        E += W;
        if (TRACE) {
          ndet = 1;
          fate = NMC_FATE_ESCAPED;
        }
        alive = false;
        continue;
      }
      z = -z;
      uz = -uz;
    }
    // ---- DROP (:224-234)
    const float absorb = W * (1.f - P.albedo);
    W -= absorb;
    Atot += absorb;
    if (!P.skip_F) {
      const float r = sqrtf(x * x + y * y);
      int ir = (int)fminf(r * P.idr, (float)BINS) + 1;
      int iz = (int)fminf(fabsf(z) * P.idz, (float)BINS) + 1;
      if (ir >= BINS) ir = BINS;
      if (iz >= BINS) iz = BINS;
      if (SMEM)
        smem_add(Flo, Fhi, ir * BINS + iz, absorb);
      else
        if (idx_ok(ir * BINS + iz, (unsigned long long)(BINS + 1) * (BINS + 1), &P.sums->flags))
          atomicAdd(P.F + (ir * BINS + iz), to_fix(absorb));
    }
    // ---- SPIN (:243-279), ROULETTE (:289-294), next HOP's draw
    const bool need_roul = W < kTHRESHOLD;
    const SpinDraws d = spin_draws<TT>(rng, need_roul, keys);
    float costheta;
    if (PHASE == kPhaseTT)
      costheta = tt_sample<FAST>(P.phase, d.a, d.b);
    else if (PHASE == kPhaseIsoRef)
      costheta = 2.f * d.a - 1.f;  // kernels.metal:252 overrides the HG sample
    else
      costheta = hg_sample<FAST>(P.phase, d.a);
    spin<FAST>(costheta, TT ? d.c : d.b, ux, uy, uz);
    ++nsc;
    if (need_roul) {
      if (d.roul <= kCHANCE) {
        W /= kCHANCE;
      } else {
        if (TRACE) fate = NMC_FATE_ROULETTE;
        alive = false;
      }
    }
    if (TRACE && nev < P.trace.k_events) {
      P.trace.events[pidx * P.trace.k_events + nev] = make_float4(x, y, z, W);
      ++nev;
    }
    step_u = d.step;
    if (alive && nsub >= P.step_cap) {  // device-side cap: not a reference behaviour
      if (TRACE) fate = NMC_FATE_STEPCAP;
      alive = false;
      atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
    }
  }

  __syncthreads();
  if (threadIdx.x < 6 && s_tot[threadIdx.x]) {
    unsigned long long* dst[6] = {&P.sums->photons, &P.sums->substeps, &P.sums->scatters,
                                  &P.sums->S,       &P.sums->A,        &P.sums->E};
    atomicAdd(dst[threadIdx.x], s_tot[threadIdx.x]);
    if (threadIdx.x == 5) atomicAdd(&P.sums->rd, s_tot[5]);
  }
  if (threadIdx.x == 0 && s_rd2 != 0.0) atomicAdd(&P.sums->rd_sumsq, s_rd2);
  if (SMEM) {  // fold the block's tallies into the global ones (scale 2^31 -> 2^32)
    for (int k = threadIdx.x; k < nF; k += blockDim.x) {
      const unsigned long long v = ((unsigned long long)Fhi[k] << 32) | Flo[k];
      if (v) atomicAdd(P.F + k, v << 1);
    }
    for (int k = threadIdx.x; k < nJ; k += blockDim.x) {
      const unsigned long long v = ((unsigned long long)Jhi[k] << 32) | Jlo[k];
      if (v) atomicAdd(P.J + k, v << 1);
    }
  }
}

template <int PHASE, bool TRACE, bool SMEM, bool FAST>
const void* kernel_ptr(uint32_t rng_kind) {
  if (rng_kind == NMC_RNG_TAUS_REF) return (const void*)mcsub_kernel<PHASE, TausRng, TRACE, SMEM, FAST>;
  return (const void*)mcsub_kernel<PHASE, PhiloxRng<PHASE == kPhaseTT>, TRACE, SMEM, FAST>;
}

template <int PHASE, bool FAST>
const void* pick3(uint32_t rng_kind, bool trace, bool smem) {
  if (trace) return smem ? kernel_ptr<PHASE, true, true, FAST>(rng_kind) : kernel_ptr<PHASE, true, false, FAST>(rng_kind);
  return smem ? kernel_ptr<PHASE, false, true, FAST>(rng_kind) : kernel_ptr<PHASE, false, false, FAST>(rng_kind);
}

template <bool FAST>
const void* pick2(const SubParams& p, bool trace, bool smem) {
  if (p.phase_kind == kPhaseTT) return pick3<kPhaseTT, FAST>(p.rng.kind, trace, smem);
  if (p.phase_kind == kPhaseIsoRef) return pick3<kPhaseIsoRef, FAST>(p.rng.kind, trace, smem);
  return pick3<kPhaseHG, FAST>(p.rng.kind, trace, smem);
}

}  // namespace

size_t mcsub_smem_bytes(int bins) {
  const size_t nJ = (size_t)bins + 1, nF = nJ * nJ;
  return 2 * (nF + nJ) * sizeof(uint32_t);
}

// Shared-memory privatisation while the tally fits next to a second block
// (BINS <= 160); larger grids deposit straight into the global u64 tally.
static bool smem_fits(int bins) { return mcsub_smem_bytes(bins) <= 200 * 1024; }

static cudaError_t prepare(const SubParams& p, bool trace, const void** f, size_t* sh) {
  const bool smem = !p.skip_F && !p.global_tallies && smem_fits(p.bins);
  *f = p.fast_math ? pick2<true>(p, trace, smem) : pick2<false>(p, trace, smem);
  *sh = smem ? mcsub_smem_bytes(p.bins) : 0;
  if (*sh > 48 * 1024)
    return cudaFuncSetAttribute(*f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*sh);
  return cudaSuccess;
}

cudaError_t launch_mcsub(const SubParams& p, bool trace, int grid, int block, cudaStream_t stream) {
  const void* f;
  size_t sh;
  cudaError_t e = prepare(p, trace, &f, &sh);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&p};
  return cudaLaunchKernel(f, dim3(grid), dim3(block), args, sh, stream);
}

cudaError_t mcsub_occupancy(const SubParams& p, bool trace, int block, int* blocks_per_sm) {
  const void* f;
  size_t sh;
  cudaError_t e = prepare(p, trace, &f, &sh);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, sh);
}

}  // namespace nmc
