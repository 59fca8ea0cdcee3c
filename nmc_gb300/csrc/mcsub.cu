// mcsub.cu - semi-infinite medium photon transport (MCSubKernel,
// kernels.metal:59-319) as a persistent CUDA kernel for sm_103a.
//
// One loop trip is one HOP-ESCAPE-DROP-SPIN-ROULETTE cycle of one photon.
// The cylindrical tallies F(r,z) and J(r) are privatised per block in shared
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

template <int PHASE, class RNG, bool TRACE, bool SMEM>
__global__ void __launch_bounds__(512) mcsub_kernel(const SubParams P) {
  extern __shared__ uint32_t smem[];
  const int BINS = P.bins;
  const int nJ = BINS + 1, nF = nJ * nJ;
  uint32_t* Flo = smem;
  uint32_t* Fhi = Flo + nF;
  uint32_t* Jlo = Fhi + nF;
  uint32_t* Jhi = Jlo + nJ;
  if (SMEM) {
    for (int k = threadIdx.x; k < 2 * (nF + nJ); k += blockDim.x) smem[k] = 0u;
    __syncthreads();
  }

  unsigned long long t_ph = 0, t_sub = 0, t_sc = 0, t_S = 0, t_A = 0, t_E = 0;
  double t_rd2 = 0.0;

  RNG rng;
  float x = 0.f, y = 0.f, z = 0.f, ux = 0.f, uy = 0.f, uz = 1.f, W = 0.f;
  float rsp = 0.f, Atot = 0.f, E = 0.f;
  uint32_t nsc = 0, nsub = 0, fate = NMC_FATE_ALIVE, ndet = 0, nev = 0;
  unsigned long long pidx = 0;
  bool alive = false, have = false;

  while (true) {
    if (!alive) {
      if (have) {
        t_S += to_fix(rsp);
        t_A += to_fix(Atot);
        t_E += to_fix(E);
        t_rd2 += (double)E * (double)E;
        t_sub += nsub;
        t_sc += nsc;
        ++t_ph;
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
      pidx = next_photon(&P.sums->work);
      if (pidx >= P.n) break;
      have = true;
      const unsigned long long pid = P.first + pidx;
      if constexpr (std::is_same<RNG, TausRng>::value) {
        rng.init_photon(pid, P.rng.batch, false, false);
      } else {
        rng.init(P.rng.k0, P.rng.k1, pid);
      }
      // ---- LAUNCH (kernels.metal:106-168)
      rsp = 0.f;
      x = y = z = 0.f;
      ux = uy = uz = 0.f;
      if (P.mcflag == 0) {
        const float r = rng.launch_u();
        x = P.radius * sqrtf(r);
        y = 0.f;
        z = P.zs;
        uz = 1.f;
        float t = P.n1 / P.n2;
        t = (1.f - t) / (1.f + t);
        rsp = t * t;
      } else if (P.mcflag == 1) {
        float r;
        while ((r = rng.launch_u()) <= 0.f) {
        }
        x = P.radius * sqrtf(-logf(r));
        z = P.zs;
        while ((r = rng.launch_u()) <= 0.f) {
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
      } else if (P.mcflag == 2) {
        x = P.xs;
        y = P.ys;
        z = P.zs;
        const float costheta = 1.f - 2.f * rng.launch_u();
        const float sintheta = sqrtf(fmaxf(1.f - costheta * costheta, 0.f));
        float sp, cp;
        sincospif(2.f * rng.launch_u(), &sp, &cp);
        ux = sintheta * cp;
        uy = sintheta * sp;
        uz = costheta;
      }
      W = 1.f - rsp;
      Atot = 0.f;
      E = 0.f;
      nsc = nsub = ndet = nev = 0;
      fate = NMC_FATE_ALIVE;
      alive = true;
    }

    // ---- HOP (:183-187)
    rng.new_hop();
    float rnd;
    while ((rnd = rng.step_u()) <= 0.f) {
    }
    const float s = -logf(rnd) / P.mut;
    x = fmaf(s, ux, x);
    y = fmaf(s, uy, y);
    z = fmaf(s, uz, z);
    ++nsub;
    if (P.boundaryflag == 1 && z <= P.zs) {  // ESCAPE (:190-214)
      rnd = rng.fres_u();
      float uz1;
      if (rnd > rfresnel(P.n1, P.n2, -uz, &uz1)) {
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
          atomicAdd(P.J + ir, to_fix(W));
        E += W;
        ndet = 1;
        fate = NMC_FATE_ESCAPED;
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
    {
      const float r = sqrtf(x * x + y * y);
      int ir = (int)fminf(r * P.idr, (float)BINS) + 1;
      int iz = (int)fminf(fabsf(z) * P.idz, (float)BINS) + 1;
      if (ir >= BINS) ir = BINS;
      if (iz >= BINS) iz = BINS;
      if (SMEM)
        smem_add(Flo, Fhi, ir * BINS + iz, absorb);
      else
        atomicAdd(P.F + (ir * BINS + iz), to_fix(absorb));
    }
    // ---- SPIN (:243-279)
    float costheta;
    if (PHASE == kPhaseTT) {
      costheta = tt_sample(P.phase, rng);
    } else {
      const float u = rng.cos_u();
      costheta = (PHASE == kPhaseIsoRef) ? 2.f * u - 1.f : hg_sample(P.phase, u);
    }
    spin(costheta, rng.psi_u(), ux, uy, uz);
    ++nsc;
    // ---- ROULETTE (:289-294)
    if (W < kTHRESHOLD) {
      if (rng.roul_u() <= kCHANCE)
        W /= kCHANCE;
      else {
        fate = NMC_FATE_ROULETTE;
        alive = false;
      }
    }
    if (TRACE && nev < P.trace.k_events) {
      P.trace.events[pidx * P.trace.k_events + nev] = make_float4(x, y, z, W);
      ++nev;
    }
    if (alive && nsub >= P.step_cap) {  // device-side cap: not a reference behaviour
      fate = NMC_FATE_STEPCAP;
      alive = false;
      atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
    }
  }

  warp_add_u64(&P.sums->photons, t_ph);
  warp_add_u64(&P.sums->substeps, t_sub);
  warp_add_u64(&P.sums->scatters, t_sc);
  warp_add_u64(&P.sums->S, t_S);
  warp_add_u64(&P.sums->A, t_A);
  warp_add_u64(&P.sums->E, t_E);
  warp_add_u64(&P.sums->rd, t_E);
  warp_add_f64(&P.sums->rd_sumsq, t_rd2);

  if (SMEM) {  // fold the block's tallies into the global ones (scale 2^31 -> 2^32)
    __syncthreads();
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

template <int PHASE, bool TRACE, bool SMEM>
const void* kernel_ptr(uint32_t rng_kind) {
  if (rng_kind == NMC_RNG_TAUS_REF) return (const void*)mcsub_kernel<PHASE, TausRng, TRACE, SMEM>;
  return (const void*)mcsub_kernel<PHASE, PhiloxRng<PHASE == kPhaseTT>, TRACE, SMEM>;
}

template <int PHASE>
const void* pick3(uint32_t rng_kind, bool trace, bool smem) {
  if (trace) return smem ? kernel_ptr<PHASE, true, true>(rng_kind) : kernel_ptr<PHASE, true, false>(rng_kind);
  return smem ? kernel_ptr<PHASE, false, true>(rng_kind) : kernel_ptr<PHASE, false, false>(rng_kind);
}

const void* pick(const SubParams& p, bool trace, bool smem, int phase) {
  if (phase == kPhaseTT) return pick3<kPhaseTT>(p.rng.kind, trace, smem);
  if (phase == kPhaseIsoRef) return pick3<kPhaseIsoRef>(p.rng.kind, trace, smem);
  return pick3<kPhaseHG>(p.rng.kind, trace, smem);
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
  const bool smem = smem_fits(p.bins);
  *f = pick(p, trace, smem, p.phase_kind);
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
