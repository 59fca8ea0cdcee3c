// mcxyz_kernel.cuh - voxel photon transport (MCXYZKernel,
// kernels.metal:321-754, and the two-term variant MCXYZKernelTT,
// kernels.metal:757-1118) as one persistent CUDA kernel for sm_103a,
// instantiated by mcxyz.cu (tissue-map media) and mcxyz_voxel.cu (media with
// per-voxel optical properties, forward and adjoint).
//
// Modes: kTissue reads a uint8 tissue map and a 19-entry table (the
// reference's model); kVoxel reads (mua, mus, 1/mus, g) per voxel; kRecord,
// kScore and kAdjoint are kVoxel plus the passes of the perturbation Monte
// Carlo adjoint: the record pass (kRecord) is the forward run that also
// appends every detection event (photon, radial bin, weight) to a list; the
// score replay (kScore) gives every photon its total score when deposits
// score too; the accumulating replay (kAdjoint) replays each scoring photon
// (the same transport code and random streams, hence the same trajectory;
// sub-steps are bit-identical across the modes) carrying D = the
// photon's remaining detected score sum_k G[bin_k] w_k over events not yet
// passed, and accumulates per voxel v (the voxel whose properties the step
// used)
//   L_v += D * s        for every charged path length s (absorption),
//   M_v += D / mus_v - D * s'   for the scatterings and the hop lengths s'
//                       whose probability depends on mus_v,
//   Q_v += D * dln p_HG(cos; g_v)/dg  for every scattering in voxel v,
// from which dScore/dmua_v = -L_v (pathwise: the weight is exp(-sum mua s)),
// dScore/dmus_v = M_v and dScore/dg_v = Q_v (likelihood ratio).  s' = s
// everywhere.  Only a step to a voxel face reaches the detection plane
// (kernels.metal:534-637).  There the reference relocates the photon to the
// plane after charging the whole step, and the rest of the hop becomes a
// fixed length (:571-573), so neither that rest nor the scattering that
// ends it depends on the exponential draw.
//
// Design:
//  * persistent threads: the grid fills the GPU once; a thread that retires a
//    photon takes the next photon index from a warp-aggregated counter;
//  * one voxel sub-step per loop trip (the reference's inner do-while over
//    RAY_DEPTH crossings, :505-685, flattened); the SPIN, roulette and the
//    next hop's step run together at a hop's end from one Philox block, so
//    no random state is carried across sub-steps;
//  * positions are an integer voxel-lattice cell plus an FP32 offset in the
//    cell: the "littlest step" ls = 1e-7 (definitions.h:59) stays ~200 ulps
//    above the offset's rounding, so FP32 stepping walks voxels the way FP64
//    arithmetic does (the reference's global FP32 coordinates round ls away
//    at mm-scale positions and stall photons at faces);
//  * optical properties live in shared memory, re-read each sub-step rather
//    than held in registers; the uint8 tissue map is read through the
//    read-only path (L2-resident: 8 MB for 200^3);
//  * deposits are merged in a register while the photon stays in one voxel
//    and flushed as u64 fixed-point atomics (exact, bit-reproducible);
//    per-photon totals go to shared-memory block sums.
#include <cuda_runtime.h>

#include <type_traits>

#include "engine.h"

namespace nmc {
namespace {

constexpr uint32_t kAlive = 1u, kBflag = 2u, kSurf = 4u, kHave = 8u, kFixed = 16u;

__device__ __forceinline__ void to_lattice(float x, float d, float dmax, int& k, float& f) {
  const float q = floorf(__fdiv_rn(x, d));
  k = (int)q;
  f = fmaf(-q, d, x);
  if (f < 0.f) {
    --k;
    f = fminf(f + d, dmax);
  } else if (f >= d) {
    ++k;
    f -= d;
  }
}

// Brings an offset that left [0, d) by less than one cell back into it.
__device__ __forceinline__ void norm_axis(int& k, float& f, float d, float dmax) {
  const bool up = f >= d, dn = f < 0.f;
  k += (int)up - (int)dn;
  f = up ? f - d : (dn ? fminf(f + d, dmax) : f);
}

// The reference's voxel index `(int)(N/2.0 + x/d)` (kernels.metal:641-643,
// C truncation toward zero) from cell k and offset f: half = N/2 rounded
// down, odd = N is odd (then the index steps at f = d/2, hd = d/2).  The
// launch formula `(int)(N/2 + x/d)` (:472-474) is the even case with half = N/2.
__device__ __forceinline__ int lookup_index(int k, float f, int half, int odd, float hd) {
  int A = half + k;
  bool frac_pos;
  if (odd) {
    const bool up = f >= hd;
    A += (int)up;
    frac_pos = !up || f > hd;
  } else {
    frac_pos = f > 0.f;
  }
  return A + (int)((A < 0) & frac_pos);
}

struct Deposit {
  unsigned int idx;
  float acc;
  __device__ __forceinline__ void flush(unsigned long long* F3D, unsigned int nvox, unsigned int* flags) {
    if (acc > 0.f && idx_ok(idx, nvox, flags)) atomicAdd(F3D + idx, to_fix(acc));
    acc = 0.f;
  }
  __device__ __forceinline__ void add(unsigned long long* F3D, unsigned int i, float v, unsigned int nvox,
                                      unsigned int* flags) {
    if (i != idx) {
      flush(F3D, nvox, flags);
      idx = i;
    }
    acc += v;
  }
};

// LAUNCH (kernels.metal:349-463; the two-term kernel :778-870 has no
// Gaussian branch).  `d.next()` yields launch uniforms in draw order.
template <bool TT, bool FAST, class D>
__device__ __forceinline__ void launch_photon(const XyzParams& P, D& d, float& x, float& y, float& z,
                                              float& ux, float& uy, float& uz, float& W) {
  using M = Math<FAST>;
  W = 1.f;
  x = y = z = 0.f;
  ux = uy = uz = 0.f;  // tagPhoton() zero initialisation
  if (P.launchflag == 1) {
    x = P.xs;
    y = P.ys;
    z = P.zs;
    ux = P.ux0;
    uy = P.uy0;
    uz = P.uz0;
  } else if (P.mcflag == 0 || (P.mcflag == 1 && !TT)) {
    const bool gauss = P.mcflag == 1;
    float r, sp, cp;
    while ((r = d.next()) <= 0.f) {
    }
    float rad = gauss ? P.radius * sqrtf(-logf(r)) : P.radius * sqrtf(r);
    while ((r = d.next()) <= 0.f) {
    }
    M::sincos2pi(r, &sp, &cp);
    x = P.xs + rad * cp;
    y = P.ys + rad * sp;
    z = P.zs;
    while ((r = d.next()) <= 0.f) {
    }
    rad = P.waist * sqrtf(r);
    while ((r = d.next()) <= 0.f) {
    }
    M::sincos2pi(r, &sp, &cp);
    const float xf = rad * cp, yf = rad * sp;
    const float temp = sqrtf((x - xf) * (x - xf) + (y - yf) * (y - yf) + P.zfocus * P.zfocus);
    ux = -(x - xf) / temp;
    uy = -(y - yf) / temp;
    uz = sqrtf(1.f - ux * ux - uy * uy);
    if (gauss) {  // :423-427
      float uz_new = uz;
      const float int_rsp = rfresnel(P.n2, P.n1, fabsf(uz), &uz_new);
      W = W * (1.f - int_rsp);
      snell(P.n2, P.n1, ux, uy, uz);
    }
  } else if (P.mcflag == 2) {
    const float costheta = 1.f - 2.f * d.next();
    const float sintheta = sqrtf(fmaxf(1.f - costheta * costheta, 0.f));
    float sp, cp;
    M::sincos2pi(d.next(), &sp, &cp);
    x = P.xs;
    y = P.ys;
    z = P.zs;
    ux = sintheta * cp;
    uy = sintheta * sp;
    uz = costheta;
  } else if (P.mcflag == 3) {
    float r;
    while ((r = d.next()) <= 0.f) {
    }
    x = P.radius * (r * 2.f - 1.f);
    while ((r = d.next()) <= 0.f) {
    }
    y = P.radius * (r * 2.f - 1.f);
    z = P.zs;
    uz = 1.f;
  } else if (P.mcflag == 4) {
    z = P.zs;
    uz = 1.f;
  }
}

// Adjoint sums of the voxel the photon is in, merged while it stays there.
struct AdjAcc {
  unsigned int idx;
  float L, M, Q;
  __device__ __forceinline__ void flush(const XyzParams& P) {
    if (idx != 0xFFFFFFFFu && idx_ok(idx, (unsigned long long)P.Nx * P.Ny * P.Nz, &P.sums->flags)) {
      if (L != 0.f) atomicAdd(P.gL + idx, (double)L);
      if (M != 0.f) atomicAdd(P.gM + idx, (double)M);
      if (Q != 0.f) atomicAdd(P.gQ + idx, (double)Q);
    }
    L = M = Q = 0.f;
  }
  __device__ __forceinline__ void at(const XyzParams& P, unsigned int i) {
    if (i != idx) {
      flush(P);
      idx = i;
    }
  }
};

// Henyey-Greenstein cos(theta) for a per-voxel g (kernels.metal:696-703),
// rounded like the tissue table's constants (phase_const): 1-g^2, 1+g^2 in
// one rounding, 1/(2g) correctly rounded, so a per-voxel medium and the same
// medium as a tissue map sample the same angles.
template <bool FAST>
__device__ __forceinline__ float hg_from_g(float g, float u) {
  if (g == 0.f) return 2.f * u - 1.f;
  if (flt_eq(g, 1.f)) return 1.f;
  const float t = Math<FAST>::div(fmaf(-g, g, 1.f), fmaf(2.f * g, u, 1.f - g));
  return fmaf(-t, t, fmaf(g, g, 1.f)) * __frcp_rn(2.f * g);
}

// d ln p_HG(mu; g) / dg for p = (1-g^2) / (1+g^2-2 g mu)^(3/2) / 2.
__device__ __forceinline__ float dlnhg_dg(float g, float mu) {
  return -2.f * g / (1.f - g * g) - 3.f * (g - mu) / (1.f + g * g - 2.f * g * mu);
}

template <bool TT, class RNG, bool TRACE, bool FAST, int MODE>
// 4 blocks of 256 per SM in every mode: the accumulating replay fits 64
// registers without spills too (left to itself the compiler takes 78 and 3
// blocks, 7% slower)
__global__ void __launch_bounds__(256, 4) mcxyz_kernel(const XyzParams P) {
  using M = Math<FAST>;
  constexpr bool SW = MODE == kSweep;  // many tissue tables, one per set
  constexpr bool VOX = MODE == kVoxel || MODE == kAdjoint || MODE == kRecord || MODE == kScore;
  constexpr bool ADJ = MODE == kAdjoint || MODE == kScore;  // replays
  constexpr bool REC = MODE == kRecord;
  // Tissue-map kernels of the one-term model flush the merged deposit where
  // a crossing changes the voxel index, instead of testing the index at every
  // deposit: their boundary flag, once cleared, stays cleared, so the next
  // deposit after such a crossing always goes to the new index and the
  // deposits merge into the same groups (same u64 sums).  The two-term
  // kernel sets the flag again at every crossing and keeps the test.
  constexpr bool DEPX = MODE == kTissue && !TT;
  __shared__ float4 s_core[NMC_NTISS];
  __shared__ PhaseConst s_ph[NMC_NTISS];
  __shared__ unsigned long long s_tot[5];  // photons, substeps, scatters, A, rd
  __shared__ double s_rd2;
  if (!VOX && !SW) {
    for (int t = threadIdx.x; t < NMC_NTISS; t += blockDim.x) {
      s_core[t] = P.core[t];
      s_ph[t] = P.phase[t];
    }
  }
  if (threadIdx.x < 5) s_tot[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) s_rd2 = 0.0;
  __syncthreads();

  const uint32_t k0 = P.rng.k0;
  uint32_t k1 = P.rng.k1;  // a sweep set s draws from key (k0, k1 + s)
  // Philox keys: the host's round-key table of (k0, k1), or in a sweep the
  // photon's set key (k0, k1 + set)
  auto keys = [&]() {
    if constexpr (SW)
      return SeedKeys{k0, k1};
    else
      return RoundKeys{P.rng.rk};
  };
  const bool hard_kill = !(P.flags & NMC_FLAG_NO_HARD_KILL);
  constexpr bool back = MODE == kAdjoint;  // accumulating replay
  constexpr bool score = MODE == kScore;   // score replay: D[photon] = its total score
  constexpr bool replay = back || score;   // replays write no tallies
  const float* __restrict__ GF = ADJ ? P.adj_GF : nullptr;
  const int NyNx = P.Ny * P.Nx;
  const unsigned int nvox = (unsigned int)(NyNx * P.Nz);
  // odd grids step the voxel index at the cell's midpoint; +inf turns the
  // test off for even grids without a branch
  const float hdx_e = P.ox ? P.hdx : __int_as_float(0x7f800000), hdy_e = P.oy ? P.hdy : __int_as_float(0x7f800000);

  RNG rng;
  int kx = 0, ky = 0, kz = 0, tiss = 0;
  unsigned int hop_end = 0;  // the sub-step count at which the hop's RAY_DEPTH crossings run out
  float fx = 0.f, fy = 0.f, fz = 0.f, ux = 0.f, uy = 0.f, uz = 1.f;
  float W = 0.f, sleft = 0.f, Rd_loc = 0.f, Atot = 0.f;
  float D = 0.f, Dabs = 0.f;  // adjoint: remaining detected score, sum of |event scores| replayed
  float gf_i = 0.f;           // adjoint: upstream fluence gradient of voxel i (0 without a fluence loss)
  unsigned int i = 0, slot = 0, nsc = 0, nsub = 0, st = 0;
  unsigned int set = 0, sbase = 0;  // sweep: the photon's set and its table offset
  unsigned long long pidx = ~0ull;  // the photon; ~0 before the first (its run of queue indices)
  uint32_t fate = NMC_FATE_ALIVE, ndet = 0, nev = 0;  // trace only
  Deposit dep{0xFFFFFFFFu, 0.f};
  // record pass: the thread's chunk of the deposit list and its fill
  constexpr unsigned int kNoChunk = 0xFFFFFFFFu, kDeadChunk = 0xFFFFFFFEu;
  unsigned int dl_chunk = (REC && P.dl_pool) ? kNoChunk : kDeadChunk, dl_pos = kDepChunk;
  // the next record goes to a fresh chunk (its header names the photon)
  // when the current one is full; past the pool's end the list stops
  auto dl_put = [&](unsigned int a, unsigned int b) {
    if (dl_chunk == kDeadChunk) return;
    if (dl_pos >= kDepChunk) {
      if (dl_chunk != kNoChunk) P.dl_fill[dl_chunk] = dl_pos;
      const unsigned long long c = atomicAdd(P.dl_next, 1ull);
      if (c >= P.dl_chunks) {
        dl_chunk = kDeadChunk;
        return;
      }
      dl_chunk = (unsigned int)c;
      P.dl_pool[(size_t)dl_chunk * kDepChunk] = make_uint2(0xFFFFFFFFu, (unsigned int)pidx);
      dl_pos = 1;
      if (a == 0xFFFFFFFFu) return;  // the chunk's header is the photon's
    }
    P.dl_pool[(size_t)dl_chunk * kDepChunk + dl_pos++] = make_uint2(a, b);
  };
  auto dl_deposit = [&]() {  // the merged deposit about to be flushed to F3D
    if (REC && dep.acc > 0.f) dl_put(dep.idx, __float_as_uint(dep.acc));
  };
  AdjAcc adj{0xFFFFFFFFu, 0.f, 0.f, 0.f};

  auto kill = [&](uint32_t why) {
    if (TRACE && (st & kAlive)) fate = why;
    st &= ~kAlive;
  };

  while (true) {
    if (!(st & kAlive)) {
      if (back && (st & kHave)) {
        adj.flush(P);
        // every recorded event has been met again: D is back to zero up to
        // the rounding of the two summation orders
        if (!(fabsf(D) <= 1e-4f * Dabs)) atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_REPLAY);
      }
      if (score && (st & kHave) && idx_ok(pidx, P.n, &P.sums->flags)) P.adj_Dw[pidx] = D;
      if (SW && (st & kHave)) {  // per-set sums
        XyzSweepSums* q = P.sw_sums + set;
        atomicAdd(&q->photons, 1ull);
        atomicAdd(&q->substeps, (unsigned long long)nsub);
        atomicAdd(&q->scatters, (unsigned long long)nsc);
        atomicAdd(&q->A, to_fix(Atot));
        if (Rd_loc > 0.f) {
          atomicAdd(&q->rd, to_fix(Rd_loc));
          atomicAdd(&q->rd2, (double)Rd_loc * (double)Rd_loc);
        }
      }
      if ((st & kHave) && !replay && !SW) {  // retire the finished photon
        dl_deposit();
        dep.flush(P.F3D, nvox, &P.sums->flags);
        if (Rd_loc > 0.f && idx_ok(slot, P.nslots, &P.sums->flags))
          atomicAdd(P.rd_slots + slot, to_fix(Rd_loc));  // :753
        atomicAdd(&s_tot[0], 1ull);
        atomicAdd(&s_tot[1], (unsigned long long)nsub);
        atomicAdd(&s_tot[2], (unsigned long long)nsc);
        atomicAdd(&s_tot[3], to_fix(Atot));
        atomicAdd(&s_tot[4], to_fix(Rd_loc));
        if (Rd_loc > 0.f) atomicAdd(&s_rd2, (double)Rd_loc * (double)Rd_loc);
        if (TRACE) {
          nmc_photon_record r;
          r.n_scatt = nsc;
          r.n_sub = nsub;
          r.fate = fate;
          r.n_detect = ndet;
          r.w_final = W;
          r.absorbed = Atot;
          r.detected = Rd_loc;
          r.x = (float)kx * P.dx + fx;
          r.y = (float)ky * P.dy + fy;
          r.z = (float)kz * P.dz + fz;
          if (idx_ok(pidx, P.n, &P.sums->flags)) P.trace.recs[pidx] = r;
        }
      }
      pidx = next_photon_run(&P.sums->work, P.per_fetch, pidx);
      if (pidx >= P.n) break;
      if (back) {  // only photons with a score contribute
        D = P.adj_D[pidx];
        Dabs = 0.f;
        if (D == 0.f) {
          st = 0;
          continue;
        }
      }
      if (score) D = 0.f;
      unsigned long long pid = P.first + pidx;
      if (REC) dl_put(0xFFFFFFFFu, (unsigned int)pidx);  // the photon's deposits follow
      if (SW) {  // the queue slot whose budget holds this photon: last k with prefix[k] <= pidx
        unsigned int lo = 0, hi = (unsigned int)P.sw_nsets;
        while (hi - lo > 1) {
          const unsigned int mid = (lo + hi) >> 1;
          if (__ldg(P.sw_prefix + mid) <= pidx) lo = mid; else hi = mid;
        }
        set = __ldg(P.sw_order + lo);
        sbase = set * NMC_NTISS;
        pid = __ldg(P.sw_first + lo) + (pidx - __ldg(P.sw_prefix + lo));
        k1 = P.rng.k1 + set;
      }
      slot = (unsigned int)(pid % P.nslots);
      float x, y, z;
      if constexpr (std::is_same<RNG, TausRng>::value) {
        rng.init_photon(pid, P.rng.batch, TT, P.rng.tt_replay != 0);
        typename TausRng::Seq d{&rng};
        launch_photon<TT, FAST>(P, d, x, y, z, ux, uy, uz, W);
      } else {
        rng.init(pid);
        LaunchDraws d{rng.block(0xFFFFFFFFu, keys()), 0};
        launch_photon<TT, FAST>(P, d, x, y, z, ux, uy, uz, W);
      }
      to_lattice(x, P.dx, P.dxmax, kx, fx);
      to_lattice(y, P.dy, P.dymax, ky, fy);
      to_lattice(z, P.dz, P.dzmax, kz, fz);
      const int ix = min(max(lookup_index(kx, fx, P.Nx / 2, 0, 0.f), 0), P.Nx - 1);  // :472-480
      const int iy = min(max(lookup_index(ky, fy, P.Ny / 2, 0, 0.f), 0), P.Ny - 1);
      const int iz = min(max(lookup_index(kz, fz, 0, 0, 0.f), 0), P.Nz - 1);
      i = (unsigned int)(iz * NyNx + ix * P.Ny + iy);
      if (!VOX) tiss = idx_ok(i, nvox, &P.sums->flags) ? __ldg(P.V + i) : 0;
      if (ADJ && GF) gf_i = idx_ok(i, nvox, &P.sums->flags) ? __ldg(GF + i) : 0.f;
      sleft = M::neglog(rng.first_step(keys()));  // HOP (:501-502)
      hop_end = kRAY_DEPTH + 1;
      Rd_loc = Atot = 0.f;
      nsc = nsub = 0;
      if (TRACE) {
        fate = NMC_FATE_ALIVE;
        ndet = nev = 0;
      }
      st = kAlive | kBflag | kSurf | kHave;
      dep.idx = DEPX ? i : 0xFFFFFFFFu;
      dep.acc = 0.f;
      adj.idx = 0xFFFFFFFFu;
    }

    // ---- one voxel sub-step (:505-682).  The same-voxel move (:515-533) and
    // the step to the nearest face (:534-682) share one straight path; only
    // the face landing, the voxel lookup and the tissue load are predicated
    // on the crossing, so the lanes of a warp stay together.
    const float4 c = VOX ? __ldg(P.vox + (idx_ok(i, nvox, &P.sums->flags) ? i : 0u))
                         : (SW ? __ldg(P.sw_core + sbase + tiss) : s_core[tiss]);  // mua, mus, 1/mus, g
    float s = sleft * c.z;
    ++nsub;
    // FindVoxelFace2 (helpers.metal:85-114) in cell-local form: path length
    // to the face ahead on each axis
    const float rx = M::rcp(fabsf(ux)), ry = M::rcp(fabsf(uy)), rz = M::rcp(fabsf(uz));
    // offset to the face ahead; it is 0 only for a photon on a lower face
    // moving down (an upper face is never reached: offsets stay below d)
    const float dxf = ux >= 0.f ? P.dx - fx : fx, dyf = uy >= 0.f ? P.dy - fy : fy;
    const float tx = dxf * rx;
    const float ty = dyf * ry;
    const float tz = (uz >= 0.f ? P.dz - fz : fz) * rz;
    const int ax = (tx <= ty) ? ((tx <= tz) ? 0 : 2) : ((ty <= tz) ? 1 : 2);
    // SameVoxel (helpers.metal:27-39): the end point stays in the cell, upper
    // faces included; a photon on a lower x or y face moving down stays for
    // up to one cell (the reference compares with the cell below's upper face)
    // with the properties of the cell above.  Per-voxel media take the
    // physical rule instead (the photon steps into the cell below at once):
    // the reference's makes the hop's distribution in the cell below depend
    // on two cells' mus through a moving support, which the likelihood-ratio
    // adjoint cannot differentiate.  The two differ only for photons exactly
    // on a lower face (a beam launched on a voxel face).
    const float sx = (!VOX && dxf == 0.f) ? P.dx * rx : tx;
    const float sy = (!VOX && dyf == 0.f) ? P.dy * ry : ty;
    const bool sv = s <= fminf(sx, fminf(sy, tz));
    if (!sv) s = kLS + fminf(tx, fminf(ty, tz));
    const float D_in = D;
    const bool fixed_before = (st & kFixed) != 0;
    float e_dep = 0.f;  // adjoint: score of this sub-step's deposit
    {
      const float absorb = M::absorbed(W, c.x * s);
      W -= absorb;
      Atot += absorb;
      if (replay) {
        const float gf = (st & kBflag) ? gf_i : 0.f;
        e_dep = gf * absorb;
        if (score) {
          D += e_dep;
        } else {
          adj.at(P, i);
          // later scores carry exp(-mua s); this deposit's own derivative is
          // d[W (1 - exp(-mua s))]/dmua = s * W_after
          adj.L = fmaf(D - e_dep, s, adj.L);
          if (gf != 0.f) adj.L = fmaf(-gf * s, W, adj.L);
          D -= e_dep;
          Dabs += fabsf(e_dep);
        }
      } else if (DEPX) {
        if (st & kBflag) dep.acc += absorb;
      } else if (!SW && (st & kBflag)) {
        if (REC && i != dep.idx) dl_deposit();
        dep.add(P.F3D, i, absorb, nvox, &P.sums->flags);
      }
    }
    sleft = sv ? 0.f : sleft - s * c.y;
    {
      bool moved = false;
      if (!TT) {  // surface detection (:556-637), on steps that leave the cell
        // (tested by every lane: the predicate costs less than a branch on sv)
        const float rel = (float)(P.ksurf - kz) * P.dz + (P.fsurf - fz);  // zsurf - z
        const float su = s * uz;
        const bool cross = !sv && ((P.det_state == NMC_DET_REFLECTANCE && su <= rel && uz < 0.f) ||
                                   (P.det_state == NMC_DET_TRANSMITTANCE && su >= rel && uz > 0.f));
        if (__builtin_expect(cross, 0)) {
          const float dl_b = rel / uz;
          if (back) st |= kFixed;  // the rest of this hop is a fixed length
          sleft = (s - dl_b) * c.y;
          fx = fmaf(dl_b, ux, fx);
          fy = fmaf(dl_b, uy, fy);
          norm_axis(kx, fx, P.dx, P.dxmax);
          norm_axis(ky, fy, P.dy, P.dymax);
          kz = P.ksurf;
          fz = P.fsurf;
          moved = true;
          float uz_t = 0.f;
          const float rsp = rfresnel(P.n1, P.n2, fabsf(uz), &uz_t);
          if (rsp < 1.f) {
            bool det = P.det_everything != 0;
            const float gx = (float)kx * P.dx + fx, gy = (float)ky * P.dy + fy;
            const float ro = sqrtf(gx * gx + gy * gy);
            if (!det) {
              const float th_exit = flt_eq(uz_t, 1.f) ? 0.f : kRAD_DEG * acosf(uz_t);
              det = (ro >= P.r_min) && (ro <= P.r_max) && (th_exit <= P.na);
            }
            if (det) {
              const float dw = W * (1.f - rsp);
              const unsigned int rbin = (unsigned int)min((int)(ro * P.rd_idr), P.rd_bins);
              if (replay) {
                const float e = P.adj_G[rbin] * dw;  // this event's score is now behind the photon
                if (score) {
                  D += e;
                } else {
                  D -= e;
                  Dabs += fabsf(e);
                }
              } else {
                const int jx = min(max(lookup_index(kx, fx, P.hx, P.ox, P.hdx), 0), P.Nx - 1);
                const int jy = min(max(lookup_index(ky, fy, P.hy, P.oy, P.hdy), 0), P.Ny - 1);
                Rd_loc += dw;
                if (!SW) {
                  const unsigned int i2d = (unsigned int)(jx * P.Ny + jy);
                  if (idx_ok(i2d, (unsigned long long)P.Nx * P.Ny, &P.sums->flags)) {
                    atomicAdd(P.Rd2D + i2d, to_fix(dw));
                    atomicAdd(P.Det2D + i2d, 1u);
                  }
                  if (P.rd_r && idx_ok(rbin, (unsigned)P.rd_bins + 1u, &P.sums->flags))
                    atomicAdd(P.rd_r + rbin, to_fix(dw));
                }
                if (REC) {  // record pass: keep (photon, bin, weight) for the backward pass
                  const unsigned long long k = atomicAdd(P.ev_count, 1ull);
                  if (k < P.ev_cap) P.ev[k] = AdjEvent{(unsigned int)pidx, rbin, dw, 0.f};
                }
              }
              if (TRACE) ++ndet;
              uz = -uz;
              W = W * rsp;
            }
          } else {
            uz = -uz;
            W = W * rsp;
          }
        }
      }
      if (!moved) {
        fx = fmaf(s, ux, fx);
        fy = fmaf(s, uy, fy);
        fz = fmaf(s, uz, fz);
        if (!sv) {
          // the face the step aims at is crossed by exactly ls*|u| (as in
          // FP64): one landing for the crossed axis, its operands selected,
          // so the lanes of a warp crossing different axes stay together
          const float ua = ax == 0 ? ux : (ax == 1 ? uy : uz);
          const float da = ax == 0 ? P.dx : (ax == 1 ? P.dy : P.dz);
          const float dma = ax == 0 ? P.dxmax : (ax == 1 ? P.dymax : P.dzmax);
          const bool p = ua >= 0.f;
          const float fa = p ? kLS * ua : fminf(fmaf(kLS, ua, da), dma);
          const int step = p ? 1 : -1;
          kx += ax == 0 ? step : 0;
          ky += ax == 1 ? step : 0;
          kz += ax == 2 ? step : 0;
          fx = ax == 0 ? fa : fx;
          fy = ax == 1 ? fa : fy;
          fz = ax == 2 ? fa : fz;
        }
        // offsets leave [0, d) only when a point lands on a face (an upper
        // face of the same-voxel end point, a tie between faces)
        // (one unsigned compare per axis: a negative offset has the sign bit
        // set and compares above d; -0 and NaN enter, and norm_axis leaves
        // them as they are)
        if (__builtin_expect((__float_as_uint(fx) >= __float_as_uint(P.dx)) | (__float_as_uint(fy) >= __float_as_uint(P.dy)) |
            (__float_as_uint(fz) >= __float_as_uint(P.dz)), 0)) {
          norm_axis(kx, fx, P.dx, P.dxmax);
          norm_axis(ky, fy, P.dy, P.dymax);
          norm_axis(kz, fz, P.dz, P.dzmax);
        }
      }
    }
    // the step length s is the hop length whose probability depends on mus
    if (back && !fixed_before) adj.M = fmaf(-D_in, s, adj.M);
    if (!sv) {
      // voxel index (:641-643): inside the grid this is the cell plus N/2
      int ix = P.hx + kx + (int)(fx >= hdx_e);
      int iy = P.hy + ky + (int)(fy >= hdy_e);
      int iz = kz;
      const bool inside = (unsigned)ix < (unsigned)P.Nx && (unsigned)iy < (unsigned)P.Ny &&
                          (unsigned)iz < (unsigned)P.Nz;
      if (__builtin_expect(!inside, 0)) {  // C truncation toward zero outside the grid
        ix = lookup_index(kx, fx, P.hx, P.ox, P.hdx);
        iy = lookup_index(ky, fy, P.hy, P.oy, P.hdy);
        iz = lookup_index(kz, fz, 0, 0, 0.f);
      }
      if (TT) {  // :981-993
        const float zrel = (float)(kz - P.ksurf) * P.dz + (fz - P.fsurf);  // z - zsurf
        if (zrel < 0.f && (st & kSurf)) {
          st &= ~kSurf;
          Rd_loc += W;
          if (TRACE) ++ndet;
          if (!SW) {
            const int jx = min(max(ix, 0), P.Nx - 1), jy = min(max(iy, 0), P.Ny - 1);
            if (idx_ok((unsigned)(jx * P.Ny + jy), (unsigned long long)P.Nx * P.Ny, &P.sums->flags))
              atomicAdd(P.Rd2D + (unsigned int)(jx * P.Ny + jy), to_fix(W));
          }
        }
        if (kz < 0) {
          kill(NMC_FATE_BOUNDARY);
          sleft = 0.f;
        }
        st |= kBflag;
      }
      if (__builtin_expect(!inside, 0)) {  // boundary modes (:646-672)
        const bool xo = (unsigned)ix >= (unsigned)P.Nx, yo = (unsigned)iy >= (unsigned)P.Ny;
        const bool zlo = iz < 0, zhi = iz >= P.Nz;
        ix = min(max(ix, 0), P.Nx - 1);
        iy = min(max(iy, 0), P.Ny - 1);
        iz = min(max(iz, 0), P.Nz - 1);
        if (P.boundaryflag == 1) {
          if (xo || yo || zlo || zhi) {
            kill(NMC_FATE_BOUNDARY);
            sleft = 0.f;
          }
        } else if (P.boundaryflag == 2 && zlo) {
          kill(NMC_FATE_BOUNDARY);
          sleft = 0.f;
          if (xo || yo || zhi) st &= ~kBflag;
        } else if (P.boundaryflag == 0 || P.boundaryflag == 2) {
          if (xo || yo || zlo || zhi) st &= ~kBflag;
        }
      }
      i = (unsigned int)(iz * NyNx + ix * P.Ny + iy);  // :675-679
      if (DEPX && i != dep.idx) {
        dep.flush(P.F3D, nvox, &P.sums->flags);
        dep.idx = i;
      }
      if (!VOX) tiss = idx_ok(i, nvox, &P.sums->flags) ? __ldg(P.V + i) : 0;
      if (ADJ && GF) gf_i = idx_ok(i, nvox, &P.sums->flags) ? __ldg(GF + i) : 0.f;
    }
    if (__builtin_expect(nsub >= P.step_cap, 0)) {  // device-side cap: not a reference behaviour
      kill(NMC_FATE_STEPCAP);
      atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
      continue;
    }
    // the hop goes on while more than ls of it is left (the reference
    // zeroes sleft <= ls, :554, :571, and loops while sleft > 0, :685),
    // at most RAY_DEPTH crossings
    if (nsub < hop_end && sleft > kLS) continue;

    // ---- SPIN (:688-731 / :1046-1097), ROULETTE (:733-748), next HOP (:501)
    const bool need_roul = W < kTHRESHOLD;
    const SpinDraws d = spin_draws<TT>(rng, need_roul, keys());
    float costheta;
    if constexpr (VOX) {
      const float4 cv = __ldg(P.vox + i);  // the voxel the photon scatters in
      costheta = hg_from_g<FAST>(cv.w, d.a);
      if (back) {
        adj.at(P, i);
        // D / mus: density of the scattering point, which also places this
        // hop's last deposit
        if (!(st & kFixed)) adj.M = fmaf(D + e_dep, cv.z, adj.M);
        if (!flt_eq(cv.w, 1.f)) adj.Q = fmaf(D, dlnhg_dg(cv.w, costheta), adj.Q);
        st &= ~kFixed;
      }
    } else {
      const PhaseConst& ph = SW ? P.sw_phase[sbase + tiss] : s_ph[tiss];
      costheta = TT ? tt_sample<FAST>(ph, d.a, d.b) : hg_sample<FAST>(ph, d.a);
    }
    spin<FAST>(costheta, TT ? d.c : d.b, ux, uy, uz);
    ++nsc;
    // W < MIN_VALUE implies W < THRESHOLD: one rare test covers both kills
    if (__builtin_expect(need_roul || (hard_kill && (int)nsc > kMAX_SCATT), 0)) {
      if (need_roul) {
        if (d.roul <= kCHANCE)
          W /= kCHANCE;
        else
          kill(NMC_FATE_ROULETTE);
      }
      if (hard_kill && (W < kMIN_VALUE || (int)nsc > kMAX_SCATT))
        kill(W < kMIN_VALUE ? NMC_FATE_MINWEIGHT : NMC_FATE_MAXSCATT);
    }
    if (TRACE && nev < P.trace.k_events) {
      if (idx_ok(pidx, P.n, &P.sums->flags)) P.trace.events[pidx * P.trace.k_events + nev] =
          make_float4((float)kx * P.dx + fx, (float)ky * P.dy + fy, (float)kz * P.dz + fz, W);
      ++nev;
    }
    sleft = M::neglog(d.step);
    hop_end = nsub + kRAY_DEPTH + 1;
  }

  if (REC && dl_chunk < kDeadChunk) P.dl_fill[dl_chunk] = dl_pos;
  __syncthreads();
  if (threadIdx.x < 5 && s_tot[threadIdx.x]) {
    unsigned long long* dst = threadIdx.x == 0   ? &P.sums->photons
                              : threadIdx.x == 1 ? &P.sums->substeps
                              : threadIdx.x == 2 ? &P.sums->scatters
                              : threadIdx.x == 3 ? &P.sums->A
                                                 : &P.sums->rd;
    atomicAdd(dst, s_tot[threadIdx.x]);
  }
  if (threadIdx.x == 0 && s_rd2 != 0.0) atomicAdd(&P.sums->rd_sumsq, s_rd2);
}

}  // namespace
}  // namespace nmc
