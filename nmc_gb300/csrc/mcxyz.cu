// mcxyz.cu - voxel photon transport (MCXYZKernel, kernels.metal:321-754, and
// the two-term variant MCXYZKernelTT, kernels.metal:757-1118) as one
// persistent CUDA kernel for sm_103a.
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

constexpr uint32_t kAlive = 1u, kBflag = 2u, kSurf = 4u, kHave = 8u;

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
  __device__ __forceinline__ void flush(unsigned long long* F3D) {
    if (acc > 0.f) atomicAdd(F3D + idx, to_fix(acc));
    acc = 0.f;
  }
  __device__ __forceinline__ void add(unsigned long long* F3D, unsigned int i, float v) {
    if (i != idx) {
      flush(F3D);
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

template <bool TT, class RNG, bool TRACE, bool FAST>
__global__ void __launch_bounds__(256, 4) mcxyz_kernel(const XyzParams P) {
  using M = Math<FAST>;
  __shared__ float4 s_core[NMC_NTISS];
  __shared__ PhaseConst s_ph[NMC_NTISS];
  __shared__ unsigned long long s_tot[5];  // photons, substeps, scatters, A, rd
  __shared__ double s_rd2;
  for (int t = threadIdx.x; t < NMC_NTISS; t += blockDim.x) {
    s_core[t] = P.core[t];
    s_ph[t] = P.phase[t];
  }
  if (threadIdx.x < 5) s_tot[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) s_rd2 = 0.0;
  __syncthreads();

  const uint32_t k0 = P.rng.k0, k1 = P.rng.k1;
  const bool hard_kill = !(P.flags & NMC_FLAG_NO_HARD_KILL);
  const int NyNx = P.Ny * P.Nx;

  RNG rng;
  int kx = 0, ky = 0, kz = 0, tiss = 0, depth = 0;
  float fx = 0.f, fy = 0.f, fz = 0.f, ux = 0.f, uy = 0.f, uz = 1.f;
  float W = 0.f, sleft = 0.f, Rd_loc = 0.f, Atot = 0.f;
  unsigned int i = 0, slot = 0, nsc = 0, nsub = 0, st = 0;
  unsigned long long pidx = 0;
  uint32_t fate = NMC_FATE_ALIVE, ndet = 0, nev = 0;  // trace only
  Deposit dep{0xFFFFFFFFu, 0.f};

  auto kill = [&](uint32_t why) {
    if (TRACE && (st & kAlive)) fate = why;
    st &= ~kAlive;
  };

  while (true) {
    if (!(st & kAlive)) {
      if (st & kHave) {  // retire the finished photon
        dep.flush(P.F3D);
        if (Rd_loc > 0.f) atomicAdd(P.rd_slots + slot, to_fix(Rd_loc));  // :753
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
          P.trace.recs[pidx] = r;
        }
      }
      pidx = next_photon(&P.sums->work);
      if (pidx >= P.n) break;
      const unsigned long long pid = P.first + pidx;
      slot = (unsigned int)(pid % P.nslots);
      float x, y, z;
      if constexpr (std::is_same<RNG, TausRng>::value) {
        rng.init_photon(pid, P.rng.batch, TT, P.rng.tt_replay != 0);
        typename TausRng::Seq d{&rng};
        launch_photon<TT, FAST>(P, d, x, y, z, ux, uy, uz, W);
      } else {
        rng.init(pid);
        LaunchDraws d{rng.block(0xFFFFFFFFu, k0, k1), 0};
        launch_photon<TT, FAST>(P, d, x, y, z, ux, uy, uz, W);
      }
      to_lattice(x, P.dx, P.dxmax, kx, fx);
      to_lattice(y, P.dy, P.dymax, ky, fy);
      to_lattice(z, P.dz, P.dzmax, kz, fz);
      const int ix = min(max(lookup_index(kx, fx, P.Nx / 2, 0, 0.f), 0), P.Nx - 1);  // :472-480
      const int iy = min(max(lookup_index(ky, fy, P.Ny / 2, 0, 0.f), 0), P.Ny - 1);
      const int iz = min(max(lookup_index(kz, fz, 0, 0, 0.f), 0), P.Nz - 1);
      i = (unsigned int)(iz * NyNx + ix * P.Ny + iy);
      tiss = __ldg(P.V + i);
      sleft = M::neglog(rng.first_step(k0, k1));  // HOP (:501-502)
      depth = 0;
      Rd_loc = Atot = 0.f;
      nsc = nsub = 0;
      if (TRACE) {
        fate = NMC_FATE_ALIVE;
        ndet = nev = 0;
      }
      st = kAlive | kBflag | kSurf | kHave;
      dep.idx = 0xFFFFFFFFu;
      dep.acc = 0.f;
    }

    // ---- one voxel sub-step (:505-682).  The same-voxel move (:515-533) and
    // the step to the nearest face (:534-682) share one straight path; only
    // the face landing, the voxel lookup and the tissue load are predicated
    // on the crossing, so the lanes of a warp stay together.
    const float4 c = s_core[tiss];  // mua, mus, 1/mus, g
    float s = sleft * c.z;
    ++nsub;
    ++depth;
    // FindVoxelFace2 (helpers.metal:85-114) in cell-local form: path length
    // to the face ahead on each axis
    const float rx = M::rcp(fabsf(ux)), ry = M::rcp(fabsf(uy)), rz = M::rcp(fabsf(uz));
    const float tx = (ux >= 0.f ? P.dx - fx : fx) * rx;
    const float ty = (uy >= 0.f ? P.dy - fy : fy) * ry;
    const float tz = (uz >= 0.f ? P.dz - fz : fz) * rz;
    const int ax = (tx <= ty) ? ((tx <= tz) ? 0 : 2) : ((ty <= tz) ? 1 : 2);
    // SameVoxel (helpers.metal:27-39): the end point stays in the cell, upper
    // faces included; a photon on a lower x or y face moving down stays for
    // up to one cell (the reference compares with the cell below's upper face)
    const float sx = (ux < 0.f && fx == 0.f) ? P.dx * rx : tx;
    const float sy = (uy < 0.f && fy == 0.f) ? P.dy * ry : ty;
    const bool sv = s <= fminf(sx, fminf(sy, tz));
    if (!sv) s = kLS + fminf(tx, fminf(ty, tz));
    {
      const float absorb = M::absorbed(W, c.x * s);
      W -= absorb;
      Atot += absorb;
      if (st & kBflag) dep.add(P.F3D, i, absorb);
    }
    sleft = sv ? 0.f : sleft - s * c.y;
    if (sleft <= kLS) sleft = 0.f;
    {
      bool moved = false;
      if (!TT && !sv) {  // surface detection (:556-637)
        const float rel = (float)(P.ksurf - kz) * P.dz + (P.fsurf - fz);  // zsurf - z
        const float su = s * uz;
        const bool cross = (P.det_state == NMC_DET_REFLECTANCE && su <= rel && uz < 0.f) ||
                           (P.det_state == NMC_DET_TRANSMITTANCE && su >= rel && uz > 0.f);
        if (cross) {
          const float dl_b = rel / uz;
          sleft = (s - dl_b) * c.y;
          if (sleft <= kLS) sleft = 0.f;
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
            if (!det) {
              const float th_exit = flt_eq(uz_t, 1.f) ? 0.f : kRAD_DEG * acosf(uz_t);
              const float gx = (float)kx * P.dx + fx, gy = (float)ky * P.dy + fy;
              const float ro = sqrtf(gx * gx + gy * gy);
              det = (ro >= P.r_min) && (ro <= P.r_max) && (th_exit <= P.na);
            }
            if (det) {
              const int jx = min(max(lookup_index(kx, fx, P.hx, P.ox, P.hdx), 0), P.Nx - 1);
              const int jy = min(max(lookup_index(ky, fy, P.hy, P.oy, P.hdy), 0), P.Ny - 1);
              const float dw = W * (1.f - rsp);
              Rd_loc += dw;
              const unsigned int i2d = (unsigned int)(jx * P.Ny + jy);
              atomicAdd(P.Rd2D + i2d, to_fix(dw));
              atomicAdd(P.Det2D + i2d, 1u);
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
          // the face the step aims at is crossed by exactly ls*|u| (as in FP64)
          if (ax == 0) {
            const bool p = ux >= 0.f;
            kx += p ? 1 : -1;
            fx = p ? kLS * ux : fminf(fmaf(kLS, ux, P.dx), P.dxmax);
          } else if (ax == 1) {
            const bool p = uy >= 0.f;
            ky += p ? 1 : -1;
            fy = p ? kLS * uy : fminf(fmaf(kLS, uy, P.dy), P.dymax);
          } else {
            const bool p = uz >= 0.f;
            kz += p ? 1 : -1;
            fz = p ? kLS * uz : fminf(fmaf(kLS, uz, P.dz), P.dzmax);
          }
        }
        // offsets leave [0, d) only when a point lands on a face (an upper
        // face of the same-voxel end point, a tie between faces)
        if (fx < 0.f || fx >= P.dx || fy < 0.f || fy >= P.dy || fz < 0.f || fz >= P.dz) {
          norm_axis(kx, fx, P.dx, P.dxmax);
          norm_axis(ky, fy, P.dy, P.dymax);
          norm_axis(kz, fz, P.dz, P.dzmax);
        }
      }
    }
    if (!sv) {
      // voxel index (:641-643): inside the grid this is the cell plus N/2
      int ix = P.hx + kx + (P.ox ? (int)(fx >= P.hdx) : 0);
      int iy = P.hy + ky + (P.oy ? (int)(fy >= P.hdy) : 0);
      int iz = kz;
      const bool inside = (unsigned)ix < (unsigned)P.Nx && (unsigned)iy < (unsigned)P.Ny &&
                          (unsigned)iz < (unsigned)P.Nz;
      if (!inside) {  // C truncation toward zero outside the grid
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
          const int jx = min(max(ix, 0), P.Nx - 1), jy = min(max(iy, 0), P.Ny - 1);
          atomicAdd(P.Rd2D + (unsigned int)(jx * P.Ny + jy), to_fix(W));
        }
        if (kz < 0) {
          kill(NMC_FATE_BOUNDARY);
          sleft = 0.f;
        }
        st |= kBflag;
      }
      if (!inside) {  // boundary modes (:646-672)
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
      tiss = __ldg(P.V + i);
    }
    if (nsub >= P.step_cap) {  // device-side cap: not a reference behaviour
      kill(NMC_FATE_STEPCAP);
      atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
      continue;
    }
    if (depth <= kRAY_DEPTH && sleft > 0.f) continue;  // :685

    // ---- SPIN (:688-731 / :1046-1097), ROULETTE (:733-748), next HOP (:501)
    const PhaseConst& ph = s_ph[tiss];
    const bool need_roul = W < kTHRESHOLD;
    const SpinDraws d = spin_draws<TT>(rng, need_roul, k0, k1);
    const float costheta = TT ? tt_sample<FAST>(ph, d.a, d.b) : hg_sample<FAST>(ph, d.a);
    spin<FAST>(costheta, TT ? d.c : d.b, ux, uy, uz);
    ++nsc;
    if (need_roul) {
      if (d.roul <= kCHANCE)
        W /= kCHANCE;
      else
        kill(NMC_FATE_ROULETTE);
    }
    if (hard_kill && (W < kMIN_VALUE || (int)nsc > kMAX_SCATT))
      kill(W < kMIN_VALUE ? NMC_FATE_MINWEIGHT : NMC_FATE_MAXSCATT);
    if (TRACE && nev < P.trace.k_events) {
      P.trace.events[pidx * P.trace.k_events + nev] =
          make_float4((float)kx * P.dx + fx, (float)ky * P.dy + fy, (float)kz * P.dz + fz, W);
      ++nev;
    }
    sleft = M::neglog(d.step);
    depth = 0;
  }

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

template <bool TT, bool TRACE, bool FAST>
const void* kernel_for(uint32_t rng_kind) {
  if (rng_kind == NMC_RNG_TAUS_REF) return (const void*)mcxyz_kernel<TT, TausRng, TRACE, FAST>;
  return (const void*)mcxyz_kernel<TT, PhiloxRng<TT>, TRACE, FAST>;
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
