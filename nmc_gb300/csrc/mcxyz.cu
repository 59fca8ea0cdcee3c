// mcxyz.cu - voxel photon transport (MCXYZKernel, kernels.metal:321-754, and
// the two-term variant MCXYZKernelTT, kernels.metal:757-1118) as one
// persistent CUDA kernel for sm_103a.
//
// Design:
//  * persistent threads: the grid fills the GPU once; a thread that retires a
//    photon takes the next photon index from a warp-aggregated counter;
//  * one voxel sub-step per loop trip (the reference's inner do-while over
//    RAY_DEPTH crossings, :505-685, flattened), SPIN/roulette predicated at
//    the hop's end, so lanes of a warp stay on the same trip;
//  * positions are an integer voxel-lattice cell plus an FP32 offset in the
//    cell: the "littlest step" ls = 1e-7 (definitions.h:59) stays ~200 ulps
//    above the offset's rounding, so FP32 stepping walks voxels the way FP64
//    arithmetic does (the reference's global FP32 coordinates round ls away
//    at mm-scale positions and stall photons at faces);
//  * optical properties live in shared memory; the uint8 tissue map is read
//    through the read-only path (L2-resident: 8 MB for 200^3);
//  * deposits are merged in a register while the photon stays in one voxel
//    and flushed as u64 fixed-point atomics, which keeps F3D exact and
//    bit-reproducible.
#include <cuda_runtime.h>

#include <type_traits>

#include "engine.h"

namespace nmc {
namespace {

__device__ __forceinline__ void to_lattice(float x, float d, float dmax, int& k, float& f) {
  const float q = floorf(__fdiv_rn(x, d));
  k = (int)q;
  f = fmaf(-q, d, x);
  if (f < 0.f) {
    --k;
    f += d;
    if (f > dmax) f = dmax;
  } else if (f >= d) {
    ++k;
    f -= d;
  }
}

__device__ __forceinline__ void norm_axis(int& k, float& f, float d, float dmax) {
  if (f >= d) {
    ++k;
    f -= d;
    if (f > dmax) f = dmax;
  } else if (f < 0.f) {
    --k;
    f += d;
    if (f > dmax) f = dmax;
  }
}

// (int)(H2/2 + k + f/d) with C truncation toward zero, H2 = 2*half: the
// reference's index formulas `(int)(Nx/2.0 + x/dx)` (kernels.metal:641-643,
// H2 = Nx) and `(int)(Nx/2 + x/dx)` (:472-474, H2 = 2*(Nx/2)).
__device__ __forceinline__ int lookup_index(int k, float f, float id, int H2) {
  float t = f * id;
  int A = (H2 >> 1) + k;
  if (H2 & 1) {
    t += 0.5f;
    if (t >= 1.f) {
      ++A;
      t -= 1.f;
    }
  }
  return A >= 0 ? A : (t > 0.f ? A + 1 : A);
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

template <bool TT, class RNG, bool TRACE>
__global__ void __launch_bounds__(256) mcxyz_kernel(const XyzParams P) {
  __shared__ float4 s_core[NMC_NTISS];
  __shared__ PhaseConst s_ph[NMC_NTISS];
  for (int t = threadIdx.x; t < NMC_NTISS; t += blockDim.x) {
    s_core[t] = P.core[t];
    s_ph[t] = P.phase[t];
  }
  __syncthreads();

  const bool hard_kill = !(P.flags & NMC_FLAG_NO_HARD_KILL);
  const int NyNx = P.Ny * P.Nx;

  unsigned long long t_ph = 0, t_sub = 0, t_sc = 0, t_A = 0, t_rd = 0;
  double t_rd2 = 0.0;

  RNG rng;
  int kx = 0, ky = 0, kz = 0;
  float fx = 0.f, fy = 0.f, fz = 0.f, ux = 0.f, uy = 0.f, uz = 1.f;
  float iux = 0.f, iuy = 0.f, iuz = 1.f;
  float W = 0.f, sleft = 0.f, mua = 0.f, mus = 1.f, imus = 1.f, Rd_loc = 0.f, Atot = 0.f;
  unsigned int i = 0;
  int tiss = 0, bflag = 1, surfflag = 1, depth = 0;
  uint32_t nsc = 0, nsub = 0, ndet = 0, fate = NMC_FATE_ALIVE, nev = 0;
  unsigned long long pidx = 0;
  bool alive = false, have = false, hop_start = true;
  Deposit dep{0xFFFFFFFFu, 0.f};

  while (true) {
    if (!alive) {
      if (have) {  // retire the finished photon
        dep.flush(P.F3D);
        const unsigned long long pid = P.first + pidx;
        if (Rd_loc > 0.f) atomicAdd(P.rd_slots + (pid % P.nslots), to_fix(Rd_loc));  // :753
        t_rd += to_fix(Rd_loc);
        t_rd2 += (double)Rd_loc * (double)Rd_loc;
        t_A += to_fix(Atot);
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
          r.detected = Rd_loc;
          r.x = (float)kx * P.dx + fx;
          r.y = (float)ky * P.dy + fy;
          r.z = (float)kz * P.dz + fz;
          P.trace.recs[pidx] = r;
        }
      }
      pidx = next_photon(&P.sums->work);
      if (pidx >= P.n) break;
      have = true;
      const unsigned long long pid = P.first + pidx;
      if constexpr (std::is_same<RNG, TausRng>::value) {
        rng.init_photon(pid, P.rng.batch, TT, P.rng.tt_replay != 0);
      } else {
        rng.init(P.rng.k0, P.rng.k1, pid);
      }
      // ---- LAUNCH (kernels.metal:349-463; two-term :778-870)
      W = 1.f;
      float x = 0.f, y = 0.f, z = 0.f;
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
        while ((r = rng.launch_u()) <= 0.f) {
        }
        float rad = gauss ? P.radius * sqrtf(-logf(r)) : P.radius * sqrtf(r);
        while ((r = rng.launch_u()) <= 0.f) {
        }
        sincospif(2.f * r, &sp, &cp);
        x = P.xs + rad * cp;
        y = P.ys + rad * sp;
        z = P.zs;
        while ((r = rng.launch_u()) <= 0.f) {
        }
        rad = P.waist * sqrtf(r);
        while ((r = rng.launch_u()) <= 0.f) {
        }
        sincospif(2.f * r, &sp, &cp);
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
        const float costheta = 1.f - 2.f * rng.launch_u();
        const float sintheta = sqrtf(fmaxf(1.f - costheta * costheta, 0.f));
        float sp, cp;
        sincospif(2.f * rng.launch_u(), &sp, &cp);
        x = P.xs;
        y = P.ys;
        z = P.zs;
        ux = sintheta * cp;
        uy = sintheta * sp;
        uz = costheta;
      } else if (P.mcflag == 3) {
        float r;
        while ((r = rng.launch_u()) <= 0.f) {
        }
        x = P.radius * (r * 2.f - 1.f);
        while ((r = rng.launch_u()) <= 0.f) {
        }
        y = P.radius * (r * 2.f - 1.f);
        z = P.zs;
        ux = 0.f;
        uy = 0.f;
        uz = 1.f;
      } else if (P.mcflag == 4) {
        z = P.zs;
        ux = 0.f;
        uy = 0.f;
        uz = 1.f;
      }
      to_lattice(x, P.dx, P.dxmax, kx, fx);
      to_lattice(y, P.dy, P.dymax, ky, fy);
      to_lattice(z, P.dz, P.dzmax, kz, fz);
      iux = __frcp_rn(fabsf(ux));
      iuy = __frcp_rn(fabsf(uy));
      iuz = __frcp_rn(fabsf(uz));
      // launch voxel (:472-487): integer Nx/2 in this formula
      int ix = lookup_index(kx, fx, P.idx, 2 * (P.Nx / 2));
      int iy = lookup_index(ky, fy, P.idy, 2 * (P.Ny / 2));
      int iz = lookup_index(kz, fz, P.idz, 0);
      ix = min(max(ix, 0), P.Nx - 1);
      iy = min(max(iy, 0), P.Ny - 1);
      iz = min(max(iz, 0), P.Nz - 1);
      i = (unsigned int)(iz * NyNx + ix * P.Ny + iy);
      tiss = __ldg(P.V + i);
      const float4 c = s_core[tiss];
      mua = c.x;
      mus = c.y;
      imus = c.z;
      bflag = 1;
      surfflag = 1;
      Rd_loc = 0.f;
      Atot = 0.f;
      nsc = nsub = ndet = nev = 0;
      fate = NMC_FATE_ALIVE;
      alive = true;
      hop_start = true;
      dep.idx = 0xFFFFFFFFu;
      dep.acc = 0.f;
    }

    if (hop_start) {  // HOP (:501-503)
      rng.new_hop();
      float r;
      while ((r = rng.step_u()) <= 0.f) {
      }
      sleft = -logf(r);
      depth = 0;
      hop_start = false;
    }

    // ---- one voxel sub-step (:505-682)
    float s = sleft * imus;
    const float ex = fmaf(s, ux, fx), ey = fmaf(s, uy, fy), ez = fmaf(s, uz, fz);
    const bool sv = (ex <= P.dx) && (ex >= 0.f || (fx == 0.f && ex >= -P.dx)) && (ey <= P.dy) &&
                    (ey >= 0.f || (fy == 0.f && ey >= -P.dy)) && (ez >= 0.f) && (ez <= P.dz);
    ++nsub;
    if (sv) {  // SameVoxel (helpers.metal:27-39): move, drop, end the hop
      fx = ex;
      fy = ey;
      fz = ez;
      norm_axis(kx, fx, P.dx, P.dxmax);
      norm_axis(ky, fy, P.dy, P.dymax);
      norm_axis(kz, fz, P.dz, P.dzmax);
      const float absorb = -W * expm1f(-mua * s);
      W -= absorb;
      Atot += absorb;
      if (bflag) dep.add(P.F3D, i, absorb);
      sleft = 0.f;
    } else {
      // FindVoxelFace2 (helpers.metal:85-114) in cell-local form
      const float tx = (ux >= 0.f ? P.dx - fx : fx) * iux;
      const float ty = (uy >= 0.f ? P.dy - fy : fy) * iuy;
      const float tz = (uz >= 0.f ? P.dz - fz : fz) * iuz;
      const int ax = (tx <= ty) ? ((tx <= tz) ? 0 : 2) : ((ty <= tz) ? 1 : 2);
      s = kLS + fminf(tx, fminf(ty, tz));
      const float absorb = -W * expm1f(-mua * s);
      W -= absorb;
      Atot += absorb;
      if (bflag) dep.add(P.F3D, i, absorb);
      sleft -= s * mus;
      if (sleft <= kLS) sleft = 0.f;

      bool moved = false;
      if (!TT) {  // surface detection (:556-637)
        const float rel = (float)(P.ksurf - kz) * P.dz + (P.fsurf - fz);  // zsurf - z
        const float su = s * uz;
        const bool cross = (P.det_state == NMC_DET_REFLECTANCE && su <= rel && uz < 0.f) ||
                           (P.det_state == NMC_DET_TRANSMITTANCE && su >= rel && uz > 0.f);
        if (cross) {
          const float dl_b = rel / uz;
          sleft = (s - dl_b) * mus;
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
              const int jx = min(max(lookup_index(kx, fx, P.idx, P.Nx), 0), P.Nx - 1);
              const int jy = min(max(lookup_index(ky, fy, P.idy, P.Ny), 0), P.Ny - 1);
              const float dw = W * (1.f - rsp);
              Rd_loc += dw;
              const unsigned int i2d = (unsigned int)(jx * P.Ny + jy);
              atomicAdd(P.Rd2D + i2d, to_fix(dw));
              atomicAdd(P.Det2D + i2d, 1u);
              ++ndet;
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
        // the face the step aims at is crossed by exactly ls*|u| (as in FP64)
        if (ax == 0) {
          if (ux >= 0.f) { ++kx; fx = kLS * ux; } else { --kx; fx = fminf(P.dx + kLS * ux, P.dxmax); }
        } else if (ax == 1) {
          if (uy >= 0.f) { ++ky; fy = kLS * uy; } else { --ky; fy = fminf(P.dy + kLS * uy, P.dymax); }
        } else {
          if (uz >= 0.f) { ++kz; fz = kLS * uz; } else { --kz; fz = fminf(P.dz + kLS * uz, P.dzmax); }
        }
        norm_axis(kx, fx, P.dx, P.dxmax);
        norm_axis(ky, fy, P.dy, P.dymax);
        norm_axis(kz, fz, P.dz, P.dzmax);
      }
      int ix = lookup_index(kx, fx, P.idx, P.Nx);  // :641-643
      int iy = lookup_index(ky, fy, P.idy, P.Ny);
      int iz = lookup_index(kz, fz, P.idz, 0);
      if (TT) {  // :981-993
        const float zrel = (float)(kz - P.ksurf) * P.dz + (fz - P.fsurf);  // z - zsurf
        if (zrel < 0.f && surfflag == 1) {
          surfflag = 0;
          Rd_loc += W;
          ++ndet;
          const int jx = min(max(ix, 0), P.Nx - 1), jy = min(max(iy, 0), P.Ny - 1);
          atomicAdd(P.Rd2D + (unsigned int)(jx * P.Ny + jy), to_fix(W));
        }
        if (kz < 0) {
          if (alive) fate = NMC_FATE_BOUNDARY;
          alive = false;
          sleft = 0.f;
        }
        bflag = 1;
      }
      if (P.boundaryflag == 0) {  // :646-672
        if (iz >= P.Nz) { iz = P.Nz - 1; bflag = 0; }
        if (ix >= P.Nx) { ix = P.Nx - 1; bflag = 0; }
        if (iy >= P.Ny) { iy = P.Ny - 1; bflag = 0; }
        if (iz < 0) { iz = 0; bflag = 0; }
        if (ix < 0) { ix = 0; bflag = 0; }
        if (iy < 0) { iy = 0; bflag = 0; }
      } else if (P.boundaryflag == 1) {
        const bool out = iz >= P.Nz || ix >= P.Nx || iy >= P.Ny || iz < 0 || ix < 0 || iy < 0;
        iz = min(max(iz, 0), P.Nz - 1);
        ix = min(max(ix, 0), P.Nx - 1);
        iy = min(max(iy, 0), P.Ny - 1);
        if (out) {
          if (alive) fate = NMC_FATE_BOUNDARY;
          alive = false;
          sleft = 0.f;
        }
      } else if (P.boundaryflag == 2) {
        if (iz >= P.Nz) { iz = P.Nz - 1; bflag = 0; }
        if (ix >= P.Nx) { ix = P.Nx - 1; bflag = 0; }
        if (iy >= P.Ny) { iy = P.Ny - 1; bflag = 0; }
        if (iz < 0) {
          iz = 0;
          if (alive) fate = NMC_FATE_BOUNDARY;
          alive = false;
          sleft = 0.f;
        }
        if (ix < 0) { ix = 0; bflag = 0; }
        if (iy < 0) { iy = 0; bflag = 0; }
      }
      i = (unsigned int)(iz * NyNx + ix * P.Ny + iy);  // :675-679
      tiss = __ldg(P.V + i);
      const float4 c = s_core[tiss];
      mua = c.x;
      mus = c.y;
      imus = c.z;
    }
    ++depth;
    if (nsub >= P.step_cap) {  // device-side cap: not a reference behaviour
      if (alive) fate = NMC_FATE_STEPCAP;
      alive = false;
      atomicOr(&P.sums->flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
      continue;
    }
    if (depth <= kRAY_DEPTH && sleft > 0.f) continue;  // :685

    // ---- SPIN (:688-731 / :1046-1097) and ROULETTE (:733-748)
    const PhaseConst& ph = s_ph[tiss];
    const float costheta = TT ? tt_sample(ph, rng) : hg_sample(ph, rng.cos_u());
    spin(costheta, rng.psi_u(), ux, uy, uz);
    iux = __frcp_rn(fabsf(ux));
    iuy = __frcp_rn(fabsf(uy));
    iuz = __frcp_rn(fabsf(uz));
    ++nsc;
    if (W < kTHRESHOLD) {
      if (rng.roul_u() <= kCHANCE) {
        W /= kCHANCE;
      } else {
        if (alive) fate = NMC_FATE_ROULETTE;
        alive = false;
      }
    }
    if (hard_kill && (W < kMIN_VALUE || (int)nsc > kMAX_SCATT)) {
      if (alive) fate = W < kMIN_VALUE ? NMC_FATE_MINWEIGHT : NMC_FATE_MAXSCATT;
      alive = false;
    }
    if (TRACE && nev < P.trace.k_events) {
      P.trace.events[pidx * P.trace.k_events + nev] =
          make_float4((float)kx * P.dx + fx, (float)ky * P.dy + fy, (float)kz * P.dz + fz, W);
      ++nev;
    }
    hop_start = true;
  }

  warp_add_u64(&P.sums->photons, t_ph);
  warp_add_u64(&P.sums->substeps, t_sub);
  warp_add_u64(&P.sums->scatters, t_sc);
  warp_add_u64(&P.sums->A, t_A);
  warp_add_u64(&P.sums->rd, t_rd);
  warp_add_f64(&P.sums->rd_sumsq, t_rd2);
}

template <bool TT, bool TRACE>
cudaError_t launch_t(const XyzParams& p, int grid, int block, cudaStream_t st) {
  if (p.rng.kind == NMC_RNG_TAUS_REF)
    mcxyz_kernel<TT, TausRng, TRACE><<<grid, block, 0, st>>>(p);
  else
    mcxyz_kernel<TT, PhiloxRng<TT>, TRACE><<<grid, block, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_mcxyz(const XyzParams& p, bool two_term, bool trace, int grid, int block,
                         cudaStream_t stream) {
  if (two_term) return trace ? launch_t<true, true>(p, grid, block, stream)
                             : launch_t<true, false>(p, grid, block, stream);
  return trace ? launch_t<false, true>(p, grid, block, stream)
               : launch_t<false, false>(p, grid, block, stream);
}

cudaError_t mcxyz_occupancy(bool two_term, bool trace, int block, int* blocks_per_sm) {
  const void* f;
  if (two_term)
    f = trace ? (const void*)mcxyz_kernel<true, PhiloxRng<true>, true>
              : (const void*)mcxyz_kernel<true, PhiloxRng<true>, false>;
  else
    f = trace ? (const void*)mcxyz_kernel<false, PhiloxRng<false>, true>
              : (const void*)mcxyz_kernel<false, PhiloxRng<false>, false>;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, f, block, 0);
}

}  // namespace nmc
