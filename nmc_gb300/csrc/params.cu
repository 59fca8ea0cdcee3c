// params.cu - host-side construction of the kernels' parameter blocks from
// the reference's configuration (RunParams / TissueParams,
// definitions.h:186-218) and the extension knobs.  Derived constants are
// computed in double and rounded once to float.
#include <cmath>

#include "engine.h"

namespace nmc {

namespace {

bool flt_eq_host(float a, float b) {  // FltEq, helpers.metal:21-25
  const float e = b * 1.1920928955078125e-7f * 2.f;
  return (a >= b - e) && (a <= b + e);
}

// zsurf = k * dz + f with 0 <= f < dz.
void lattice_split(float zsurf, float dz, int* k, float* f) {
  const double q = std::floor((double)zsurf / (double)dz);
  double rem = (double)zsurf - q * (double)dz;
  int kk = (int)q;
  if (rem < 0) {
    rem += dz;
    --kk;
  }
  if (rem >= dz) {
    rem -= dz;
    ++kk;
  }
  *k = kk;
  *f = (float)rem;
  if (*f >= dz) *f = std::nextafter(dz, 0.f);
}

}  // namespace

// Photons a thread takes from the work queue at a time: the largest power
// of two not above the request, 1 to 64.
uint32_t fetch_run(uint32_t want) {
  uint32_t p = 1;
  while (p < 64 && 2 * p <= want) p *= 2;
  return p;
}

bool tissue_usable(const nmc_tissue_params& tp, int t) {
  return std::isfinite(tp.muav[t]) && tp.muav[t] >= 0.f && tp.musv[t] > 0.f && std::isfinite(tp.musv[t]) &&
         std::isfinite(tp.gv[t]) && std::isfinite(tp.gf[t]) && std::isfinite(tp.af[t]) &&
         std::isfinite(tp.gb[t]) && std::isfinite(tp.ab[t]) && std::isfinite(tp.CC[t]);
}

PhaseConst phase_const(const nmc_tissue_params& tp, int t) {
  PhaseConst p{};
  const double g = tp.gv[t];
  p.hg_mode = (tp.gv[t] == 0.f) ? 1 : (flt_eq_host(tp.gv[t], 1.f) ? 2 : 0);
  if (p.hg_mode == 0) {  // kernels.metal:696-703
    p.hg_a = (float)(1.0 - g * g);
    p.hg_b = (float)(1.0 - g);
    p.hg_c = (float)(2.0 * g);
    p.hg_d = (float)(1.0 + g * g);
    p.hg_e = (float)(1.0 / (2.0 * g));
  }
  const double gf = tp.gf[t], af = tp.af[t], gb = tp.gb[t], ab = tp.ab[t];  // :894-905
  p.cc = tp.CC[t];
  p.f_iso = gf == 0.0;
  p.b_iso = gb == 0.0;
  if (!p.f_iso) {
    p.f_q1e = (float)((1.0 + gf * gf) / (2.0 * gf));
    p.f_iq2 = (float)(1.0 / std::pow(1.0 - gf, 2.0 * af));
    p.f_iq3 = (float)(1.0 / std::pow(1.0 + gf, 2.0 * af));
    p.f_ninva = (float)(-1.0 / af);
    p.f_e = (float)(1.0 / (2.0 * gf));
  }
  if (!p.b_iso) {
    p.b_q1e = (float)((1.0 + gb * gb) / (2.0 * gb));
    p.b_iq2 = (float)(1.0 / std::pow(1.0 - gb, 2.0 * ab));
    p.b_iq3 = (float)(1.0 / std::pow(1.0 + gb, 2.0 * ab));
    p.b_ninva = (float)(-1.0 / ab);
    p.b_e = (float)(1.0 / (2.0 * gb));
  }
  return p;
}

RngParams rng_params(const nmc_ext& e, int sim) {
  RngParams r{};
  r.kind = e.rng;
  r.k0 = (uint32_t)e.seed;
  r.k1 = (uint32_t)(e.seed >> 32);
  philox_round_keys(r.k0, r.k1, r.rk);
  r.tt_replay = (sim == NMC_SIM_MCXYZ_TT && (e.flags & NMC_FLAG_TT_REPLAY_RUN1)) ? 1u : 0u;
  r.batch = e.photons_per_dispatch;
  return r;
}

void fill_xyz(XyzParams& p, const nmc_run_params& rp, const nmc_tissue_params& tp, const nmc_ext& e,
              int sim) {
  p.Nx = rp.Nx;
  p.Ny = rp.Ny;
  p.Nz = rp.Nz;
  p.dx = rp.dx;
  p.dy = rp.dy;
  p.dz = rp.dz;
  p.idx = (float)(1.0 / rp.dx);
  p.idy = (float)(1.0 / rp.dy);
  p.idz = (float)(1.0 / rp.dz);
  p.dxmax = std::nextafter(rp.dx, 0.f);
  p.dymax = std::nextafter(rp.dy, 0.f);
  p.dzmax = std::nextafter(rp.dz, 0.f);
  p.hx = rp.Nx / 2;
  p.hy = rp.Ny / 2;
  p.ox = rp.Nx & 1;
  p.oy = rp.Ny & 1;
  p.hdx = (float)(0.5 * rp.dx);
  p.hdy = (float)(0.5 * rp.dy);
  lattice_split(rp.zsurf, rp.dz, &p.ksurf, &p.fsurf);
  p.boundaryflag = rp.boundaryflag;
  p.det_state = rp.det_state;
  p.launchflag = rp.launchflag;
  p.mcflag = rp.mcflag;
  p.xs = rp.xs;
  p.ys = rp.ys;
  p.zs = rp.zs;
  p.ux0 = rp.ux0;
  p.uy0 = rp.uy0;
  p.uz0 = rp.uz0;
  p.radius = rp.radius;
  p.waist = rp.waist;
  p.zfocus = rp.zfocus;
  p.n1 = rp.n1;
  p.n2 = rp.n2;
  if (flt_eq_host(rp.xd, 0.f)) {  // kernels.metal:590-599
    p.r_min = 0.f;
    p.r_max = rp.det_radius;
  } else {
    p.r_min = rp.xd - rp.det_radius;
    p.r_max = p.r_min + 2.f * rp.det_radius;
  }
  p.na = rp.na;
  p.det_everything = (p.r_min <= 0.f && std::isinf(p.r_max) && rp.na >= 90.f) ? 1 : 0;
  for (int t = 0; t < NMC_NTISS; ++t) {
    const float mus = tp.musv[t];
    p.core[t] = make_float4(tp.muav[t], mus, mus > 0.f ? (float)(1.0 / mus) : 0.f, tp.gv[t]);
    p.phase[t] = phase_const(tp, t);
  }
  p.flags = e.flags;
  p.fast_math = (e.flags & NMC_FLAG_PRECISE_MATH) ? 0 : 1;
  p.step_cap = 4000000u;
  p.per_fetch = fetch_run(e.photons_per_fetch);
  p.rng = rng_params(e, sim);
}

void fill_sub(SubParams& p, const nmc_run_params& rp, const nmc_tissue_params& tp, const nmc_ext& e) {
  const int L = 1;  // FIRST_TISSUE_LAYER_MCSUB, definitions.h:50
  p.mua = tp.muav[L];
  p.mus = tp.musv[L];
  p.mut = p.mua + p.mus;
  p.albedo = p.mus / p.mut;
  p.n1 = rp.n1;
  p.n2 = rp.n2;
  p.dr = e.sub_dr;
  p.dz = e.sub_dz;
  p.idr = (float)(1.0 / e.sub_dr);
  p.idz = (float)(1.0 / e.sub_dz);
  p.bins = e.sub_bins;
  p.mcflag = e.sub_mcflag;
  p.boundaryflag = e.sub_boundaryflag;
  p.radius = e.sub_radius;
  p.waist = e.sub_waist;
  p.zfocus = e.sub_zfocus;
  p.xs = e.sub_xs;
  p.ys = e.sub_ys;
  p.zs = e.sub_zs;
  p.phase = phase_const(tp, L);
  p.phase_kind = e.phase == NMC_PHASE_TWO_TERM      ? kPhaseTT
                 : e.phase == NMC_PHASE_ISOTROPIC_REF ? kPhaseIsoRef
                                                      : kPhaseHG;
  p.fast_math = (e.flags & NMC_FLAG_PRECISE_MATH) ? 0 : 1;
  p.skip_F = (e.flags & NMC_FLAG_SKIP_FLUENCE) ? 1 : 0;
  p.global_tallies = (e.flags & NMC_FLAG_GLOBAL_TALLIES) ? 1 : 0;
  p.rng = rng_params(e, NMC_SIM_MCSUB);
  p.step_cap = 10000000u;
  p.per_fetch = fetch_run(e.photons_per_fetch);
}

}  // namespace nmc
