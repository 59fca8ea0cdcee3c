// nmc_device.cuh - device building blocks shared by the transport kernels.
//
// Random streams, the optical helpers of the photon step (Fresnel, phase
// function samplers, SPIN), fixed-point tally arithmetic and the parameter
// blocks the kernels receive.  Physics follows NMC/NMCCode/helpers.metal and
// NMC/NMCCode/kernels.metal; line references are given per function.
#pragma once

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cstdint>
#include <type_traits>

#include "nmc_abi.h"

namespace nmc {

namespace cg = cooperative_groups;

// ------------------------------------------------------------ constants
// definitions.h:16-82
constexpr float kLS = 10E-8f;             // ls
constexpr float kPIref = 3.1415926f;      // PI as the reference defines it
constexpr float kTHRESHOLD = 0.0001f;
constexpr float kCHANCE = 0.1f;
constexpr float kMIN_VALUE = 1E-6f;
constexpr int kMAX_SCATT = 10000;
constexpr int kRAY_DEPTH = 100;
constexpr float kCOS90D = 1.0E-6f;
constexpr float kCOSZERO = 1.0F - 1.0E-6F;
constexpr float kRAD_DEG = (float)(180.0F / 3.1415926);
constexpr uint32_t kPhiloxTag = 0x4E4D4321u;

// Tallies are accumulated as unsigned 64-bit fixed point with 32 fractional
// bits: integer addition is associative, so every tally is bit-reproducible
// whatever the order in which threads deposit.
constexpr float kFix = 4294967296.0f;     // 2^32
constexpr double kUnfix = 1.0 / 4294967296.0;

__device__ __forceinline__ unsigned long long to_fix(float v) {
  // below 2^32 the 32-bit conversion gives the same integer and is cheaper
  const float t = v * kFix;
  if (!(v > 0.f)) return 0ull;
  return t < kFix ? (unsigned long long)__float2uint_rn(t) : __float2ull_rn(t);
}

// ----------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Round r (0-based)
// XORs the key words k0 + r W0 and k1 + r W1 into the state.  SeedKeys
// derives them round by round from the seed words; RoundKeys reads the ten
// pairs from a table the host filled (RngParams::rk), which a kernel keeps
// in its parameter block, so every round's XOR takes a constant operand
// instead of a key addition.  Both give the same numbers.
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

struct SeedKeys {
  uint32_t k0, k1;
  __device__ __forceinline__ uint32_t a(int r) const { return k0 + (uint32_t)r * kPhiloxW0; }
  __device__ __forceinline__ uint32_t b(int r) const { return k1 + (uint32_t)r * kPhiloxW1; }
};

struct RoundKeys {
  const uint32_t* rk;  // rk[2r] = k0 + r W0, rk[2r+1] = k1 + r W1
  __device__ __forceinline__ uint32_t a(int r) const { return rk[2 * r]; }
  __device__ __forceinline__ uint32_t b(int r) const { return rk[2 * r + 1]; }
};

template <class KEYS>
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, const KEYS& k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.a(r), lo1, hi0 ^ c.w ^ k.b(r), lo0);
  }
  return c;
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
  return philox4x32_10(c, SeedKeys{k0, k1});
}

// The round-key table of seed words (k0, k1), as RoundKeys reads it.
inline void philox_round_keys(uint32_t k0, uint32_t k1, uint32_t rk[20]) {
  for (int r = 0; r < 10; ++r) {
    rk[2 * r] = k0 + (uint32_t)r * kPhiloxW0;
    rk[2 * r + 1] = k1 + (uint32_t)r * kPhiloxW1;
  }
}

// 0 < u < 1, u = (2k+1) 2^-24 from the top 23 bits k of x (exact in float).
// Built without an int->float conversion: 1 + k 2^-23 is the float with
// mantissa k, and (1 + k 2^-23) - (1 - 2^-24) is exact (Sterbenz).
__device__ __forceinline__ float u01(uint32_t x) {
  return __uint_as_float((x >> 9) | 0x3F800000u) - 0.99999994039535522f;
}

// Per-photon Philox layout (identical in the oracle): key = (seed lo, seed
// hi); counter = (photon lo, photon hi, c2, 0x4E4D4321).  Hops are numbered
// h = 0, 1, ...; the SPIN that ends hop h-1 and the step of hop h come from
// one block, so a block is generated and consumed at a single point of the
// photon loop and no random state stays live across voxel sub-steps:
//   c2 = 0xFFFFFFFF        launch block, slots in draw order
//   c2 = h                 w = step of hop h; for h >= 1 x, y, z = SPIN draws
//                          of the event ending hop h-1: (cos, psi, roulette)
//                          or, two-term, (choice, sample, psi)
//   c2 = h | 0x40000000    aux block, made only when used: x = two-term
//                          roulette of that SPIN, y = Fresnel test of hop h
// The key words come from the kernel parameters (uniform across the grid).
struct SpinDraws {
  float a, b, c;  // HG: cos, psi, roulette; two-term: choice, sample, psi
  float roul;     // roulette draw (two-term); equal to c for HG
  float step;     // uniform for the step of the next hop
};

struct LaunchDraws {
  uint4 l;
  uint32_t n;
  __device__ __forceinline__ float next() {
    const uint32_t k = n++;
    return u01(k == 0 ? l.x : k == 1 ? l.y : k == 2 ? l.z : l.w);
  }
};

template <bool TT>
struct PhiloxRng {
  uint32_t plo, phi, hop;
  template <class KEYS>
  __device__ __forceinline__ uint4 block(uint32_t c2, const KEYS& k) const {
    return philox4x32_10(make_uint4(plo, phi, c2, kPhiloxTag), k);
  }
  __device__ __forceinline__ uint4 block(uint32_t c2, uint32_t k0, uint32_t k1) const {
    return block(c2, SeedKeys{k0, k1});
  }
  __device__ __forceinline__ void init(uint64_t photon) {
    plo = (uint32_t)photon;
    phi = (uint32_t)(photon >> 32);
    hop = 0;
  }
  template <class F>
  __device__ __forceinline__ void launch(uint32_t k0, uint32_t k1, F&& use) {
    LaunchDraws d{block(0xFFFFFFFFu, k0, k1), 0};
    use(d);
  }
  template <class KEYS>
  __device__ __forceinline__ float first_step(const KEYS& k) {
    hop = 0;
    return u01(block(0u, k).w);
  }
  __device__ __forceinline__ float first_step(uint32_t k0, uint32_t k1) { return first_step(SeedKeys{k0, k1}); }
  template <class KEYS>
  __device__ __forceinline__ SpinDraws spin_draws(bool need_roul, const KEYS& k) {
    ++hop;
    const uint4 b = block(hop, k);
    SpinDraws d;
    d.a = u01(b.x);
    d.b = u01(b.y);
    d.c = u01(b.z);
    d.step = u01(b.w);
    d.roul = d.c;
    if (TT && need_roul) d.roul = u01(block(hop | 0x40000000u, k).x);
    return d;
  }
  __device__ __forceinline__ SpinDraws spin_draws(bool need_roul, uint32_t k0, uint32_t k1) {
    return spin_draws(need_roul, SeedKeys{k0, k1});
  }
  template <class KEYS>
  __device__ __forceinline__ float fres_u(const KEYS& k) const {
    return u01(block(hop | 0x40000000u, k).y);
  }
  __device__ __forceinline__ float fres_u(uint32_t k0, uint32_t k1) const { return fres_u(SeedKeys{k0, k1}); }
};

// The reference's generator (helpers.metal:319-371), drawn sequentially in
// the reference's order.  Used to replay the reference's own photon streams.
struct TausRng {
  uint32_t s1, s2, s3, s4;
  __device__ __forceinline__ static uint32_t taus(uint32_t z, int a, int b, int c, uint32_t m) {
    const uint32_t bb = ((z << a) ^ z) >> b;
    return ((z & m) << c) ^ bb;
  }
  __device__ __forceinline__ static uint32_t xsh(uint32_t x) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
  }
  __device__ __forceinline__ void seed(uint32_t a, uint32_t b, uint32_t c) {
    a = xsh(a);
    b = xsh(b);
    c = xsh(c);
    s1 = taus(a, 13, 19, 12, 429496729u);
    s2 = taus(b, 2, 25, 4, 4294967288u);
    s3 = taus(c, 3, 11, 17, 429496280u);
    s4 = xsh(a + b + c) ^ 1013904223u;
    s1 ^= s4;
    s2 ^= s1;
    s3 ^= s2;
  }
  // Seeding per photon (run, index) as kernels.metal:91-95 / :339-343 / :772.
  __device__ __forceinline__ void init_photon(uint64_t photon, uint64_t batch, bool tt,
                                              bool tt_replay) {
    const uint32_t run = (uint32_t)(photon / batch) + 1u;
    const uint32_t index = (uint32_t)(photon % batch);
    if (tt) {
      const uint32_t nr = (tt_replay ? 0u : run) + 1u;
      seed(nr * index, nr * 1234u, index * 1234u);
    } else {
      const uint32_t nr = run + 1u;
      seed((nr ^ (index * 2654435761u)) + 12345u, (nr * 1103515245u) ^ (index * 1013904223u),
           (index ^ nr) * 1664525u + 1013904223u);
    }
  }
  __device__ __forceinline__ float next() {
    s1 = taus(s1, 13, 19, 12, 429496729u);
    s2 = taus(s2, 2, 25, 4, 4294967288u);
    s3 = taus(s3, 3, 11, 17, 429496280u);
    s4 = xsh(s4);
    return (float)((s1 ^ s2 ^ s3 ^ s4) >> 8) * (1.0f / 16777216.0f);
  }
  // The same interface as PhiloxRng, drawing in the reference's order:
  // launch draws, then per hop the step (with the `rnd <= 0` retry of
  // kernels.metal:183,501), the SPIN draws, the roulette draw when W is below
  // THRESHOLD (:289-290, :740-741).
  struct Seq {
    TausRng* g;
    __device__ __forceinline__ float next() { return g->next(); }
  };
  template <class F>
  __device__ __forceinline__ void launch(uint32_t, uint32_t, F&& use) {
    Seq s{this};
    use(s);
  }
  __device__ __forceinline__ float step_draw() {
    float r;
    while ((r = next()) <= 0.f) {
    }
    return r;
  }
  __device__ __forceinline__ float first_step(uint32_t, uint32_t) { return step_draw(); }
  template <class KEYS>
  __device__ __forceinline__ float first_step(const KEYS&) { return step_draw(); }
  template <bool TT>
  __device__ __forceinline__ SpinDraws spin_draws_t(bool need_roul) {
    SpinDraws d;
    d.a = next();
    d.b = next();
    if (TT) d.c = next();
    d.roul = need_roul ? next() : 1.f;
    if (!TT) d.c = d.roul;
    d.step = step_draw();
    return d;
  }
  __device__ __forceinline__ float fres_u(uint32_t, uint32_t) { return next(); }
  template <class KEYS>
  __device__ __forceinline__ float fres_u(const KEYS&) { return next(); }
};

// Uniform access to the two generators from the kernels.
template <bool TT, class RNG, class KEYS>
__device__ __forceinline__ SpinDraws spin_draws(RNG& rng, bool need_roul, const KEYS& k) {
  if constexpr (std::is_same<RNG, TausRng>::value)
    return rng.template spin_draws_t<TT>(need_roul);
  else
    return rng.spin_draws(need_roul, k);
}
template <bool TT, class RNG>
__device__ __forceinline__ SpinDraws spin_draws(RNG& rng, bool need_roul, uint32_t k0, uint32_t k1) {
  return spin_draws<TT>(rng, need_roul, SeedKeys{k0, k1});
}

// ---------------------------------------------------------------- optics
// FltEq (helpers.metal:21-25) with error = 1.
__device__ __forceinline__ bool flt_eq(float a, float b) {
  const float e = b * 1.1920928955078125e-7f * 2.f;
  return (a >= b - e) && (a <= b + e);
}

// Fresnel::RFresnel (helpers.metal:243-291): unpolarised reflectance from
// medium n1 into n2 at incidence cosine ca1; *ca2 = transmitted cosine.
__device__ __forceinline__ float rfresnel(float n1, float n2, float ca1, float* ca2) {
  if (flt_eq(n1, n2)) {
    *ca2 = ca1;
    return 0.f;
  }
  if (ca1 > kCOSZERO) {
    *ca2 = ca1;
    const float r = (n2 - n1) / (n2 + n1);
    return r * r;
  }
  if (ca1 < kCOS90D) {
    *ca2 = 0.f;
    return 1.f;
  }
  const float sa1 = sqrtf(fmaf(-ca1, ca1, 1.f));
  const float sa2 = n1 * sa1 / n2;
  if (sa2 >= 1.f) {
    *ca2 = 0.f;
    return 1.f;
  }
  const float c2 = sqrtf(fmaf(-sa2, sa2, 1.f));
  *ca2 = c2;
  const float cap = ca1 * c2 - sa1 * sa2, cam = ca1 * c2 + sa1 * sa2;
  const float sap = sa1 * c2 + ca1 * sa2, sam = sa1 * c2 - ca1 * sa2;
  return 0.5f * sam * sam * (cam * cam + cap * cap) / (sap * sap * cam * cam);
}

// Fresnel::Snell (helpers.metal:293-314).
__device__ __forceinline__ void snell(float n1, float n2, float& ux, float& uy, float& uz) {
  const float sc = 1.f - (1.f - uz * uz) * n1 * n1 / n2 / n2;
  if (sc < 0.f) {
    if (fabsf(uz) > 1.f) uz = uz < 0.f ? -1.f : 1.f;
    return;
  }
  ux = ux * n1 / n2;
  uy = uy * n1 / n2;
  uz = sqrtf(sc);
}

// Per-tissue phase-function constants, precomputed on the host in double.
// HG (kernels.metal:696-703): cos = (d - (a / (b + c u))^2) * e with
// a = 1-g^2, b = 1-g, c = 2g, d = 1+g^2, e = 1/(2g); mode 1 = isotropic
// (g == 0), mode 2 = straight ahead (g == 1).
// Two-term (kernels.metal:1060-1070): per branch q1/(2g), 1/q2, 1/q3,
// -1/alpha, 1/(2g); iso flag when g == 0.
struct __align__(16) PhaseConst {
  float hg_a, hg_b, hg_c, hg_d, hg_e;
  int hg_mode;
  float cc;
  float f_q1e, f_iq2, f_iq3, f_ninva, f_e;
  float b_q1e, b_iq2, b_iq3, b_ninva, b_e;
  int f_iso, b_iso;
};

// Arithmetic of the photon step in two accuracy grades.  PRECISE uses
// CUDA's correctly-rounded or 1-ulp library functions; FAST uses the SFU
// approximations (MUFU lg2/ex2/sin/cos/rcp, a few ulp).  The grade in use
// is the one whose per-photon agreement with the FP64 oracle meets the
// parity tests' bar.
template <bool FAST>
struct Math {
  static __device__ __forceinline__ float neglog(float u) { return FAST ? -__logf(u) : -logf(u); }
  // weight absorbed over optical depth x: W (1 - e^-x)
  static __device__ __forceinline__ float absorbed(float W, float x) {
    return FAST ? W - W * __expf(-x) : -W * expm1f(-x);
  }
  static __device__ __forceinline__ float rcp(float x) { return FAST ? __fdividef(1.f, x) : __frcp_rn(x); }
  static __device__ __forceinline__ float div(float a, float b) { return FAST ? __fdividef(a, b) : a / b; }
  static __device__ __forceinline__ void sincos2pi(float u, float* s, float* c) {
    if (FAST)
      __sincosf(6.2831853071795865f * u, s, c);
    else
      sincospif(2.f * u, s, c);
  }
  static __device__ __forceinline__ float pow(float x, float y) { return FAST ? __powf(x, y) : powf(x, y); }
  // sqrt of x >= 0
  static __device__ __forceinline__ float sqrt(float x) {
    return FAST ? x * rsqrtf(fmaxf(x, 1e-30f)) : sqrtf(x);
  }
};

// The general form is evaluated for every mode and the isotropic and
// straight-ahead modes select over it (for g = 0 it is NaN, 0 x inf), so a
// warp whose lanes sit in tissues of different modes takes no branch.
template <bool FAST>
__device__ __forceinline__ float hg_sample(const PhaseConst& p, float u) {
  const float t = Math<FAST>::div(p.hg_a, fmaf(p.hg_c, u, p.hg_b));
  const float c = fmaf(-t, t, p.hg_d) * p.hg_e;
  return p.hg_mode == 1 ? 2.f * u - 1.f : (p.hg_mode == 2 ? 1.f : c);
}

// Two-term sample from the branch choice and the sample uniform.
template <bool FAST>
__device__ __forceinline__ float tt_sample(const PhaseConst& p, float uc, float u) {
  float c;
  if (uc <= p.cc) {
    c = p.f_iso ? 2.f * u - 1.f
                : p.f_q1e - Math<FAST>::pow(fmaf(u, p.f_iq2, (1.f - u) * p.f_iq3), p.f_ninva) * p.f_e;
  } else {
    c = p.b_iso ? 2.f * u - 1.f
                : p.b_q1e - Math<FAST>::pow(fmaf(u, p.b_iq2, (1.f - u) * p.b_iq3), p.b_ninva) * p.b_e;
    c = -c;
  }
  if (c >= 1.f) c = 1.0f - 1e-9f;
  if (c <= -1.f) c = -(1.0f - 1e-9f);
  return c;
}

// SPIN (kernels.metal:253-279, :704-730): rotate (ux, uy, uz) by polar
// cos(theta) and azimuth psi = 2 pi u.  Near |uz| -> 1 the rotation and a
// renormalisation run in FP64 (1 - uz^2 loses all FP32 bits there).
template <bool FAST>
__device__ __forceinline__ void spin(float costheta, float upsi, float& ux, float& uy,
                                     float& uz) {
  const float sintheta = Math<FAST>::sqrt(fmaxf(fmaf(-costheta, costheta, 1.f), 0.f));
  float sinpsi, cospsi;
  Math<FAST>::sincos2pi(upsi, &sinpsi, &cospsi);
  const float auz = fabsf(uz);
  // one test on the common path; the two near-vertical cases behind it
  if (__builtin_expect(1.f - auz < 1e-5f, 0)) {
    if (auz >= 1.f) {  // 1 - |uz| <= 1e-12 in FP32
      ux = sintheta * cospsi;
      uy = sintheta * sinpsi;
      uz = uz >= 0.f ? costheta : -costheta;
    } else {
      const double dz = uz, temp = sqrt(1.0 - dz * dz);
      const double st = sintheta, ct = costheta, cp = cospsi, sp = sinpsi;
      double nx = st * (ux * dz * cp - uy * sp) / temp + ux * ct;
      double ny = st * (uy * dz * cp + ux * sp) / temp + uy * ct;
      double nz = -st * cp * temp + dz * ct;
      const double inv = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
      ux = (float)(nx * inv);
      uy = (float)(ny * inv);
      uz = (float)(nz * inv);
    }
  } else {
    const float temp2 = fmaf(-uz, uz, 1.f);
    const float itemp = rsqrtf(temp2);
    const float temp = temp2 * itemp;
    const float nx = fmaf(sintheta * (ux * uz * cospsi - uy * sinpsi), itemp, ux * costheta);
    const float ny = fmaf(sintheta * (uy * uz * cospsi + ux * sinpsi), itemp, uy * costheta);
    const float nz = fmaf(-sintheta * cospsi, temp, uz * costheta);
    ux = nx;
    uy = ny;
    uz = nz;
  }
}

// ----------------------------------------------------------- index checks
// The checked build (-DNMC_CHECK_BOUNDS, nmc_gb300/_build/checked/) tests
// every tally index against its buffer; an index out of range raises
// NMC_DEVFLAG_BOUNDS and the access is skipped.  compute-sanitizer is not
// available for these kernels, so this is the bounds checker; in the normal
// build the test compiles away.
#ifdef NMC_CHECK_BOUNDS
__device__ __forceinline__ bool idx_ok(unsigned long long i, unsigned long long n, unsigned int* flags) {
  if (i < n) return true;
  atomicOr(flags, (unsigned int)NMC_DEVFLAG_BOUNDS);
  return false;
}
#else
__device__ __forceinline__ bool idx_ok(unsigned long long, unsigned long long, unsigned int*) { return true; }
#endif

// ----------------------------------------------------------- work queue
// Hands out photon indices in warp-aggregated chunks: one atomic per group
// of threads that need a photon at the same time.
__device__ __forceinline__ unsigned long long next_photon(unsigned long long* counter) {
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (unsigned long long)g.size());
  base = g.shfl(base, 0);
  return base + g.thread_rank();
}

// The same with runs of `per` consecutive photons per thread (per a power of
// two): a run starts at a multiple of per, so the thread continues its run
// while the next index is not one; pidx = ~0 means no run yet.
__device__ __forceinline__ unsigned long long next_photon_run(unsigned long long* counter, unsigned int per,
                                                              unsigned long long pidx) {
  if (pidx != ~0ull && ((pidx + 1) & (per - 1)) != 0) return pidx + 1;
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (unsigned long long)g.size() * per);
  base = g.shfl(base, 0);
  return base + (unsigned long long)g.thread_rank() * per;
}

// Sums a per-thread value over the threads of the warp that are here
// together (any subset), then one atomic per group.
__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, unsigned long long v) {
  cg::coalesced_group g = cg::coalesced_threads();
  v = cg::reduce(g, v, cg::plus<unsigned long long>());
  if (g.thread_rank() == 0 && v) atomicAdd(dst, v);
}
__device__ __forceinline__ void warp_add_f64(double* dst, double v) {
  cg::coalesced_group g = cg::coalesced_threads();
  v = cg::reduce(g, v, cg::plus<double>());
  if (g.thread_rank() == 0 && v != 0.0) atomicAdd(dst, v);
}

// ------------------------------------------------------------ parameters
// Totals every launch adds into (device memory, one per handle).
struct DevSums {
  unsigned long long photons, substeps, scatters;
  unsigned long long S, A, E, rd;  // fixed point 2^-32, since the last fold
  double rd_sumsq;
  unsigned int flags, pad;
  unsigned long long work;         // photon counter of the running launch
  double carry[4];                 // S, A, E, rd moved out of the fixed-point words by folds
};

struct RngParams {
  uint32_t kind;  // NMC_RNG_*
  uint32_t k0, k1;
  uint32_t rk[20];  // Philox round keys of (k0, k1) (philox_round_keys)
  uint32_t tt_replay;
  uint64_t batch;  // photons_per_dispatch (Taus run/index mapping)
};

struct TraceParams {
  nmc_photon_record* recs;
  float4* events;
  uint32_t k_events;
};

}  // namespace nmc
