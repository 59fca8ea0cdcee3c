// nmc_oracle.cpp - CPU oracle for the photon-transport engine.
//
// TEST INFRASTRUCTURE ONLY: called by tests/, __graft_entry__.smoke() and the
// CPU baseline of bench.py, never by the product.
//
// A line-by-line restatement, in plain C++ templated on the arithmetic type
// (double for the parity oracle, float to study FP32 rounding) and on the
// random stream, of the reference's photon kernels:
//   MCSubKernel    NMC/NMCCode/kernels.metal:59-319
//   MCXYZKernel    NMC/NMCCode/kernels.metal:321-754
//   MCXYZKernelTT  NMC/NMCCode/kernels.metal:757-1118
// and of the helpers they call (NMC/NMCCode/helpers.metal): FltEq :21-25,
// SameVoxel :27-39, FindVoxelFace2 :85-114, Fresnel::RFresnel :243-291,
// Fresnel::Snell :293-314, RandomGen :319-371.  Constants are those of
// NMC/NMCCode/definitions.h.  Per-photon order of random draws is the
// reference's, so with the reference's own generator (NMC_RNG_TAUS_REF) a
// photon follows the reference's trajectory, and with Philox it follows the
// GPU engine's.
//
// Departures, each because the reference's behaviour is undefined there:
//  * the two-term sampler takes the isotropic branch when g_f or g_b is 0
//    (kernels.metal:1062,1066 divide by 2g);
//  * the two-term Rd2D index is clamped to the grid (kernels.metal:984 uses
//    unclamped indices);
//  * every photon has a step cap (NMC_FATE_STEPCAP) so that no input can
//    loop forever.
#include "nmc_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// Start of thread t's share when n photons are split over nt threads (the
// first n % nt threads take one photon more); overflow-free for any n.
uint64_t share_begin(uint64_t n, int t, int nt) {
  return n / (uint64_t)nt * (uint64_t)t + std::min<uint64_t>((uint64_t)t, n % (uint64_t)nt);
}

// ---------------------------------------------------------------- constants
constexpr double kPI = 3.1415926;               // definitions.h:60 PI
constexpr double kLS = 10E-8;                   // definitions.h:59 ls
constexpr double kTHRESHOLD = 0.0001;           // definitions.h:64
constexpr double kCHANCE = 0.1;                 // definitions.h:65
constexpr double kMIN_VALUE = 1E-6;             // definitions.h:66
constexpr int kMAX_SCATT = 10000;               // definitions.h:19
constexpr int kRAY_DEPTH = 100;                 // definitions.h:21
constexpr double kCOS90D = 1.0E-6;              // definitions.h:70
constexpr float kCOSZERO = 1.0F - 1.0E-6F;      // definitions.h:71
constexpr double kONE_MINUS_COSZERO = 1.0E-12;  // definitions.h:72
const double kRAD_DEG = 180.0F / kPI;           // definitions.h:77
constexpr int kMCSUB_LAYER = 1;                 // FIRST_TISSUE_LAYER_MCSUB
constexpr uint64_t kStepCap = 100000000ull;     // oracle-only safety cap
constexpr uint32_t kPhiloxTag = 0x4E4D4321u;    // counter word 3

// ------------------------------------------------------------------- RNGs
void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

// What a uniform is used for.  The reference draws sequentially from one
// stream; the Philox layout below gives every use a fixed slot instead.
enum Draw { D_LAUNCH, D_STEP, D_COS, D_PSI, D_ROUL, D_FRES, D_CHOICE, D_SAMPLE };

// Philox layout of the GPU engine (same definition as in the CUDA
// kernels): key = (seed lo, seed hi); counter = (photon lo, photon hi, c2,
// 0x4E4D4321).  Hops are numbered h = 0, 1, ...; the SPIN that ends hop h
// and the step of hop h+1 come from one block, so each block is consumed at
// one point of the photon loop:
//   c2 = 0xFFFFFFFF          launch block, slots used in draw order
//   c2 = h                   event block h: w = step of hop h; for h >= 1
//                            x, y, z are the draws of the SPIN ending hop h-1
//                              HG / isotropic: x = cos, y = psi, z = roulette
//                              two-term:       x = choice, y = sample, z = psi
//   c2 = h | 0x40000000      aux block h, generated only when used:
//                            x = roulette of the SPIN ending hop h-1 (two-term),
//                            y = Fresnel test during hop h (mcsub)
// u = (2k+1) 2^-24 with k the top 23 bits of the word: 0 < u < 1, exact in
// float and double, so the reference's `while (rnd <= 0)` loops never repeat.
struct PhiloxStream {
  uint32_t k0, k1, id_lo, id_hi;
  bool tt;
  uint32_t hop = 0xFFFFFFFFu, nlaunch = 0;
  uint32_t cb[4], nb[4], ab[4], nab[4], lb[4];
  bool c_ok = false, n_ok = false, a_ok = false, na_ok = false, l_ok = false;
  PhiloxStream(uint64_t seed, uint64_t photon, bool two_term)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), id_lo((uint32_t)photon),
        id_hi((uint32_t)(photon >> 32)), tt(two_term) {}
  void gen(uint32_t c2, uint32_t* out) {
    uint32_t c[4] = {id_lo, id_hi, c2, kPhiloxTag};
    philox10(c, k0, k1);
    std::memcpy(out, c, sizeof c);
  }
  void new_hop() {
    ++hop;
    // the "next" blocks of the previous hop are this hop's current ones
    if (n_ok) std::memcpy(cb, nb, sizeof cb);
    c_ok = n_ok;
    if (na_ok) std::memcpy(ab, nab, sizeof ab);
    a_ok = na_ok;
    n_ok = na_ok = false;
  }
  uint32_t cur(int k) {
    if (!c_ok) {
      gen(hop, cb);
      c_ok = true;
    }
    return cb[k];
  }
  uint32_t next(int k) {
    if (!n_ok) {
      gen(hop + 1, nb);
      n_ok = true;
    }
    return nb[k];
  }
  uint32_t aux_cur(int k) {
    if (!a_ok) {
      gen(hop | 0x40000000u, ab);
      a_ok = true;
    }
    return ab[k];
  }
  uint32_t aux_next(int k) {
    if (!na_ok) {
      gen((hop + 1) | 0x40000000u, nab);
      na_ok = true;
    }
    return nab[k];
  }
  uint32_t word(Draw d) {
    switch (d) {
      case D_LAUNCH:
        if (!l_ok) {
          gen(0xFFFFFFFFu, lb);
          l_ok = true;
        }
        return lb[(nlaunch++) & 3];
      case D_STEP: return cur(3);
      case D_COS: return next(0);
      case D_CHOICE: return next(0);
      case D_SAMPLE: return next(1);
      case D_PSI: return tt ? next(2) : next(1);
      case D_ROUL: return tt ? aux_next(0) : next(2);
      case D_FRES: return aux_cur(1);
    }
    return 0;
  }
  template <class R>
  R u(Draw d) {
    const uint32_t x = word(d);
    return R(x >> 9) * R(1.0 / 8388608.0) + R(1.0 / 16777216.0);
  }
};

// RandomGen, helpers.metal:319-371.
struct TausStream {
  uint32_t s1, s2, s3, s4;
  static uint32_t taus(uint32_t z, int a, int b, int c, uint32_t m) {
    const uint32_t bb = ((z << a) ^ z) >> b;
    return ((z & m) << c) ^ bb;
  }
  static uint32_t xsh(uint32_t x) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
  }
  TausStream(uint32_t a, uint32_t b, uint32_t c) {
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
  float next_f() {
    s1 = taus(s1, 13, 19, 12, 429496729u);
    s2 = taus(s2, 2, 25, 4, 4294967288u);
    s3 = taus(s3, 3, 11, 17, 429496280u);
    s4 = xsh(s4);
    const uint32_t r = s1 ^ s2 ^ s3 ^ s4;
    return (float)(r >> 8) * (1.0f / 16777216.0f);
  }
  void new_hop() {}
  template <class R>
  R u(Draw) {
    return R(next_f());
  }
};

// Seeds of the reference's generator for photon (run, index):
// kernels.metal:91-95 (mcsub) and :339-343 (mcxyz) use numRuns = run + 1;
// :772 (two-term) uses (numRuns*index, numRuns*1234, index*1234).
TausStream taus_for(int sim_type, uint64_t photon, uint64_t batch, bool tt_replay) {
  const uint32_t run = (uint32_t)(photon / batch) + 1u;  // main.m:159 iRunNum
  const uint32_t index = (uint32_t)(photon % batch);
  if (sim_type == NMC_SIM_MCXYZ_TT) {
    const uint32_t nr = (tt_replay ? 0u : run) + 1u;
    return TausStream(nr * index, nr * 1234u, index * 1234u);
  }
  const uint32_t nr = run + 1u;
  return TausStream((nr ^ (index * 2654435761u)) + 12345u,
                    (nr * 1103515245u) ^ (index * 1013904223u),
                    (index ^ nr) * 1664525u + 1013904223u);
}

// ----------------------------------------------------------------- helpers
template <class R>
bool flt_eq(R a, R b) {  // helpers.metal:21-25 with error = 1
  const R e = b * R(FLT_EPSILON) * R(2);
  return (a >= b - e) && (a <= b + e);
}

template <class R>
R rfresnel(R n1, R n2, R ca1, R* ca2) {  // helpers.metal:243-291
  R r = 0;
  if (flt_eq(n1, n2)) {
    *ca2 = ca1;
    r = 0;
  } else if (ca1 > R(kCOSZERO)) {
    *ca2 = ca1;
    r = (n2 - n1) / (n2 + n1);
    r *= r;
  } else if (ca1 < R(kCOS90D)) {
    *ca2 = 0;
    r = 1;
  } else {
    const R sa1 = std::sqrt(R(1) - ca1 * ca1);
    const R sa2 = n1 * sa1 / n2;
    if (sa2 >= R(1)) {
      *ca2 = 0;
      r = 1;
    } else {
      const R c2 = std::sqrt(R(1) - sa2 * sa2);
      *ca2 = c2;
      const R cap = ca1 * c2 - sa1 * sa2, cam = ca1 * c2 + sa1 * sa2;
      const R sap = sa1 * c2 + ca1 * sa2, sam = sa1 * c2 - ca1 * sa2;
      r = R(0.5) * sam * sam * (cam * cam + cap * cap) / (sap * sap * cam * cam);
    }
  }
  return r;
}

template <class R>
void snell(R n1, R n2, R* ux, R* uy, R* uz) {  // helpers.metal:293-314
  const R x = *ux, y = *uy, z = *uz;
  const R sc = R(1) - (R(1) - z * z) * n1 * n1 / n2 / n2;
  if (sc < R(0)) {
    if (std::fabs(z) > R(1)) *uz = z < R(0) ? R(-1) : R(1);
    return;
  }
  *ux = x * n1 / n2;
  *uy = y * n1 / n2;
  *uz = std::sqrt(sc);
}

template <class R>
bool same_voxel(R x1, R y1, R z1, R x2, R y2, R z2, R dx, R dy, R dz) {  // :27-39
  const R xmin = std::min(std::floor(x1 / dx), std::floor(x2 / dx)) * dx;
  const R ymin = std::min(std::floor(y1 / dy), std::floor(y2 / dy)) * dy;
  const R zmin = std::min(std::floor(z1 / dz), std::floor(z2 / dz)) * dz;
  const R xmax = xmin + dx, ymax = ymin + dy, zmax = zmin + dz;
  return x1 <= xmax && x2 <= xmax && y1 <= ymax && y2 <= ymax && z1 < zmax && z2 <= zmax;
}

template <class R>
R find_voxel_face2(R x1, R y1, R z1, R dx, R dy, R dz, R ux, R uy, R uz) {  // :85-114
  const int ix1 = (int)std::floor(x1 / dx), iy1 = (int)std::floor(y1 / dy),
            iz1 = (int)std::floor(z1 / dz);
  const int ix2 = ux >= R(0) ? ix1 + 1 : ix1;
  const int iy2 = uy >= R(0) ? iy1 + 1 : iy1;
  const int iz2 = uz >= R(0) ? iz1 + 1 : iz1;
  const R xs = std::fabs((R(ix2) * dx - x1) / ux);
  const R ys = std::fabs((R(iy2) * dy - y1) / uy);
  const R zs = std::fabs((R(iz2) * dz - z1) / uz);
  return std::min(std::min(xs, ys), zs);
}

// Henyey-Greenstein sample (kernels.metal:244-251, :696-703).
template <class R>
R hg_costheta(R g, R rnd) {
  if (flt_eq(g, R(0))) return R(2) * rnd - R(1);
  if (flt_eq(g, R(1))) return R(1);
  const R temp = (R(1) - g * g) / (R(1) - g + R(2) * g * rnd);
  return (R(1) + g * g - temp * temp) / (R(2) * g);
}

// Two-term parameters q1 = 1+g^2, q2 = (1-g)^(2a), q3 = (1+g)^(2a)
// (kernels.metal:900-905).
template <class R>
struct TTq {
  R q1f, q2f, q3f, q1b, q2b, q3b;
  void set(R gf, R af, R gb, R ab) {
    q1f = R(1) + gf * gf;
    q2f = std::pow(R(1) - gf, R(2) * af);
    q3f = std::pow(R(1) + gf, R(2) * af);
    q1b = R(1) + gb * gb;
    q2b = std::pow(R(1) - gb, R(2) * ab);
    q3b = std::pow(R(1) + gb, R(2) * ab);
  }
};

// One two-term cos(theta) from two draws (kernels.metal:1058-1070).
template <class R, class G>
R tt_costheta(G& rng, const TTq<R>& q, R gf, R af, R gb, R ab, R cc) {
  R rnd = rng.template u<R>(D_CHOICE);
  R c;
  if (rnd <= cc) {
    rnd = rng.template u<R>(D_SAMPLE);
    if (gf == R(0))
      c = R(2) * rnd - R(1);
    else
      c = (q.q1f / (R(2) * gf)) -
          std::pow(rnd / q.q2f + (R(1) - rnd) / q.q3f, -R(1) / af) / (R(2) * gf);
  } else {
    rnd = rng.template u<R>(D_SAMPLE);
    if (gb == R(0))
      c = R(2) * rnd - R(1);
    else
      c = (q.q1b / (R(2) * gb)) -
          std::pow(rnd / q.q2b + (R(1) - rnd) / q.q3b, -R(1) / ab) / (R(2) * gb);
    c *= R(-1);
  }
  if (c >= R(1)) c = R(1.0 - 1e-9);
  if (c <= R(-1)) c = -R(1.0 - 1e-9);
  return c;
}

// psi sample and the new direction (kernels.metal:255-279, :706-730).
template <class R>
void spin_u(R costheta, R u_psi, R& ux, R& uy, R& uz) {
  const R sintheta = std::sqrt(R(1) - costheta * costheta);
  const R psi = R(2.0 * kPI) * u_psi;
  const R cospsi = std::cos(psi);
  const R sinpsi = psi < R(kPI) ? std::sqrt(R(1) - cospsi * cospsi)
                                : -std::sqrt(R(1) - cospsi * cospsi);
  R uxx, uyy, uzz;
  if (R(1) - std::fabs(uz) <= R(kONE_MINUS_COSZERO)) {
    uxx = sintheta * cospsi;
    uyy = sintheta * sinpsi;
    uzz = costheta * (uz >= R(0) ? R(1) : R(-1));
  } else {
    const R temp = std::sqrt(R(1) - uz * uz);
    uxx = sintheta * (ux * uz * cospsi - uy * sinpsi) / temp + ux * costheta;
    uyy = sintheta * (uy * uz * cospsi + ux * sinpsi) / temp + uy * costheta;
    uzz = -sintheta * cospsi * temp + uz * costheta;
  }
  ux = uxx;
  uy = uyy;
  uz = uzz;
}

template <class R, class G>
void spin(G& rng, R costheta, R& ux, R& uy, R& uz) {
  spin_u<R>(costheta, rng.template u<R>(D_PSI), ux, uy, uz);
}

// Replays a fixed list of uniforms (used by the sampler entry points).
struct FixedDraws {
  double v[2];
  int k = 0;
  template <class R>
  R u(Draw) {
    return R(v[k++]);
  }
};

// ------------------------------------------------------------ run context
struct Cfg {
  int sim;
  nmc_run_params rp;
  nmc_tissue_params tp;
  const uint8_t* v;
  nmc_ext ext;
};

struct Tally {
  std::vector<double> J, F, F3D, Rd2D, Det, slots;
  double S = 0, A = 0, E = 0, rd = 0, rd2 = 0, ph = 0, sub = 0, sc = 0;
};

struct Trace {
  nmc_photon_record* rec;
  float* ev;
  uint32_t k;
  uint32_t nev = 0;
  void event(double x, double y, double z, double w) {
    if (!ev || nev >= k) return;
    float* e = ev + 4 * (size_t)nev;
    e[0] = (float)x;
    e[1] = (float)y;
    e[2] = (float)z;
    e[3] = (float)w;
    ++nev;
  }
};

// ---------------------------------------------------------------- MCSub
template <class R, class G>
void mcsub_photon(const Cfg& c, G& rng, Tally& T, Trace& tr) {
  const nmc_ext& e = c.ext;
  const R mua = c.tp.muav[kMCSUB_LAYER], mus = c.tp.musv[kMCSUB_LAYER];
  const R g = c.tp.gv[kMCSUB_LAYER];
  const R n1 = c.rp.n1, n2 = c.rp.n2;
  const int BINS = e.sub_bins;
  const R dr = e.sub_dr, dz = e.sub_dz, zs = e.sub_zs;
  TTq<R> q;
  const R gf = c.tp.gf[kMCSUB_LAYER], af = c.tp.af[kMCSUB_LAYER];
  const R gb = c.tp.gb[kMCSUB_LAYER], ab = c.tp.ab[kMCSUB_LAYER];
  const R cc = c.tp.CC[kMCSUB_LAYER];
  if (e.phase == NMC_PHASE_TWO_TERM) q.set(gf, af, gb, ab);

  R px = 0, py = 0, pz = 0, ux = 0, uy = 0, uz = 0;
  const R mut = mua + mus, albedo = mus / mut;  // :100-101
  R Rsptot = 0, Atot = 0, rsp = 0, E = 0, W = 0, rnd, temp;
  uint32_t nsub = 0, nsc = 0, fate = NMC_FATE_ALIVE, ndet = 0;

  if (e.sub_mcflag == 0) {  // :106-121
    rnd = rng.template u<R>(D_LAUNCH);
    px = R(e.sub_radius) * std::sqrt(rnd);
    py = 0;
    pz = zs;
    ux = 0;
    uy = 0;
    uz = 1;
    temp = n1 / n2;
    temp = (R(1) - temp) / (R(1) + temp);
    rsp = temp * temp;
  } else if (e.sub_mcflag == 1) {  // :122-147
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    px = R(e.sub_radius) * std::sqrt(-std::log(rnd));
    py = 0;
    pz = zs;
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    const R xfocus = R(e.sub_waist) * std::sqrt(-std::log(rnd));
    const R zf = e.sub_zfocus;
    temp = std::sqrt((px - xfocus) * (px - xfocus) + zf * zf);
    const R sintheta = -(px - xfocus) / temp, costheta = zf / temp;
    ux = sintheta;
    uy = 0;
    uz = costheta;
    R uzn = uz;
    rsp = rfresnel(n2, n1, costheta, &uzn);
    uz = uzn;
    ux = std::sqrt(R(1) - uz * uz);
  } else if (e.sub_mcflag == 2) {  // :148-164
    px = e.sub_xs;
    py = e.sub_ys;
    pz = zs;
    const R costheta = R(1) - R(2) * rng.template u<R>(D_LAUNCH);
    const R sintheta = std::sqrt(R(1) - costheta * costheta);
    const R psi = R(2.0 * kPI) * rng.template u<R>(D_LAUNCH);
    const R cospsi = std::cos(psi);
    const R sinpsi = psi < R(kPI) ? std::sqrt(R(1) - cospsi * cospsi)
                                  : -std::sqrt(R(1) - cospsi * cospsi);
    ux = sintheta * cospsi;
    uy = sintheta * sinpsi;
    uz = costheta;
    rsp = 0;
  }
  W = R(1) - rsp;  // :166-168
  Rsptot += rsp;
  bool alive = true;

  do {  // :176-305
    rng.new_hop();
    while ((rnd = rng.template u<R>(D_STEP)) <= R(0)) {
    }
    R s = -std::log(rnd) / mut;
    px += s * ux;
    py += s * uy;
    pz += s * uz;
    ++nsub;
    if (e.sub_boundaryflag == 1 && pz <= zs) {  // :190-214
      rnd = rng.template u<R>(D_FRES);
      R uz1;
      if (rnd > rfresnel(n1, n2, -uz, &uz1)) {
        px -= s * ux;
        py -= s * uy;
        pz -= s * uz;
        s = std::fabs(pz / uz);
        px += s * ux;
        py += s * uy;
        const R r = std::sqrt(px * px + py * py);
        long ir = (long)(r / dr) + 1;
        if (ir > BINS) ir = BINS;
        if (!T.J.empty()) T.J[ir] += (double)W;
        E += W;
        ndet = 1;
        alive = false;
        fate = NMC_FATE_ESCAPED;
      } else {
        pz = -pz;
        uz = -uz;
      }
    }
    if (alive) {
      const R absorb = W * (R(1) - albedo);  // :224-234
      W -= absorb;
      Atot += absorb;
      const R r = std::sqrt(px * px + py * py);
      long ir = (long)(r / dr) + 1;
      long iz = (long)(std::fabs(pz) / dz) + 1;
      if (ir >= BINS) ir = BINS;
      if (iz >= BINS) iz = BINS;
      if (!T.F.empty()) T.F[ir * BINS + iz] += (double)absorb;

      R costheta;  // :243-252
      if (e.phase == NMC_PHASE_TWO_TERM) {
        costheta = tt_costheta(rng, q, gf, af, gb, ab, cc);
      } else {
        rnd = rng.template u<R>(D_COS);
        costheta = hg_costheta(g, rnd);
        if (e.phase == NMC_PHASE_ISOTROPIC_REF) costheta = R(2) * rnd - R(1);
      }
      spin(rng, costheta, ux, uy, uz);
      ++nsc;
      if (W < R(kTHRESHOLD)) {  // :289-294
        rnd = rng.template u<R>(D_ROUL);
        if (rnd <= R(kCHANCE))
          W /= R(kCHANCE);
        else {
          alive = false;
          fate = NMC_FATE_ROULETTE;
        }
      }
      tr.event(px, py, pz, W);
    }
    if (alive && nsub >= kStepCap) {
      alive = false;
      fate = NMC_FATE_STEPCAP;
    }
  } while (alive);

  T.S += (double)Rsptot;
  T.A += (double)Atot;
  T.E += (double)E;
  T.rd += (double)E;
  T.rd2 += (double)E * (double)E;
  T.sub += nsub;
  T.sc += nsc;
  if (tr.rec) {
    nmc_photon_record& o = *tr.rec;
    o.n_scatt = nsc;
    o.n_sub = nsub;
    o.fate = fate;
    o.n_detect = ndet;
    o.w_final = (float)W;
    o.absorbed = (float)Atot;
    o.detected = (float)E;
    o.x = (float)px;
    o.y = (float)py;
    o.z = (float)pz;
  }
}

// -------------------------------------------------------------- MCXYZ(TT)
template <class R>
struct Voxel {
  int Nx, Ny, Nz;
  R dx, dy, dz;
};

// launch (kernels.metal:366-463; the two-term kernel :796-870 lacks mcflag 1)
template <class R, class G>
void xyz_launch(const nmc_run_params& rp, bool tt, G& rng, R& x, R& y, R& z, R& ux, R& uy,
                R& uz, R& W) {
  R rnd;
  x = y = z = ux = uy = uz = 0;  // tagPhoton() zero initialisation, :30-39
  if (rp.launchflag == 1) {
    x = rp.xs;
    y = rp.ys;
    z = rp.zs;
    ux = rp.ux0;
    uy = rp.uy0;
    uz = rp.uz0;
    return;
  }
  if (rp.mcflag == 0 || (rp.mcflag == 1 && !tt)) {
    const bool gauss = rp.mcflag == 1;
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    R r = gauss ? R(rp.radius) * std::sqrt(-std::log(rnd)) : R(rp.radius) * std::sqrt(rnd);
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    R phi = rnd * R(2.0) * R(kPI);
    x = R(rp.xs) + r * std::cos(phi);
    y = R(rp.ys) + r * std::sin(phi);
    z = rp.zs;
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    r = R(rp.waist) * std::sqrt(rnd);
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    phi = rnd * R(2.0) * R(kPI);
    const R xfocus = r * std::cos(phi), yfocus = r * std::sin(phi);
    const R zf = rp.zfocus;
    const R temp = std::sqrt((x - xfocus) * (x - xfocus) + (y - yfocus) * (y - yfocus) + zf * zf);
    ux = -(x - xfocus) / temp;
    uy = -(y - yfocus) / temp;
    uz = std::sqrt(R(1) - ux * ux - uy * uy);
    if (gauss) {  // :423-427
      R uz_new = uz;
      const R int_rsp = rfresnel(R(rp.n2), R(rp.n1), std::fabs(uz), &uz_new);
      W = W * (R(1) - int_rsp);
      snell(R(rp.n2), R(rp.n1), &ux, &uy, &uz);
    }
  } else if (rp.mcflag == 2) {
    const R costheta = R(1) - R(2) * rng.template u<R>(D_LAUNCH);
    const R sintheta = std::sqrt(R(1) - costheta * costheta);
    const R psi = R(2.0 * kPI) * rng.template u<R>(D_LAUNCH);
    const R cospsi = std::cos(psi);
    const R sinpsi = psi < R(kPI) ? std::sqrt(R(1) - cospsi * cospsi)
                                  : -std::sqrt(R(1) - cospsi * cospsi);
    x = rp.xs;
    y = rp.ys;
    z = rp.zs;
    ux = sintheta * cospsi;
    uy = sintheta * sinpsi;
    uz = costheta;
  } else if (rp.mcflag == 3) {
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    x = R(rp.radius) * (rnd * R(2.0) - R(1.0));
    while ((rnd = rng.template u<R>(D_LAUNCH)) <= R(0)) {
    }
    y = R(rp.radius) * (rnd * R(2.0) - R(1.0));
    z = rp.zs;
    ux = 0;
    uy = 0;
    uz = 1;
  } else if (rp.mcflag == 4) {
    x = 0;
    y = 0;
    z = rp.zs;
    ux = 0;
    uy = 0;
    uz = 1;
  }
}

template <class R, class G>
void mcxyz_photon(const Cfg& c, bool tt, G& rng, Tally& T, Trace& tr, uint64_t slot) {
  const nmc_run_params& rp = c.rp;
  const nmc_tissue_params& tp = c.tp;
  const int Nx = rp.Nx, Ny = rp.Ny, Nz = rp.Nz;
  const R dx = rp.dx, dy = rp.dy, dz = rp.dz, zsurf = rp.zsurf;
  const bool hard_kill = !(c.ext.flags & NMC_FLAG_NO_HARD_KILL);
  R x, y, z, ux, uy, uz, W = 1;
  xyz_launch(rp, tt, rng, x, y, z, ux, uy, uz, W);
  // launch voxel (kernels.metal:472-487): integer Nx/2 here, Nx/2.0 later
  int ix = (int)(Nx / 2 + x / dx);
  int iy = (int)(Ny / 2 + y / dy);
  int iz = (int)(z / dz);
  if (ix >= Nx) ix = Nx - 1;
  if (iy >= Ny) iy = Ny - 1;
  if (iz >= Nz) iz = Nz - 1;
  if (ix < 0) ix = 0;
  if (iy < 0) iy = 0;
  if (iz < 0) iz = 0;
  long i = (long)iz * Ny * Nx + (long)ix * Ny + iy;
  int tiss = c.v[i];
  R mua = tp.muav[tiss], mus = tp.musv[tiss], g = tp.gv[tiss];
  TTq<R> q;
  if (tt) q.set(R(tp.gf[tiss]), R(tp.af[tiss]), R(tp.gb[tiss]), R(tp.ab[tiss]));
  int bflag = 1, surfflag = 1;
  bool alive = true;
  R Rd_loc = 0, Atot = 0, rnd;
  uint32_t nsub = 0, nsc = 0, fate = NMC_FATE_ALIVE, ndet = 0;
  auto kill = [&](uint32_t why) {
    if (alive) fate = why;
    alive = false;
  };

  do {  // :493-750
    rng.new_hop();
    while ((rnd = rng.template u<R>(D_STEP)) <= R(0)) {
    }
    R sleft = -std::log(rnd);
    int depth = 0;
    do {  // :505-685
      R s = sleft / mus;
      const R tx = x + s * ux, ty = y + s * uy, tz = z + s * uz;
      ++nsub;
      if (same_voxel(x, y, z, tx, ty, tz, dx, dy, dz)) {
        x = tx;
        y = ty;
        z = tz;
        const R absorb = W * (R(1) - std::exp(-mua * s));
        W -= absorb;
        Atot += absorb;
        if (bflag && !T.F3D.empty()) T.F3D[i] += (double)absorb;
        sleft = 0;
      } else {
        s = R(kLS) + find_voxel_face2(x, y, z, dx, dy, dz, ux, uy, uz);
        const R absorb = W * (R(1) - std::exp(-mua * s));
        W -= absorb;
        Atot += absorb;
        if (bflag && !T.F3D.empty()) T.F3D[i] += (double)absorb;
        sleft -= s * mus;
        if (sleft <= R(kLS)) sleft = 0;
        if (!tt) {
          // surface detection (kernels.metal:560-637)
          const R z_new = z + s * uz;
          bool cross = false;
          if (rp.det_state == NMC_DET_REFLECTANCE && z_new <= zsurf && uz < R(0))
            cross = true;
          else if (rp.det_state == NMC_DET_TRANSMITTANCE && z_new >= zsurf && uz > R(0))
            cross = true;
          if (cross) {
            const R dl_b = (zsurf - z) / uz;
            sleft = (s - dl_b) * mus;
            if (sleft <= R(kLS)) sleft = 0;
            s = dl_b;
            x += s * ux;
            y += s * uy;
            z += s * uz;
            R uz_temp = 0;
            const R rsp = rfresnel(R(rp.n1), R(rp.n2), std::fabs(uz), &uz_temp);
            if (rsp < R(1)) {
              R th_exit = 0;
              if (!flt_eq(uz_temp, R(1))) th_exit = R(kRAD_DEG) * std::acos(uz_temp);
              const R ro = std::sqrt(x * x + y * y);
              R r_min, r_max;
              if (flt_eq(R(rp.xd), R(0))) {
                r_min = 0;
                r_max = rp.det_radius;
              } else {
                r_min = R(rp.xd) - R(rp.det_radius);
                r_max = r_min + R(2) * R(rp.det_radius);
              }
              if (ro >= r_min && ro <= r_max && th_exit <= R(rp.na)) {
                int jx = (int)(Nx / 2.0 + x / dx), jy = (int)(Ny / 2.0 + y / dy);
                if (jx >= Nx) jx = Nx - 1;
                if (jy >= Ny) jy = Ny - 1;
                if (jx < 0) jx = 0;
                if (jy < 0) jy = 0;
                const R dw = W * (R(1) - rsp);
                Rd_loc += dw;
                const long i2d = (long)jx * Ny + jy;
                if (!T.Rd2D.empty()) T.Rd2D[i2d] += (double)dw;
                if (!T.Det.empty()) T.Det[i2d] += 1.0;
                ++ndet;
                uz = -uz;
                W = W * rsp;
              }
            } else {
              uz = -uz;
              W = W * rsp;
            }
          } else {
            x += s * ux;
            y += s * uy;
            z += s * uz;
          }
          ix = (int)(Nx / 2.0 + x / dx);
          iy = (int)(Ny / 2.0 + y / dy);
          iz = (int)(z / dz);
        } else {
          // two-term kernel: move, first crossing above zsurf counts as Rd
          // (kernels.metal:972-993)
          x += s * ux;
          y += s * uy;
          z += s * uz;
          ix = (int)(Nx / 2.0 + x / dx);
          iy = (int)(Ny / 2.0 + y / dy);
          iz = (int)(z / dz);
          if (z < zsurf && surfflag == 1) {
            surfflag = 0;
            Rd_loc += W;
            ++ndet;
            const int jx = std::min(std::max(ix, 0), Nx - 1);
            const int jy = std::min(std::max(iy, 0), Ny - 1);
            if (!T.Rd2D.empty()) T.Rd2D[(long)jx * Ny + jy] += (double)W;
          }
          if (z < R(0)) {
            kill(NMC_FATE_BOUNDARY);
            sleft = 0;
          }
          bflag = 1;
        }
        if (rp.boundaryflag == 0) {  // :646-672
          if (iz >= Nz) { iz = Nz - 1; bflag = 0; }
          if (ix >= Nx) { ix = Nx - 1; bflag = 0; }
          if (iy >= Ny) { iy = Ny - 1; bflag = 0; }
          if (iz < 0) { iz = 0; bflag = 0; }
          if (ix < 0) { ix = 0; bflag = 0; }
          if (iy < 0) { iy = 0; bflag = 0; }
        } else if (rp.boundaryflag == 1) {
          if (iz >= Nz) { iz = Nz - 1; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (ix >= Nx) { ix = Nx - 1; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (iy >= Ny) { iy = Ny - 1; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (iz < 0) { iz = 0; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (ix < 0) { ix = 0; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (iy < 0) { iy = 0; kill(NMC_FATE_BOUNDARY); sleft = 0; }
        } else if (rp.boundaryflag == 2) {
          if (iz >= Nz) { iz = Nz - 1; bflag = 0; }
          if (ix >= Nx) { ix = Nx - 1; bflag = 0; }
          if (iy >= Ny) { iy = Ny - 1; bflag = 0; }
          if (iz < 0) { iz = 0; kill(NMC_FATE_BOUNDARY); sleft = 0; }
          if (ix < 0) { ix = 0; bflag = 0; }
          if (iy < 0) { iy = 0; bflag = 0; }
        }
        i = (long)iz * Ny * Nx + (long)ix * Ny + iy;  // :675-679
        tiss = c.v[i];
        mua = tp.muav[tiss];
        mus = tp.musv[tiss];
        g = tp.gv[tiss];
        if (tt) q.set(R(tp.gf[tiss]), R(tp.af[tiss]), R(tp.gb[tiss]), R(tp.ab[tiss]));
      }
      ++depth;
      if (nsub >= kStepCap) {
        kill(NMC_FATE_STEPCAP);
        break;
      }
    } while (depth <= kRAY_DEPTH && sleft > R(0));
    if (fate == NMC_FATE_STEPCAP) break;

    R costheta;  // SPIN, :695-731 / :1053-1071
    if (tt) {
      costheta = tt_costheta(rng, q, R(tp.gf[tiss]), R(tp.af[tiss]), R(tp.gb[tiss]),
                             R(tp.ab[tiss]), R(tp.CC[tiss]));
    } else {
      rnd = rng.template u<R>(D_COS);
      costheta = hg_costheta(g, rnd);
    }
    spin(rng, costheta, ux, uy, uz);
    ++nsc;
    if (W < R(kTHRESHOLD)) {  // :740-744
      if (rng.template u<R>(D_ROUL) <= R(kCHANCE))
        W /= R(kCHANCE);
      else
        kill(NMC_FATE_ROULETTE);
    }
    if (hard_kill && (W < R(kMIN_VALUE) || (int)nsc > kMAX_SCATT))  // :747-748
      kill(W < R(kMIN_VALUE) ? NMC_FATE_MINWEIGHT : NMC_FATE_MAXSCATT);
    tr.event(x, y, z, W);
  } while (alive);

  if (!T.slots.empty()) T.slots[slot] += (double)Rd_loc;  // :753
  T.A += (double)Atot;
  T.rd += (double)Rd_loc;
  T.rd2 += (double)Rd_loc * (double)Rd_loc;
  T.sub += nsub;
  T.sc += nsc;
  if (tr.rec) {
    nmc_photon_record& o = *tr.rec;
    o.n_scatt = nsc;
    o.n_sub = nsub;
    o.fate = fate;
    o.n_detect = ndet;
    o.w_final = (float)W;
    o.absorbed = (float)Atot;
    o.detected = (float)Rd_loc;
    o.x = (float)x;
    o.y = (float)y;
    o.z = (float)z;
  }
}

template <class R, class G>
void run_photon(const Cfg& c, G& rng, Tally& T, Trace& tr, uint64_t photon) {
  if (c.sim == NMC_SIM_MCSUB)
    mcsub_photon<R>(c, rng, T, tr);
  else
    mcxyz_photon<R>(c, c.sim == NMC_SIM_MCXYZ_TT, rng, T, tr,
                    photon % c.ext.photons_per_dispatch);
}

bool two_term_family(const Cfg& c) {
  return c.sim == NMC_SIM_MCXYZ_TT || (c.sim == NMC_SIM_MCSUB && c.ext.phase == NMC_PHASE_TWO_TERM);
}

template <class R>
void run_range(const Cfg& c, uint64_t first, uint64_t lo, uint64_t hi, Tally& T,
               nmc_photon_record* recs, float* events, uint32_t k) {
  const bool replay = (c.ext.flags & NMC_FLAG_TT_REPLAY_RUN1) != 0;
  for (uint64_t j = lo; j < hi; ++j) {
    const uint64_t p = first + j;
    Trace tr{recs ? recs + j : nullptr, events ? events + (size_t)j * k * 4 : nullptr, k};
    if (tr.ev)
      for (size_t m = 0; m < (size_t)k * 4; ++m) tr.ev[m] = NAN;
    if (c.ext.rng == NMC_RNG_TAUS_REF) {
      TausStream g = taus_for(c.sim, p, c.ext.photons_per_dispatch, replay);
      run_photon<R>(c, g, T, tr, p);
    } else {
      PhiloxStream g(c.ext.seed, p, two_term_family(c));
      run_photon<R>(c, g, T, tr, p);
    }
    T.ph += 1;
  }
}

bool valid_inputs(const Cfg& c) {
  if (c.sim == NMC_SIM_MCSUB) {
    const int b = c.ext.sub_bins;
    return b >= 2 && c.ext.sub_dr > 0 && c.ext.sub_dz > 0 &&
           c.tp.muav[kMCSUB_LAYER] + c.tp.musv[kMCSUB_LAYER] > 0;
  }
  if (c.sim != NMC_SIM_MCXYZ && c.sim != NMC_SIM_MCXYZ_TT) return false;
  const nmc_run_params& rp = c.rp;
  if (!c.v || rp.Nx <= 0 || rp.Ny <= 0 || rp.Nz <= 0 || !(rp.dx > 0) || !(rp.dy > 0) ||
      !(rp.dz > 0))
    return false;
  const long n = (long)rp.Nx * rp.Ny * rp.Nz;
  for (long k = 0; k < n; ++k)
    if (c.v[k] >= NMC_NTISS || !(c.tp.musv[c.v[k]] > 0)) return false;
  return true;
}

// ------------------------------------------------------------ layered media
// The multi-layer extension of the mcsub kernel behind nmc_layered_run.  The
// reference declares MAXLAYERS = 100 (definitions.h:24) and never uses it, so
// this restates the engine's own model, which keeps the mcsub kernel's
// physics (kernels.metal:59-319) in every layer:
//   HOP    s = -ln(xi) / mu_t of the current layer; a step that reaches a
//          layer boundary stops there and the rest of the dimensionless step
//          carries into the next layer;
//   CROSS  Fresnel reflection R(n_i, n_t, |uz|) (helpers.metal:243-291) by a
//          random draw, as the mcsub kernel does at its surface
//          (kernels.metal:183-214); otherwise refraction (Snell) into the
//          next layer, or escape into the ambient medium (Rd(r) above,
//          Tt(r) below);
//   DROP   absorb = W mua / mu_t (kernels.metal:224-234);
//   SPIN   Henyey-Greenstein with the layer's g (kernels.metal:244-279);
//   ROULETTE below 1e-4, chance 0.1 (kernels.metal:289-294).
// Random numbers, as the engine draws them: Philox4x32-10, key (seed lo,
// seed hi), counter (photon lo, photon hi, interaction, 'LAYR'): x step,
// y cos theta, z psi, w roulette; boundary events draw their Fresnel choice
// from counter (photon lo, photon hi, event | 2^31, 'LAYR').  With
// NMC_FLAG_LAYERED_REF_STREAMS they come from the reference's generator in
// MCSubKernel's order (kernels.metal:91-95 seeding, a launch draw :113, then
// per hop the step :183, the Fresnel choice :191, cos theta :244, psi :255
// and the roulette draw :290), photon p = (run p / seed + 1, index p % seed);
// NMC_FLAG_LAYERED_ISOTROPIC samples cos theta as 2 xi - 1 (:252).
constexpr uint32_t kLayTag = 0x4C415952u;
constexpr uint32_t kLayStepCap = 20000000u;

struct LayTally {
  std::vector<double> rd, tt, az, al;
  double s[NMC_LAY_FIELDS] = {};
  bool capped = false;
};

struct LayGeom {
  nmc_layered_config c;
  std::vector<nmc_layer> lay;
  std::vector<double> z0, z1;  // z1 = +inf for a semi-infinite last layer
  double w0;
};

template <class R>
void layered_photon(const LayGeom& G, uint64_t pid, LayTally& T, double* per_photon) {
  const uint32_t c0 = (uint32_t)pid, c1 = (uint32_t)(pid >> 32);
  const uint32_t k0 = (uint32_t)G.c.seed, k1 = (uint32_t)(G.c.seed >> 32);
  auto block = [&](uint32_t c2, uint32_t* out) {
    uint32_t q[4] = {c0, c1, c2, kLayTag};
    philox10(q, k0, k1);
    std::memcpy(out, q, sizeof q);
  };
  auto u = [](uint32_t x) { return R(x >> 9) * R(1.0 / 8388608.0) + R(1.0 / 16777216.0); };
  const bool ref = (G.c.flags & NMC_FLAG_LAYERED_REF_STREAMS) != 0;
  const bool iso = (G.c.flags & NMC_FLAG_LAYERED_ISOTROPIC) != 0;
  TausStream g = taus_for(NMC_SIM_MCSUB, pid, ref ? G.c.seed : 1, false);
  if (ref) g.next_f();  // the launch draw (kernels.metal:113; radius 0 puts the beam on the axis)
  const int nl = G.c.n_layers, nr = G.c.nr, nz = G.c.nz;
  const R idr = R(1) / R(G.c.dr), idz = R(1) / R(G.c.dz);
  R x = 0, y = 0, z = 0, ux = 0, uy = 0, uz = 1, w = R(G.w0), sleft = 0, rd = 0, tt = 0, atot = 0;
  int L = 0;
  uint32_t hop = 0, ev = 0;
  bool alive = true;
  uint32_t r[4];
  if (!ref) block(0u, r);
  while (alive) {
    const nmc_layer& Ly = G.lay[L];
    const R mut = R(Ly.mua) + R(Ly.mus);
    if (sleft <= R(0)) {
      if (ref) {
        float v;
        while ((v = g.next_f()) <= 0.f) {
        }
        sleft = -std::log(R(v));
      } else {
        sleft = -std::log(u(r[0]));
      }
    }
    const R db = uz > R(0) ? (R(G.z1[L]) - z) / uz : (uz < R(0) ? (R(G.z0[L]) - z) / uz : R(INFINITY));
    const R s = mut > R(0) ? sleft / mut : R(INFINITY);
    if (s >= db) {  // CROSS
      x += db * ux;
      y += db * uy;
      z = uz > R(0) ? R(G.z1[L]) : R(G.z0[L]);
      if (mut > R(0)) sleft = std::max(sleft - db * mut, R(0));
      const bool down = uz > R(0);
      const int Ln = down ? L + 1 : L - 1;
      const R nt = Ln < 0 ? R(G.c.n_above) : (Ln >= nl ? R(G.c.n_below) : R(G.lay[Ln].n));
      R uzt = 0;
      const R Rf = rfresnel<R>(R(Ly.n), nt, std::fabs(uz), &uzt);
      R uf;
      if (ref) {
        uf = R(g.next_f());
      } else {
        uint32_t a[4];
        block(ev | 0x80000000u, a);
        uf = u(a[0]);
      }
      ++ev;
      if (uf <= Rf) {
        uz = -uz;
      } else if (Ln < 0 || Ln >= nl) {  // escapes
        const int ir = std::min((int)(std::sqrt(x * x + y * y) * idr), nr);
        if (Ln < 0) {
          if (!T.rd.empty()) T.rd[ir] += (double)w;
          rd += w;
        } else {
          if (!T.tt.empty()) T.tt[ir] += (double)w;
          tt += w;
        }
        alive = false;
      } else {  // refracted (Snell)
        const R ratio = R(Ly.n) / nt;
        ux *= ratio;
        uy *= ratio;
        uz = down ? uzt : -uzt;
        L = Ln;
      }
      if (ev > kLayStepCap) {
        T.capped = true;
        alive = false;
      }
      continue;
    }
    // interaction inside the layer: HOP, DROP, SPIN, ROULETTE
    x += s * ux;
    y += s * uy;
    z += s * uz;
    sleft = 0;
    const R absorb = w * R(Ly.mua) / mut;
    w -= absorb;
    atot += absorb;
    if (absorb > R(0)) {
      const int iz = std::min(std::max((int)(z * idz), 0), nz);
      if (!T.az.empty()) T.az[iz] += (double)absorb;
      T.al[L] += (double)absorb;
    }
    const R ucos = ref ? R(g.next_f()) : u(r[1]);
    const R cth = iso ? R(2) * ucos - R(1) : hg_costheta<R>(R(Ly.g), ucos);
    spin_u<R>(cth, ref ? R(g.next_f()) : u(r[2]), ux, uy, uz);
    if (w < R(kTHRESHOLD)) {
      if ((ref ? R(g.next_f()) : u(r[3])) <= R(kCHANCE))
        w /= R(kCHANCE);
      else
        alive = false;
    }
    ++hop;
    if (hop > kLayStepCap) {
      T.capped = true;
      alive = false;
    }
    if (!ref) block(hop, r);
  }
  if (per_photon) {
    per_photon[0] = (double)rd;
    per_photon[1] = (double)tt;
    per_photon[2] = (double)atot;
  }
  T.s[NMC_LAY_PHOTONS] += 1.0;
  T.s[NMC_LAY_RD] += (double)rd;
  T.s[NMC_LAY_RD2] += (double)rd * (double)rd;
  T.s[NMC_LAY_TT] += (double)tt;
  T.s[NMC_LAY_TT2] += (double)tt * (double)tt;
  T.s[NMC_LAY_INTERACTIONS] += (double)hop;
}

// ------------------------------------------------- polarised E-field model
// The engine's E-field transport behind nmc_efield_run, restated in R (the
// reference's E-field and Raman kernels are empty, kernels.metal:1122-1202):
// each photon carries a right-handed frame (e_par, e_perp, u) and a complex
// 2x2 Jones matrix T (rows par, perp; columns the lab inputs x, y).  theta
// from the inverse CDF of the unpolarised Mie phase function (linear within a
// table interval), phi from 1 + beta cos(2 phi - 2 phi0) by a safeguarded
// Newton inversion of its CDF, then T <- diag(S2, S1) R(phi) T rescaled to
// |T|_F^2 = 2.  Unpolarised Fresnel escape or mirror at z = 0; Raman
// conversion to the second table, isotropic and unpolarised; roulette below
// 1e-4 (chance 0.1).  Random numbers as the engine draws them: Philox4x32-10,
// key (seed lo, seed hi + setting), counter (photon lo, photon hi, hop,
// 'EFLD'): x step, y theta (or emission cos), z phi, w Raman choice; the aux
// block (hop | 2^30) gives x the Fresnel choice and y roulette.
constexpr uint32_t kEfTag = 0x45464C44u;

struct EfInput {
  nmc_efield_config c;
  int n;
  std::vector<float> S[2];    // 4 floats per angle: S1 re, im, S2 re, im
  std::vector<float> cdf[2];  // as the engine builds it (FP64 trapezoids, stored as float)
  double inv_mut[2], surv[2], p_raman[2];
  float dtheta;
  bool cone;
  float sep_inv, sep_half;
};

bool ef_cdf(const float* S, int n, std::vector<float>& cdf) {
  std::vector<double> c(n, 0.0);
  const double dth = 3.14159265358979323846 / (n - 1);
  auto dens = [&](int j) {
    const double p = 0.5 * ((double)S[4 * j] * S[4 * j] + (double)S[4 * j + 1] * S[4 * j + 1] +
                            (double)S[4 * j + 2] * S[4 * j + 2] + (double)S[4 * j + 3] * S[4 * j + 3]);
    return p * std::sin(dth * j);
  };
  for (int j = 1; j < n; ++j) c[j] = c[j - 1] + 0.5 * (dens(j - 1) + dens(j)) * dth;
  if (!(c[n - 1] > 0.0) || !std::isfinite(c[n - 1])) return false;
  cdf.resize(n);
  for (int j = 0; j < n; ++j) cdf[j] = (float)(c[j] / c[n - 1]);
  cdf[0] = 0.f;
  cdf[n - 1] = 1.f;
  return true;
}

template <class R>
struct Cx {
  R re, im;
};
template <class R>
Cx<R> cmul(Cx<R> a, Cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class R>
R cnorm(Cx<R> a) {
  return a.re * a.re + a.im * a.im;
}

// phi with CDF (phi + beta/2 (sin(2 phi - tp0) + sin tp0)) / (2 pi) = u; s0, c0 = sin, cos tp0
template <class R>
R ef_phi(R u, R beta, R s0, R c0) {
  const R two_pi = R(2.0 * 3.14159265358979323846);
  const R target = two_pi * u;
  if (std::fabs(beta) < R(1e-6)) return target;
  R lo = 0, hi = two_pi, phi = target;
  for (int it = 0; it < 40; ++it) {
    const R s2 = std::sin(R(2) * phi), c2 = std::cos(R(2) * phi);
    const R sa = s2 * c0 - c2 * s0, ca = c2 * c0 + s2 * s0;
    const R G = phi + R(0.5) * beta * (sa + s0) - target;
    if (std::fabs(G) < R(2e-6)) break;
    if (G > 0)
      hi = phi;
    else
      lo = phi;
    const R dG = R(1) + beta * ca;
    R nx = dG > R(1e-6) ? phi - G / dG : R(0.5) * (lo + hi);
    if (!(nx > lo && nx < hi)) nx = R(0.5) * (lo + hi);
    phi = nx;
  }
  return phi;
}

template <class R>
void ef_perp(R ux, R uy, R& px, R& py, R& pz) {
  const R n2 = ux * ux + uy * uy;
  if (n2 < R(1e-12)) {
    px = 0;
    py = 1;
  } else {
    const R r = R(1) / std::sqrt(n2);
    px = -uy * r;
    py = ux * r;
  }
  pz = 0;
}

template <class R>
void ef_photon(const EfInput& in, const nmc_efield_setting& q, uint32_t set, uint64_t pid, double* o) {
  const nmc_efield_config& c = in.c;
  const uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32) + set;
  const uint32_t c0 = (uint32_t)pid, c1 = (uint32_t)(pid >> 32);
  auto block = [&](uint32_t c2, uint32_t* out) {
    uint32_t b[4] = {c0, c1, c2, kEfTag};
    philox10(b, k0, k1);
    std::memcpy(out, b, sizeof b);
  };
  auto u01 = [](uint32_t x) { return R(x >> 9) * R(1.0 / 8388608.0) + R(1.0 / 16777216.0); };
  // launch: refracted direction, its s direction, initial T (the engine's host set-up)
  const double st_ = std::sin((double)q.theta_in) * c.n_outside / c.n_medium, ct_ = std::sqrt(1.0 - st_ * st_);
  R ux = R(st_ * std::cos((double)q.phi_in)), uy = R(st_ * std::sin((double)q.phi_in)), uz = R(ct_);
  R px, py, pz;
  if (st_ < 1e-9) {
    px = 0;
    py = 1;
    pz = 0;
  } else {
    ef_perp<R>(ux, uy, px, py, pz);
  }
  Cx<R> T00, T01, T10, T11;
  {
    const R qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;
    R t[2][2], f = 0;
    for (int b = 0; b < 2; ++b) {
      R bx = b == 0 ? 1 : 0, by = b == 0 ? 0 : 1, bz = 0;
      const R du = bx * ux + by * uy + bz * uz;
      bx -= du * ux;
      by -= du * uy;
      bz -= du * uz;
      t[0][b] = bx * qx + by * qy + bz * qz;
      t[1][b] = bx * px + by * py + bz * pz;
      f += t[0][b] * t[0][b] + t[1][b] * t[1][b];
    }
    const R sc = std::sqrt(R(2) / f);
    T00 = {t[0][0] * sc, 0};
    T01 = {t[0][1] * sc, 0};
    T10 = {t[1][0] * sc, 0};
    T11 = {t[1][1] * sc, 0};
  }
  R dummy;
  const R w0 = R(1) - rfresnel<R>(R(c.n_outside), R(c.n_medium), R(std::cos((double)q.theta_in)), &dummy);
  o[NMC_EF_PHOTONS] += 1.0;
  o[NMC_EF_SPECULAR] += (double)(R(1) - w0);
  R x = 0, y = 0, z = 0, w = w0, fx = 0, fy = 0, lx = 0, ly = 0;
  int med = 0;
  uint32_t nsc = 0, hop = 0;
  bool alive = true, escaped = false;
  while (alive) {
    uint32_t r[4];
    block(hop, r);
    const R s = -std::log(u01(r[0])) * R(in.inv_mut[med]);
    if (uz < 0 && z + s * uz < 0) {  // reaches the surface
      const R d = -z / uz;
      x += d * ux;
      y += d * uy;
      z = 0;
      R uzt;
      const R rsp = rfresnel<R>(R(c.n_medium), R(c.n_outside), -uz, &uzt);
      uint32_t a[4];
      block(hop | 0x40000000u, a);
      if (u01(a[0]) > rsp) {
        escaped = true;
        break;
      }
      uz = -uz;
      px = -px;
      py = -py;
      T10 = {-T10.re, -T10.im};
      T11 = {-T11.re, -T11.im};
      const R rest = s - d;
      x += rest * ux;
      y += rest * uy;
      z = rest * uz;
    } else {
      x += s * ux;
      y += s * uy;
      z += s * uz;
    }
    w *= R(in.surv[med]);
    if (med == 0 && u01(r[3]) < R(in.p_raman[0])) {  // Raman conversion
      med = 1;
      o[NMC_EF_RAMAN_N] += 1.0;
      const R ct = R(2) * u01(r[1]) - R(1), st = std::sqrt(std::max(R(0), R(1) - ct * ct));
      const R ps = R(2.0 * 3.14159265358979323846) * u01(r[2]);
      ux = st * std::cos(ps);
      uy = st * std::sin(ps);
      uz = ct;
      ef_perp<R>(ux, uy, px, py, pz);
      T00 = {1, 0};
      T01 = {0, 0};
      T10 = {0, 0};
      T11 = {1, 0};
    } else {  // scattering
      const std::vector<float>& cdf = in.cdf[med];
      const std::vector<float>& S = in.S[med];
      const R uth = u01(r[1]);
      int a0 = 0, a1 = in.n - 1;
      while (a1 - a0 > 1) {
        const int mid = (a0 + a1) >> 1;
        if (R(cdf[mid]) <= uth) a0 = mid; else a1 = mid;
      }
      const R q0 = cdf[a0], q1 = cdf[a1];
      const R fr = q1 > q0 ? std::min(std::max((uth - q0) / (q1 - q0), R(0)), R(1)) : R(0.5);
      const R th = (R(a0) + fr) * R(in.dtheta);
      const R sth = std::sin(th), cth = std::cos(th);
      auto lerp = [&](int k) { return R(S[4 * a0 + k]) + fr * (R(S[4 * a1 + k]) - R(S[4 * a0 + k])); };
      const Cx<R> S1 = {lerp(0), lerp(1)}, S2 = {lerp(2), lerp(3)};
      const R Pp = cnorm(T00) + cnorm(T01), Qp = cnorm(T10) + cnorm(T11);
      const R Cp = T00.re * T10.re + T00.im * T10.im + T01.re * T11.re + T01.im * T11.im;
      const R s1 = cnorm(S1), s2 = cnorm(S2), hd = R(0.5) * (Pp - Qp);
      const R rho = std::sqrt(hd * hd + Cp * Cp), den = (s1 + s2) * R(0.5) * (Pp + Qp);
      const R beta = den > 0 ? std::min(std::max((s2 - s1) * rho / den, R(-1)), R(1)) : R(0);
      const R irho = rho > 0 ? R(1) / rho : R(0);
      const R phi = ef_phi<R>(u01(r[2]), beta, Cp * irho, hd * irho);
      const R sph = std::sin(phi), cph = std::cos(phi);
      const R qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;  // e_par
      const R e1x = cph * qx + sph * px, e1y = cph * qy + sph * py, e1z = cph * qz + sph * pz;
      R e2x = -sph * qx + cph * px, e2y = -sph * qy + cph * py, e2z = -sph * qz + cph * pz;
      R nux = cth * ux + sth * e1x, nuy = cth * uy + sth * e1y, nuz = cth * uz + sth * e1z;
      const R ru = R(1) / std::sqrt(nux * nux + nuy * nuy + nuz * nuz);
      nux *= ru;
      nuy *= ru;
      nuz *= ru;
      const R dp = e2x * nux + e2y * nuy + e2z * nuz;
      e2x -= dp * nux;
      e2y -= dp * nuy;
      e2z -= dp * nuz;
      const R rp = R(1) / std::sqrt(e2x * e2x + e2y * e2y + e2z * e2z);
      ux = nux;
      uy = nuy;
      uz = nuz;
      px = e2x * rp;
      py = e2y * rp;
      pz = e2z * rp;
      const Cx<R> b00 = {cph * T00.re + sph * T10.re, cph * T00.im + sph * T10.im};
      const Cx<R> b01 = {cph * T01.re + sph * T11.re, cph * T01.im + sph * T11.im};
      const Cx<R> b10 = {-sph * T00.re + cph * T10.re, -sph * T00.im + cph * T10.im};
      const Cx<R> b11 = {-sph * T01.re + cph * T11.re, -sph * T01.im + cph * T11.im};
      T00 = cmul(S2, b00);
      T01 = cmul(S2, b01);
      T10 = cmul(S1, b10);
      T11 = cmul(S1, b11);
      const R fn = cnorm(T00) + cnorm(T01) + cnorm(T10) + cnorm(T11);
      const R sc = fn > 0 ? std::sqrt(R(2) / fn) : R(0);
      for (Cx<R>* t : {&T00, &T01, &T10, &T11}) {
        t->re *= sc;
        t->im *= sc;
      }
      if (med == 0) {
        if (nsc == 0) {
          fx = x;
          fy = y;
        }
        lx = x;
        ly = y;
      }
      ++nsc;
    }
    if (w < R(1e-4)) {
      uint32_t a[4];
      block(hop | 0x40000000u, a);
      if (u01(a[1]) <= R(0.1))
        w *= R(10);
      else
        alive = false;
    }
    if (++hop >= 20000000u) alive = false;
  }
  o[NMC_EF_SCATTERS] += nsc;
  if (!escaped) return;
  const R qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;  // e_par
  Cx<R> A[2][2];
  for (int a = 0; a < 2; ++a) {
    R ax = a == 0 ? 1 : 0, ay = a == 0 ? 0 : 1, az = 0;
    const R du = ax * ux + ay * uy;
    ax -= du * ux;
    ay -= du * uy;
    az -= du * uz;
    const R ra = R(1) / std::sqrt(std::max(ax * ax + ay * ay + az * az, R(1e-20)));
    const R cpar = (ax * qx + ay * qy + az * qz) * ra, cperp = (ax * px + ay * py + az * pz) * ra;
    A[a][0] = {T00.re * cpar + T10.re * cperp, T00.im * cpar + T10.im * cperp};
    A[a][1] = {T01.re * cpar + T11.re * cperp, T01.im * cpar + T11.im * cperp};
  }
  const R ex = R(std::cos(q.pol_angle)), ey = R(std::sin(q.pol_angle));
  const Cx<R> Fx = {A[0][0].re * ex + A[0][1].re * ey, A[0][0].im * ex + A[0][1].im * ey};
  const Cx<R> Fy = {A[1][0].re * ex + A[1][1].re * ey, A[1][0].im * ex + A[1][1].im * ey};
  const Cx<R> Eco = {ex * Fx.re + ey * Fy.re, ex * Fx.im + ey * Fy.im};
  const Cx<R> Ecr = {-ey * Fx.re + ex * Fy.re, -ey * Fx.im + ex * Fy.im};
  const R Ico = w * cnorm(Eco), Icr = w * cnorm(Ecr);
  if (med == 1) {
    o[NMC_EF_RAMAN_RD] += (double)w;
    o[NMC_EF_RAMAN_CO] += (double)Ico;
    o[NMC_EF_RAMAN_CROSS] += (double)Icr;
    return;
  }
  o[NMC_EF_RD] += (double)w;
  o[NMC_EF_RD2] += (double)w * (double)w;
  o[NMC_EF_CO] += (double)Ico;
  o[NMC_EF_CROSS] += (double)Icr;
  if (nsc >= 2) {  // the time-reversed partner: the transposed lab-frame amplitude
    const Cx<R> Gx = {-A[0][0].re * ey + A[0][1].re * ex, -A[0][0].im * ey + A[0][1].im * ex};
    const Cx<R> Gy = {-A[1][0].re * ey + A[1][1].re * ex, -A[1][0].im * ey + A[1][1].im * ex};
    const Cx<R> Er = {ex * Gx.re + ey * Gy.re, ex * Gx.im + ey * Gy.im};
    const R cco = cnorm(Eco), ccr = Ecr.re * Er.re + Ecr.im * Er.im;  // Re(Ecr conj(Er))
    o[NMC_EF_MULTI_CO] += (double)Ico;
    o[NMC_EF_MULTI_CROSS] += (double)Icr;
    o[NMC_EF_INTERF_CO] += (double)(w * cco);
    o[NMC_EF_INTERF_CROSS] += (double)(w * ccr);
    if (in.cone) {
      const int i = (int)std::floor((double)((lx - fx + R(in.sep_half)) * R(in.sep_inv)));
      const int j = (int)std::floor((double)((ly - fy + R(in.sep_half)) * R(in.sep_inv)));
      if (!(i >= 0 && i < c.sep_n && j >= 0 && j < c.sep_n)) o[NMC_EF_SEP_OUTSIDE] += (double)(w * cco);
    }
  }
}

}  // namespace

extern "C" {

int orc_run(int sim_type, int real_bits, const nmc_run_params* rp, const nmc_tissue_params* tp,
            const uint8_t* v, const nmc_ext* ext, uint64_t first, uint64_t n, int nthreads,
            orc_out* out, nmc_photon_record* recs, float* events, uint32_t k_events) {
  if (!rp || !tp || !ext || !out || (real_bits != 32 && real_bits != 64)) return NMC_EINVAL;
  Cfg c;
  c.sim = sim_type;
  c.rp = *rp;
  c.tp = *tp;
  c.v = v;
  c.ext = *ext;
  if (c.ext.photons_per_dispatch == 0) return NMC_EINVAL;
  if (!valid_inputs(c)) return NMC_EINVAL;
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > n) nthreads = n ? (int)n : 1;
  const size_t nJ = (size_t)c.ext.sub_bins + 1, nF = nJ * nJ;
  const size_t nvox = (size_t)rp->Nx * rp->Ny * rp->Nz, n2d = (size_t)rp->Nx * rp->Ny;
  const bool xyz = sim_type != NMC_SIM_MCSUB;
  std::vector<Tally> T(nthreads);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    const uint64_t lo = share_begin(n, t, nthreads), hi = share_begin(n, t + 1, nthreads);
    th.emplace_back([&, t, lo, hi] {
      Tally& tl = T[t];
      if (!xyz) {
        if (out->J) tl.J.assign(nJ, 0.0);
        if (out->F) tl.F.assign(nF, 0.0);
      } else {
        if (out->F3D) tl.F3D.assign(nvox, 0.0);
        if (out->Rd2D) tl.Rd2D.assign(n2d, 0.0);
        if (out->DetPhot2D) tl.Det.assign(n2d, 0.0);
        if (out->rd_slots) tl.slots.assign(c.ext.photons_per_dispatch, 0.0);
      }
      if (real_bits == 64)
        run_range<double>(c, first, lo, hi, tl, recs, events, k_events);
      else
        run_range<float>(c, first, lo, hi, tl, recs, events, k_events);
    });
  }
  for (auto& x : th) x.join();
  for (int t = 0; t < nthreads; ++t) {
    const Tally& tl = T[t];
    for (size_t k = 0; k < tl.J.size(); ++k) out->J[k] += tl.J[k];
    for (size_t k = 0; k < tl.F.size(); ++k) out->F[k] += tl.F[k];
    for (size_t k = 0; k < tl.F3D.size(); ++k) out->F3D[k] += tl.F3D[k];
    for (size_t k = 0; k < tl.Rd2D.size(); ++k) out->Rd2D[k] += tl.Rd2D[k];
    for (size_t k = 0; k < tl.Det.size(); ++k) out->DetPhot2D[k] += tl.Det[k];
    for (size_t k = 0; k < tl.slots.size(); ++k) out->rd_slots[k] += tl.slots[k];
    out->S += tl.S;
    out->A += tl.A;
    out->E += tl.E;
    out->rd_sum += tl.rd;
    out->rd_sumsq += tl.rd2;
    out->photons += tl.ph;
    out->substeps += tl.sub;
    out->scatters += tl.sc;
  }
  return 0;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox10(c, key[0], key[1]);
  for (int k = 0; k < 4; ++k) out[k] = c[k];
}

void orc_uniforms(const nmc_ext* ext, int sim_type, uint64_t photon_id, int n, double* out) {
  if (ext->rng == NMC_RNG_TAUS_REF) {
    TausStream g = taus_for(sim_type, photon_id, ext->photons_per_dispatch,
                            (ext->flags & NMC_FLAG_TT_REPLAY_RUN1) != 0);
    for (int k = 0; k < n; ++k) out[k] = g.u<double>(D_STEP);
  } else {
    // Philox: the n uniforms are hop 0's main block, then hop 1's, ...
    PhiloxStream g(ext->seed, photon_id, false);
    for (int k = 0; k < n; ++k) {
      if (k % 4 == 0) g.new_hop();
      out[k] = g.u<double>((Draw)(k % 4 == 0 ? D_STEP : k % 4 == 1 ? D_COS : k % 4 == 2 ? D_PSI : D_ROUL));
    }
  }
}

double orc_rfresnel(double n1, double n2, double ca1, double* ca2) {
  return rfresnel<double>(n1, n2, ca1, ca2);
}

double orc_tt_costheta(double gf, double af, double gb, double ab, double cc, double u_choice,
                       double u_sample) {
  FixedDraws g{{u_choice, u_sample}};
  TTq<double> q;
  q.set(gf, af, gb, ab);
  return tt_costheta<double>(g, q, gf, af, gb, ab, cc);
}

double orc_hg_costheta(double g, double u) { return hg_costheta<double>(g, u); }

int orc_efield_run(int real_bits, const nmc_efield_config* cfg, const float* S_primary, const float* S_raman,
                   const nmc_efield_setting* settings, int n_settings, int cone, int nthreads, double* out) {
  if (!cfg || !S_primary || !settings || !out || n_settings < 1 || (real_bits != 32 && real_bits != 64))
    return NMC_EINVAL;
  EfInput in;
  in.c = *cfg;
  const nmc_efield_config& c = in.c;
  in.n = c.n_angles;
  if (in.n < 2 || !(c.mua + c.mus > 0.f)) return NMC_EINVAL;
  const bool raman = c.mu_raman > 0.f;
  if (raman && (!S_raman || !(c.raman_mua + c.raman_mus > 0.f))) return NMC_EINVAL;
  in.S[0].assign(S_primary, S_primary + 4 * (size_t)in.n);
  in.S[1].assign(raman ? S_raman : S_primary, (raman ? S_raman : S_primary) + 4 * (size_t)in.n);
  if (!ef_cdf(in.S[0].data(), in.n, in.cdf[0]) || !ef_cdf(in.S[1].data(), in.n, in.cdf[1])) return NMC_EINVAL;
  const double mut0 = (double)c.mua + c.mus + c.mu_raman;
  in.inv_mut[0] = (float)(1.0 / mut0);  // the engine's per-medium constants (floats)
  in.surv[0] = (float)((c.mus + c.mu_raman) / mut0);
  in.p_raman[0] = (c.mus + c.mu_raman) > 0.f ? (float)(c.mu_raman / ((double)c.mus + c.mu_raman)) : 0.f;
  const double mut1 = raman ? (double)c.raman_mua + c.raman_mus : mut0;
  in.inv_mut[1] = (float)(1.0 / mut1);
  in.surv[1] = raman ? (float)(c.raman_mus / mut1) : in.surv[0];
  in.p_raman[1] = 0.0;
  in.dtheta = (float)(3.14159265358979323846 / (in.n - 1));
  in.cone = cone != 0;
  in.sep_inv = in.cone ? (float)(c.sep_n / (2.0 * c.sep_half_width)) : 0.f;
  in.sep_half = c.sep_half_width;
  if (nthreads < 1) nthreads = 1;
  for (int set = 0; set < n_settings; ++set) {
    const nmc_efield_setting& q = settings[set];
    const uint64_t n = q.photons;
    const int nt = (int)std::min<uint64_t>((uint64_t)nthreads, std::max<uint64_t>(n, 1));
    std::vector<std::vector<double>> part(nt, std::vector<double>(NMC_EF_FIELDS, 0.0));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t] {
        for (uint64_t i = share_begin(n, t, nt), e = share_begin(n, t + 1, nt); i < e; ++i) {
          if (real_bits == 64)
            ef_photon<double>(in, q, (uint32_t)set, i, part[t].data());
          else
            ef_photon<float>(in, q, (uint32_t)set, i, part[t].data());
        }
      });
    for (auto& x : th) x.join();
    for (int t = 0; t < nt; ++t)
      for (int k = 0; k < NMC_EF_FIELDS; ++k) out[(size_t)set * NMC_EF_FIELDS + k] += part[t][k];
  }
  return 0;
}

int orc_layered_run(int real_bits, const nmc_layered_config* cfg, const nmc_layer* layers, uint64_t first,
                    uint64_t n, int nthreads, double* out, double* rd_r, double* tt_r, double* a_z,
                    double* a_layer, double* per_photon) {
  if (!cfg || !layers || !out || (real_bits != 32 && real_bits != 64)) return NMC_EINVAL;
  if ((cfg->flags & NMC_FLAG_LAYERED_REF_STREAMS) && cfg->seed == 0) return NMC_EINVAL;
  LayGeom G;
  G.c = *cfg;
  const nmc_layered_config& c = G.c;
  if (c.n_layers < 1 || c.n_layers > 100 || c.nr < 1 || c.nz < 1 || !(c.dr > 0.f) || !(c.dz > 0.f) ||
      !(c.n_above > 0.f) || !(c.n_below > 0.f))
    return NMC_EINVAL;
  double zc = 0.0;
  for (int i = 0; i < c.n_layers; ++i) {
    const nmc_layer& q = layers[i];
    const bool last = i == c.n_layers - 1;
    if (!(q.mua >= 0.f) || !(q.mus >= 0.f) || !(q.g > -1.f) || !(q.g < 1.f) || !(q.n > 0.f) ||
        !(q.thickness > 0.f) || (!last && !std::isfinite(q.thickness)) ||
        (!std::isfinite(q.thickness) && !(q.mua + q.mus > 0.f)))
      return NMC_EINVAL;
    G.lay.push_back(q);
    G.z0.push_back(zc);
    zc += q.thickness;
    G.z1.push_back(std::isfinite(q.thickness) ? zc : INFINITY);
  }
  const double rs = ((double)c.n_above - layers[0].n) / ((double)c.n_above + layers[0].n);
  const double rsp = rs * rs;
  G.w0 = 1.0 - rsp;
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > n) nthreads = n ? (int)n : 1;
  std::vector<LayTally> T(nthreads);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    const uint64_t lo = share_begin(n, t, nthreads), hi = share_begin(n, t + 1, nthreads);
    th.emplace_back([&, t, lo, hi] {
      LayTally& tl = T[t];
      if (rd_r) tl.rd.assign((size_t)c.nr + 1, 0.0);
      if (tt_r) tl.tt.assign((size_t)c.nr + 1, 0.0);
      if (a_z) tl.az.assign((size_t)c.nz + 1, 0.0);
      tl.al.assign((size_t)c.n_layers, 0.0);
      for (uint64_t i = lo; i < hi; ++i) {
        double* pp = per_photon ? per_photon + 3 * i : nullptr;
        if (real_bits == 64)
          layered_photon<double>(G, first + i, tl, pp);
        else
          layered_photon<float>(G, first + i, tl, pp);
      }
    });
  }
  for (auto& x : th) x.join();
  bool capped = false;
  for (int t = 0; t < nthreads; ++t) {
    const LayTally& tl = T[t];
    for (int k = 0; k < NMC_LAY_FIELDS; ++k) out[k] += tl.s[k];
    for (size_t k = 0; k < tl.rd.size(); ++k) rd_r[k] += tl.rd[k];
    for (size_t k = 0; k < tl.tt.size(); ++k) tt_r[k] += tl.tt[k];
    for (size_t k = 0; k < tl.az.size(); ++k) a_z[k] += tl.az[k];
    for (int k = 0; k < c.n_layers; ++k) {
      out[NMC_LAY_A] += tl.al[k];
      if (a_layer) a_layer[k] += tl.al[k];
    }
    capped = capped || tl.capped;
  }
  out[NMC_LAY_SPECULAR] += rsp * (double)n;
  return capped ? NMC_ESTEPCAP : 0;
}

// The speckle mutual-interference post-processing of -[MetalMC
// getComputeResults:] (MetalMC.m:628-742), restated with the reference's
// types: float quantities, C's double sin / cos / atan2 / exp / sqrt of them,
// double constants MC_TWO = 2.0 and PI = 3.1415926 (definitions.h:60,77).
// The reference's dPhase / phase_total_diff_lg terms feed no output and are
// left out.  Map layout as nmc_speckle_mutual: NMC_EF_MAPS maps of nx*ny.
void orc_speckle_mutual(int nx, int ny, const float* maps, const nmc_speckle* rec, const int32_t* counts,
                        int kmax, float lambda, float lc, float* out) {
  const size_t np = (size_t)nx * ny;
  auto fin = [](float v) { return std::isfinite(v) ? v : 0.0f; };
  auto wrap = [](float a) { return (float)std::atan2(std::sin((double)a), std::cos((double)a)); };
  const double two = 2.0, pi_ref = 3.1415926;
  for (size_t p = 0; p < np; ++p) {
    const float XX_accum_temp = maps[NMC_EF_MAP_XX * np + p];
    const float XY_accum_temp = maps[NMC_EF_MAP_XY * np + p];
    const float norm_sum = XX_accum_temp + XY_accum_temp;
    const float det = maps[NMC_EF_MAP_DET * np + p];
    const float XX_accum = fin(norm_sum > 0.0f ? XX_accum_temp / norm_sum : 0.0f);
    const float XY_accum = fin(norm_sum > 0.0f ? XY_accum_temp / norm_sum : 0.0f);
    const float Ryx_accum = fin(maps[NMC_EF_MAP_RD * np + p] / det);
    const float Phase_accum = fin(maps[NMC_EF_MAP_PHASE0 * np + p] / det);
    const float Path_accum = fin(maps[NMC_EF_MAP_PHASE1 * np + p] / det);
    const float Scatt_accum = fin(maps[NMC_EF_MAP_PHASE2 * np + p] / det);
    const float Total_accum = fin(maps[NMC_EF_MAP_PHASE3 * np + p] / det);
    float XX_mutual = XX_accum, XY_mutual = XY_accum, Ryx_mutual = Ryx_accum;
    float Phase_sum = Phase_accum, Path_sum = Path_accum, Scatt_sum = Scatt_accum, Total_sum = Total_accum;
    float N_times = 1.0f;
    const int K = std::min<int>(counts[p], kmax);
    for (int k = 0; k < K; ++k) {
      const nmc_speckle& r = rec[(size_t)k * np + p];
      const float norm_c = r.XX + r.XY;
      const float XX_current = fin(norm_c > 0.0f ? r.XX / norm_c : 0.0f);
      const float XY_current = fin(norm_c > 0.0f ? r.XY / norm_c : 0.0f);
      const float Ryx_current = fin(r.Ryx);
      const float Phase_current = fin(r.Phase), Path_current = fin(r.Path), Scatt_current = fin(r.Scatt);
      const float dPath = wrap(Path_accum - Path_current);
      const float dScatt = wrap(Scatt_accum - Scatt_current);
      const float diff_linear = wrap(dPath + dScatt);
      const float interference = (float)std::sin((double)diff_linear);
      const float path_accum_mm = (float)((double)(Path_accum * lambda) / (two * pi_ref));
      const float path_current_mm = (float)((double)(Path_current * lambda) / (two * pi_ref));
      const float delta_path = (path_current_mm - path_accum_mm) / lc;
      float lc_contribution = (float)std::exp((double)(-delta_path * delta_path));
      lc_contribution = (!std::isfinite(lc_contribution) || lc <= 0.01f) ? 0.0f : lc_contribution;
      XX_mutual += (float)(((double)(XX_accum + XX_current) +
                            two * std::sqrt((double)(XX_accum * XX_current)) * interference * lc_contribution) /
                           4.0f);
      XY_mutual += (float)(((double)(XY_accum + XY_current) +
                            two * std::sqrt((double)(XY_accum * XY_current)) * interference * lc_contribution) /
                           4.0f);
      Ryx_mutual += (float)(((double)(Ryx_accum + Ryx_current) +
                             two * std::sqrt((double)(Ryx_accum * Ryx_current)) * interference * lc_contribution) /
                            4.0f);
      Phase_sum += Phase_current;
      Path_sum += Path_current;
      Scatt_sum += Scatt_current;
      Total_sum += wrap(Phase_current + Path_current + Scatt_current);
      N_times += 1.0f;
    }
    out[NMC_EF_MAP_RD * np + p] += Ryx_mutual;
    out[NMC_EF_MAP_DET * np + p] += N_times;
    out[NMC_EF_MAP_XX * np + p] += XX_mutual;
    out[NMC_EF_MAP_XY * np + p] += XY_mutual;
    out[NMC_EF_MAP_PHASE0 * np + p] += Phase_sum;
    out[NMC_EF_MAP_PHASE1 * np + p] += Path_sum;
    out[NMC_EF_MAP_PHASE2 * np + p] += Scatt_sum;
    out[NMC_EF_MAP_PHASE3 * np + p] += Total_sum;
  }
}

}  // extern "C"
