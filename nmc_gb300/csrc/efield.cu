// efield.cu - polarised electric-field transport in a semi-infinite slab of
// spheres, with the coherent-backscattering (CBS) cone and Raman conversion.
//
// No reference semantics to follow: the reference's E-field and Raman kernels
// are empty (kernels.metal:1122-1202).  Its host allocates the outputs such a
// kernel fills (MetalMC.m:206-328), which the exit maps and PolVsScatt here
// mirror.  The method, written from the physics:
//
// Field.  Each photon carries a right-handed frame (e_par, e_perp, u) and a
// complex 2x2 Jones matrix T whose column b is the field, in that frame, that
// an incident field along lab axis b (x or y) has become.  Carrying both
// columns gives the response to any incident polarisation from one path.
//
// Scattering.  theta is drawn from the unpolarised phase function
// (|S1|^2 + |S2|^2)/2 (inverse CDF of the tabulated Mie amplitudes, linear in
// each table interval); phi from the density the current field gives,
//   p(phi | theta) ∝ |S2|^2 |a_par|^2 + |S1|^2 |a_perp|^2 = 1 + beta cos(2 phi - 2 phi0),
// summed over both columns (a = rows of R(phi) T), by a safeguarded Newton
// inversion of its CDF.  Then T <- diag(S2, S1) R(phi) T, rescaled so that
// |T|_F^2 = 2.  With this sampling the photon weight is exactly the scalar
// weight (unpolarised light), and an incident polarisation e is measured as
// w |A e|^2, A = T projected on the lab analysers: the importance weight of
// the path for e relative to unpolarised light.  Absorption is the weight
// factor (mus + mu_raman)/mu_t per interaction and roulette below 1e-4
// (chance 0.1), as in the mcsub kernel (kernels.metal:224-234, 289-294).
//
// Surface.  At z = 0 the photon escapes with probability 1 - R (unpolarised
// Fresnel, the reference's RFresnel, helpers.metal:243-291) or is mirrored
// (geometric mirror of the frame; the Fresnel phases of the two polarisations
// are not modelled).
//
// CBS.  For a photon scattered at least twice, its time-reversed partner path
// (the same scatterers visited backwards) has, by reciprocity, the transposed
// amplitude in the lab frame: e'.(A^T e) = e.(A e') for input e, analyser e'.
// Every backscattered photon is paired as if it left exactly backwards, and
// the pair interferes with phase q . (rho_last - rho_first), q the
// transverse wavevector of the detection direction in air.  The kernel bins
// c = w E conj(E_reversed) by the separation rho_last - rho_first (co and
// cross channels); the cone on the angular grid is the 2-D Fourier sum of
// that histogram, two complex matrix products (twiddle_kernel, cgemm).
//
// Raman.  With probability mu_raman / (mus + mu_raman) an interaction converts
// the photon: it continues at the Raman wavelength's properties and table,
// re-emitted isotropically and unpolarised (T = I).
//
// Random numbers: Philox4x32-10, key (seed lo, seed hi + setting), counter
// (photon lo, photon hi, hop, 'EFLD'): x step, y theta (or emission cos),
// z phi, w Raman choice; the aux block (counter hop | 2^30) gives x the
// Fresnel choice and y roulette.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "nmc_abi.h"

namespace nmc {
namespace {

constexpr int kEfMaxSets = 64;
constexpr uint32_t kEfTag = 0x45464C44u;
constexpr float kEfRoulette = 1e-4f, kEfChance = 0.1f;
constexpr float kTwoPi = 6.28318530717958648f;

struct EfMedium {
  float inv_mut;  // 1 / mu_t
  float surv;     // weight kept per interaction: (mus + mu_raman) / mu_t
  float p_raman;  // P(conversion | interaction survives)
  float kmed;     // 2 pi n_medium / lambda
  const float4* S;
  int cdf_off;  // of its CDF in shared memory
};

struct EfSet {
  float ex, ey;                // incident polarisation (lab)
  float ux, uy, uz, px, py, pz;  // refracted direction and e_perp
  float w0;                    // 1 - specular reflectance
  float2 t[4];                 // initial T (rows par, perp; columns lab x, y)
  unsigned long long first;
};

struct EfParams {
  EfMedium med[2];
  const float* cdf;  // 2 * n_angles
  int n_angles;
  float dtheta;
  float n_medium, n_outside;
  const EfSet* sets;
  const unsigned long long* prefix;
  int nsets;
  unsigned long long total;
  uint32_t k0, k1;
  double* sums;  // nsets * NMC_EF_FIELDS
  double* sep;   // nsets * 2 * sep_n^2 complex (FP64 sums: no stagnation in long runs), or null
  int sep_n;
  float sep_inv, sep_half;
  double* pvs;   // nsets * 4 * (NMC_EF_MAX_ORDER + 1), or null
  double* maps;  // nsets * NMC_EF_MAPS * map_n^2 (FP64 sums, returned as float), or null
  int map_n;
  float map_inv;
  double* depth;  // nsets * depth_bins, or null
  int depth_bins;
  float depth_inv;
  unsigned long long* work;
  unsigned int* flags;
  uint32_t step_cap;
  nmc_speckle* spk;  // nsets * spk_max * map_n^2 records, or null
  int* spk_count;    // nsets * map_n^2 arrivals
  uint32_t spk_max;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float cnorm(float2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float wrap_pi(float a) { return a - kTwoPi * rintf(a * (1.f / kTwoPi)); }

// phi in [0, 2 pi) with CDF (phi + beta/2 (sin(2 phi - tp0) + sin tp0)) / (2 pi) = u,
// by Newton steps kept inside a shrinking bracket; s0, c0 = sin tp0, cos tp0.
// One sincos of 2 phi per step; in fast math its argument is first wrapped to
// [-pi, pi], where the hardware approximation's absolute error (~1e-6) stays
// below the 2e-6 tolerance.
template <bool FAST>
__device__ __forceinline__ void sincos_w(float a, float* s, float* c) {
  if (FAST) __sincosf(wrap_pi(a), s, c); else sincosf(a, s, c);
}
template <bool FAST>
__device__ __forceinline__ float sample_phi(float u, float beta, float s0, float c0) {
  const float target = kTwoPi * u;
  if (fabsf(beta) < 1e-6f) return target;
  float lo = 0.f, hi = kTwoPi, phi = target;
  for (int it = 0; it < 40; ++it) {
    float s2, c2;
    sincos_w<FAST>(2.f * phi, &s2, &c2);
    const float sa = s2 * c0 - c2 * s0, ca = c2 * c0 + s2 * s0;  // sin, cos (2 phi - tp0)
    const float G = phi + 0.5f * beta * (sa + s0) - target;
    if (fabsf(G) < 2e-6f) break;
    if (G > 0.f)
      hi = phi;
    else
      lo = phi;
    const float dG = 1.f + beta * ca;
    float nx = dG > 1e-6f ? phi - Math<FAST>::div(G, dG) : 0.5f * (lo + hi);
    if (!(nx > lo && nx < hi)) nx = 0.5f * (lo + hi);
    phi = nx;
  }
  return phi;
}

constexpr int kEfGuide = 1024;  // guide entries per scattering table

// The photon's path length, a sum of thousands of positive steps whose phase
// k * path needs ~1e-9 relative precision: an unevaluated float pair (TwoSum,
// then a Fast2Sum renormalisation), ~48 significant bits on the FP32 pipes.
struct PathSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float b) {
    const float t = hi + b, bp = t - hi;
    const float e = (hi - (t - bp)) + (b - bp);
    const float l = lo + e, h = t + l;
    lo = l - (h - t);
    hi = h;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__global__ void to_f32(const double* __restrict__ s, float* __restrict__ d, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    d[k] = (float)s[k];
}

// A unit vector perpendicular to u (the s direction z x u, or y for u along z).
__device__ __forceinline__ void perp_of(float ux, float uy, float uz, float& px, float& py, float& pz) {
  const float n2 = ux * ux + uy * uy;
  if (n2 < 1e-12f) {
    px = 0.f;
    py = 1.f;
    pz = 0.f;
  } else {
    const float r = rsqrtf(n2);
    px = -uy * r;
    py = ux * r;
    pz = 0.f;
  }
}

template <bool FAST>
__global__ void __launch_bounds__(256) efield_kernel(const EfParams P) {
  using M = Math<FAST>;
  extern __shared__ float s_cdf[];
  __shared__ double s_sum[kEfMaxSets * NMC_EF_FIELDS];
  for (int i = threadIdx.x; i < 2 * P.n_angles; i += blockDim.x) s_cdf[i] = P.cdf[i];
  for (int i = threadIdx.x; i < P.nsets * NMC_EF_FIELDS; i += blockDim.x) s_sum[i] = 0.0;
  // guide to the inverse-CDF search: s_guide[m][k] = the bracket start of
  // u = k / kEfGuide, so a draw's bracket search spans a few entries instead
  // of all n_angles (the same bracket, found in fewer dependent steps)
  __shared__ unsigned int s_guide[2 * (kEfGuide + 1)];
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * (kEfGuide + 1); i += blockDim.x) {
    const float* cdf = s_cdf + (i / (kEfGuide + 1)) * P.n_angles;
    const float u = (float)(i % (kEfGuide + 1)) * (1.f / kEfGuide);
    int a0 = 0, a1 = P.n_angles - 1;
    while (a1 - a0 > 1) {
      const int mid = (a0 + a1) >> 1;
      if (cdf[mid] <= u) a0 = mid; else a1 = mid;
    }
    s_guide[i] = (unsigned int)a0;
  }
  __syncthreads();
  const int MN = P.map_n * P.map_n, SN = P.sep_n * P.sep_n;

  while (true) {
    const unsigned long long g = next_photon(P.work);
    if (g >= P.total) break;
    int lo = 0, hi = P.nsets;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(P.prefix + mid) <= g) lo = mid; else hi = mid;
    }
    const int set = lo;
    const EfSet& S = P.sets[set];
    const unsigned long long pid = S.first + (g - __ldg(P.prefix + set));
    const uint32_t k1 = P.k1 + (uint32_t)set, c0 = (uint32_t)pid, c1 = (uint32_t)(pid >> 32);
    double* sm = s_sum + set * NMC_EF_FIELDS;
    atomicAdd(&sm[NMC_EF_PHOTONS], 1.0);
    atomicAdd(&sm[NMC_EF_SPECULAR], (double)(1.f - S.w0));

    float x = 0.f, y = 0.f, z = 0.f, ux = S.ux, uy = S.uy, uz = S.uz, px = S.px, py = S.py, pz = S.pz;
    float2 T00 = S.t[0], T01 = S.t[1], T10 = S.t[2], T11 = S.t[3];
    float w = S.w0, fx = 0.f, fy = 0.f, lx = 0.f, ly = 0.f;
    PathSum path;
    int med = 0;
    unsigned int nsc = 0;
    uint32_t hop = 0;
    bool alive = true, escaped = false;
    while (alive) {
      const uint4 r = philox4x32_10(make_uint4(c0, c1, hop, kEfTag), P.k0, k1);
      const EfMedium& Md = P.med[med];
      const float s = M::neglog(u01(r.x)) * Md.inv_mut;
      if (uz < 0.f && z + s * uz < 0.f) {  // reaches the surface
        const float d = -z / uz;
        x = fmaf(d, ux, x);
        y = fmaf(d, uy, y);
        z = 0.f;
        path.add(d);
        float uzt;
        const float rsp = rfresnel(P.n_medium, P.n_outside, -uz, &uzt);
        const uint4 a = philox4x32_10(make_uint4(c0, c1, hop | 0x40000000u, kEfTag), P.k0, k1);
        if (u01(a.x) > rsp) {
          escaped = true;
          break;
        }
        // mirrored; -M e_perp keeps the frame right-handed, so the perp row flips
        uz = -uz;
        px = -px;
        py = -py;
        T10 = make_float2(-T10.x, -T10.y);
        T11 = make_float2(-T11.x, -T11.y);
        const float rest = s - d;
        x = fmaf(rest, ux, x);
        y = fmaf(rest, uy, y);
        z = rest * uz;
        path.add(rest);
      } else {
        x = fmaf(s, ux, x);
        y = fmaf(s, uy, y);
        z = fmaf(s, uz, z);
        path.add(s);
      }
      w *= Md.surv;
      if (med == 0 && u01(r.w) < Md.p_raman) {  // Raman conversion
        med = 1;
        atomicAdd(&sm[NMC_EF_RAMAN_N], 1.0);
        if (P.depth) {
          const int b = (int)(z * P.depth_inv);
          if (b >= 0 && b < P.depth_bins) atomicAdd(P.depth + (size_t)set * P.depth_bins + b, (double)w);
        }
        const float ct = 2.f * u01(r.y) - 1.f, st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
        float sp, cp;
        M::sincos2pi(u01(r.z), &sp, &cp);
        ux = st * cp;
        uy = st * sp;
        uz = ct;
        perp_of(ux, uy, uz, px, py, pz);
        T00 = make_float2(1.f, 0.f);
        T01 = make_float2(0.f, 0.f);
        T10 = make_float2(0.f, 0.f);
        T11 = make_float2(1.f, 0.f);
      } else {  // scattering
        const float* cdf = s_cdf + Md.cdf_off;
        const float uth = u01(r.y);
        const unsigned int* gd = s_guide + med * (kEfGuide + 1);
        const int gk = min((int)(uth * kEfGuide), kEfGuide - 1);
        int a0 = (int)gd[gk], a1 = min((int)gd[gk + 1] + 1, P.n_angles - 1);
        while (a1 - a0 > 1) {
          const int mid = (a0 + a1) >> 1;
          if (cdf[mid] <= uth) a0 = mid; else a1 = mid;
        }
        const float q0 = cdf[a0], q1 = cdf[a1];
        const float fr = q1 > q0 ? fminf(fmaxf(M::div(uth - q0, q1 - q0), 0.f), 1.f) : 0.5f;
        const float th = ((float)a0 + fr) * P.dtheta;
        float sth, cth;
        if (FAST) __sincosf(th, &sth, &cth); else sincosf(th, &sth, &cth);
        const float4 A0 = __ldg(Md.S + a0), A1 = __ldg(Md.S + a1);
        const float2 S1 = make_float2(fmaf(fr, A1.x - A0.x, A0.x), fmaf(fr, A1.y - A0.y, A0.y));
        const float2 S2 = make_float2(fmaf(fr, A1.z - A0.z, A0.z), fmaf(fr, A1.w - A0.w, A0.w));
        // azimuth from the field: p ∝ 1 + beta cos(2 phi - 2 phi0)
        const float Pp = cnorm(T00) + cnorm(T01), Qp = cnorm(T10) + cnorm(T11);
        const float Cp = T00.x * T10.x + T00.y * T10.y + T01.x * T11.x + T01.y * T11.y;
        const float s1 = cnorm(S1), s2 = cnorm(S2), hd = 0.5f * (Pp - Qp);
        const float rho = sqrtf(hd * hd + Cp * Cp), den = (s1 + s2) * 0.5f * (Pp + Qp);
        const float beta = den > 0.f ? fminf(fmaxf(M::div((s2 - s1) * rho, den), -1.f), 1.f) : 0.f;
        const float irho = rho > 0.f ? M::rcp(rho) : 0.f;  // (cos, sin) of 2 phi0 = (hd, Cp) / rho
        const float phi = sample_phi<FAST>(u01(r.z), beta, Cp * irho, hd * irho);
        float sph, cph;
        if (FAST) __sincosf(phi, &sph, &cph); else sincosf(phi, &sph, &cph);
        // frame: e1 = cos e_par + sin e_perp, e2 = -sin e_par + cos e_perp
        const float qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;  // e_par
        const float e1x = cph * qx + sph * px, e1y = cph * qy + sph * py, e1z = cph * qz + sph * pz;
        float e2x = -sph * qx + cph * px, e2y = -sph * qy + cph * py, e2z = -sph * qz + cph * pz;
        float nux = cth * ux + sth * e1x, nuy = cth * uy + sth * e1y, nuz = cth * uz + sth * e1z;
        const float ru = rsqrtf(nux * nux + nuy * nuy + nuz * nuz);
        nux *= ru;
        nuy *= ru;
        nuz *= ru;
        const float dp = e2x * nux + e2y * nuy + e2z * nuz;
        e2x -= dp * nux;
        e2y -= dp * nuy;
        e2z -= dp * nuz;
        const float rp = rsqrtf(e2x * e2x + e2y * e2y + e2z * e2z);
        ux = nux;
        uy = nuy;
        uz = nuz;
        px = e2x * rp;
        py = e2y * rp;
        pz = e2z * rp;
        // Jones: rows of R(phi) T, then diag(S2, S1)
        const float2 b00 = make_float2(cph * T00.x + sph * T10.x, cph * T00.y + sph * T10.y);
        const float2 b01 = make_float2(cph * T01.x + sph * T11.x, cph * T01.y + sph * T11.y);
        const float2 b10 = make_float2(-sph * T00.x + cph * T10.x, -sph * T00.y + cph * T10.y);
        const float2 b11 = make_float2(-sph * T01.x + cph * T11.x, -sph * T01.y + cph * T11.y);
        T00 = cmul(S2, b00);
        T01 = cmul(S2, b01);
        T10 = cmul(S1, b10);
        T11 = cmul(S1, b11);
        const float fn = cnorm(T00) + cnorm(T01) + cnorm(T10) + cnorm(T11);
        const float sc = fn > 0.f ? (FAST ? 1.41421356f * rsqrtf(fn) : sqrtf(2.f / fn)) : 0.f;
        T00 = make_float2(T00.x * sc, T00.y * sc);
        T01 = make_float2(T01.x * sc, T01.y * sc);
        T10 = make_float2(T10.x * sc, T10.y * sc);
        T11 = make_float2(T11.x * sc, T11.y * sc);
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
      if (w < kEfRoulette) {
        const uint4 a = philox4x32_10(make_uint4(c0, c1, hop | 0x40000000u, kEfTag), P.k0, k1);
        if (u01(a.y) <= kEfChance)
          w *= 1.f / kEfChance;
        else
          alive = false;
      }
      if (++hop >= P.step_cap) {
        atomicOr(P.flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
        alive = false;
      }
    }
    atomicAdd(&sm[NMC_EF_SCATTERS], (double)nsc);
    if (!escaped) continue;

    // ---- detection: lab analysers x, y projected perpendicular to the exit direction
    const float qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;  // e_par
    float2 A[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      float ax = a == 0 ? 1.f : 0.f, ay = a == 0 ? 0.f : 1.f, az = 0.f;
      const float du = ax * ux + ay * uy;
      ax -= du * ux;
      ay -= du * uy;
      az -= du * uz;
      const float ra = rsqrtf(fmaxf(ax * ax + ay * ay + az * az, 1e-20f));
      const float cpar = (ax * qx + ay * qy + az * qz) * ra, cperp = (ax * px + ay * py + az * pz) * ra;
      A[a][0] = make_float2(T00.x * cpar + T10.x * cperp, T00.y * cpar + T10.y * cperp);
      A[a][1] = make_float2(T01.x * cpar + T11.x * cperp, T01.y * cpar + T11.y * cperp);
    }
    const float ex = S.ex, ey = S.ey;
    // fields of input e in the analysers x, y; co = e.(A e), cross = e_perp.(A e)
    const float2 Fx = make_float2(A[0][0].x * ex + A[0][1].x * ey, A[0][0].y * ex + A[0][1].y * ey);
    const float2 Fy = make_float2(A[1][0].x * ex + A[1][1].x * ey, A[1][0].y * ex + A[1][1].y * ey);
    const float2 Eco = make_float2(ex * Fx.x + ey * Fy.x, ex * Fx.y + ey * Fy.y);
    const float2 Ecr = make_float2(-ey * Fx.x + ex * Fy.x, -ey * Fx.y + ex * Fy.y);
    const float Ico = w * cnorm(Eco), Icr = w * cnorm(Ecr);
    if (med == 1) {
      atomicAdd(&sm[NMC_EF_RAMAN_RD], (double)w);
      atomicAdd(&sm[NMC_EF_RAMAN_CO], (double)Ico);
      atomicAdd(&sm[NMC_EF_RAMAN_CROSS], (double)Icr);
      continue;
    }
    atomicAdd(&sm[NMC_EF_RD], (double)w);
    atomicAdd(&sm[NMC_EF_RD2], (double)w * (double)w);
    atomicAdd(&sm[NMC_EF_CO], (double)Ico);
    atomicAdd(&sm[NMC_EF_CROSS], (double)Icr);
    if (nsc >= 2) {
      // time-reversed partner: the transposed lab-frame amplitude, so the
      // co channel e.(A e) is its own partner and the cross channel pairs
      // e_perp.(A e) with e.(A e_perp)
      const float2 Gx = make_float2(-A[0][0].x * ey + A[0][1].x * ex, -A[0][0].y * ey + A[0][1].y * ex);
      const float2 Gy = make_float2(-A[1][0].x * ey + A[1][1].x * ex, -A[1][0].y * ey + A[1][1].y * ex);
      const float2 Ecr_r = make_float2(ex * Gx.x + ey * Gy.x, ex * Gx.y + ey * Gy.y);
      const float2 cco = make_float2(cnorm(Eco), 0.f), ccr = cmulc(Ecr, Ecr_r);
      atomicAdd(&sm[NMC_EF_MULTI_CO], (double)Ico);
      atomicAdd(&sm[NMC_EF_MULTI_CROSS], (double)Icr);
      atomicAdd(&sm[NMC_EF_INTERF_CO], (double)(w * cco.x));
      atomicAdd(&sm[NMC_EF_INTERF_CROSS], (double)(w * ccr.x));
      if (P.sep) {
        const int i = (int)floorf((lx - fx + P.sep_half) * P.sep_inv);
        const int j = (int)floorf((ly - fy + P.sep_half) * P.sep_inv);
        if (i >= 0 && i < P.sep_n && j >= 0 && j < P.sep_n) {
          double* h0 = P.sep + (((size_t)set * 2) * SN + (size_t)i * P.sep_n + j) * 2;
          double* h1 = h0 + (size_t)SN * 2;
          atomicAdd(h0, (double)(w * cco.x));
          atomicAdd(h0 + 1, (double)(w * cco.y));
          atomicAdd(h1, (double)(w * ccr.x));
          atomicAdd(h1 + 1, (double)(w * ccr.y));
        } else {
          atomicAdd(&sm[NMC_EF_SEP_OUTSIDE], (double)(w * cco.x));
        }
      }
    }
    const float Ixx = w * cnorm(A[0][0]), Ixy = w * cnorm(A[1][0]), Iyx = w * cnorm(A[0][1]),
                Iyy = w * cnorm(A[1][1]);  // input x/y, analyser x/y
    if (P.pvs) {
      double* v = P.pvs + (size_t)set * 4 * (NMC_EF_MAX_ORDER + 1) + min(nsc, (unsigned)NMC_EF_MAX_ORDER);
      atomicAdd(v, (double)Ixx);
      atomicAdd(v + (NMC_EF_MAX_ORDER + 1), (double)Ixy);
      atomicAdd(v + 2 * (NMC_EF_MAX_ORDER + 1), (double)Iyx);
      atomicAdd(v + 3 * (NMC_EF_MAX_ORDER + 1), (double)Iyy);
    }
    if (P.maps) {
      const int ix = (int)floorf(x * P.map_inv + 0.5f * P.map_n), iy = (int)floorf(y * P.map_inv + 0.5f * P.map_n);
      if (ix >= 0 && ix < P.map_n && iy >= 0 && iy < P.map_n) {
        double* m = P.maps + (size_t)set * NMC_EF_MAPS * MN + (size_t)ix * P.map_n + iy;
        const float ph_path = (float)fmod(path.value() * (double)P.med[0].kmed, 6.283185307179586);
        const float a_co = atan2f(Eco.y, Eco.x), a_cr = atan2f(Ecr.y, Ecr.x);
        atomicAdd(m + NMC_EF_MAP_XX * (size_t)MN, (double)Ixx);
        atomicAdd(m + NMC_EF_MAP_XY * (size_t)MN, (double)Ixy);
        atomicAdd(m + NMC_EF_MAP_YX * (size_t)MN, (double)Iyx);
        atomicAdd(m + NMC_EF_MAP_YY * (size_t)MN, (double)Iyy);
        atomicAdd(m + NMC_EF_MAP_RD * (size_t)MN, (double)w);
        atomicAdd(m + NMC_EF_MAP_DET * (size_t)MN, 1.0);
        atomicAdd(m + NMC_EF_MAP_PHASE0 * (size_t)MN, (double)a_co);
        atomicAdd(m + NMC_EF_MAP_PHASE1 * (size_t)MN, (double)wrap_pi(ph_path));
        atomicAdd(m + NMC_EF_MAP_PHASE2 * (size_t)MN, (double)a_cr);
        atomicAdd(m + NMC_EF_MAP_PHASE3 * (size_t)MN, (double)wrap_pi(a_co + ph_path));
        if (P.spk) {  // the pixel's speckle record (struct SPECKLE, definitions.h:220-229)
          const size_t pix = (size_t)ix * P.map_n + iy;
          const int k = atomicAdd(P.spk_count + (size_t)set * MN + pix, 1);
          if (k < (int)P.spk_max)
            P.spk[((size_t)set * P.spk_max + k) * MN + pix] =
                nmc_speckle{a_co, wrap_pi(ph_path), a_cr, wrap_pi(a_co + ph_path), Ixx, Ixy, w};
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < P.nsets * NMC_EF_FIELDS; i += blockDim.x)
    if (s_sum[i] != 0.0) atomicAdd(P.sums + i, s_sum[i]);
}

// ---- CBS cone: two complex matrix products (the 2-D Fourier sum of the
// separation histogram on the angular grid).
//   W[i][a] = exp(i k0 sin(theta_i) rho_a),  T1 = W H  (cone_n x sep_n),  C = T1 W^T.
__global__ void twiddle_kernel(float2* W, int rows, int cols, float k0, float th_half, float rho_half) {
  const int n = rows * cols;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = t / cols, a = t % cols;
    const double th = -th_half + (i + 0.5) * (2.0 * th_half / rows);
    const double rho = -rho_half + (a + 0.5) * (2.0 * rho_half / cols);
    const double ph = fmod((double)k0 * sin(th) * rho, 6.283185307179586);
    double sv, cv;
    sincos(ph, &sv, &cv);
    W[t] = make_float2((float)cv, (float)sv);
  }
}

// C[M x N] = A[M x K] B[K x N] (complex, row-major; B transposed when TB:
// B[n][k]), 16 x 16 tiles through shared memory.
template <bool TB>
__global__ void cgemm_kernel(const float2* __restrict__ A, const float2* __restrict__ B, float2* __restrict__ C,
                             int Mr, int N, int K) {
  __shared__ float2 sa[16][17], sb[16][17];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
  float2 acc = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < K; k0 += 16) {
    sa[ty][tx] = (row < Mr && k0 + tx < K) ? A[(size_t)row * K + k0 + tx] : make_float2(0.f, 0.f);
    const int kb = k0 + ty;
    float2 bv = make_float2(0.f, 0.f);
    if (kb < K && col < N) bv = TB ? B[(size_t)col * K + kb] : B[(size_t)kb * N + col];
    sb[ty][tx] = bv;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float2 a = sa[ty][k], b = sb[k][tx];
      acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
      acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
    }
    __syncthreads();
  }
  if (row < Mr && col < N) C[(size_t)row * N + col] = acc;
}

// ---- the reference's speckle mutual interference (MetalMC.m:628-742), one
// thread per pixel, its records in order.  The variable types follow the
// reference: float quantities, double sin / cos / atan2 / exp / sqrt of
// them (C's math functions of float arguments) and double constants.
__device__ __forceinline__ float keep_finite(float v) { return isfinite(v) ? v : 0.0f; }
__device__ __forceinline__ float wrap_ref(float a) { return (float)atan2(sin((double)a), cos((double)a)); }

__global__ void speckle_mutual_kernel(int npix, const float* __restrict__ maps, const nmc_speckle* __restrict__ rec,
                                      const int* __restrict__ counts, int kmax, float lambda, float lc,
                                      float* __restrict__ out) {
  const double two = 2.0, pi_ref = 3.1415926;  // MC_TWO, PI (definitions.h:60,77)
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const float xx_t = maps[NMC_EF_MAP_XX * (size_t)npix + p], xy_t = maps[NMC_EF_MAP_XY * (size_t)npix + p];
    const float norm = xx_t + xy_t;
    const float ndet = maps[NMC_EF_MAP_DET * (size_t)npix + p];
    const float xx_a = keep_finite(norm > 0.0f ? xx_t / norm : 0.0f);
    const float xy_a = keep_finite(norm > 0.0f ? xy_t / norm : 0.0f);
    const float ryx_a = keep_finite(maps[NMC_EF_MAP_RD * (size_t)npix + p] / ndet);
    const float ph_a = keep_finite(maps[NMC_EF_MAP_PHASE0 * (size_t)npix + p] / ndet);
    const float path_a = keep_finite(maps[NMC_EF_MAP_PHASE1 * (size_t)npix + p] / ndet);
    const float sc_a = keep_finite(maps[NMC_EF_MAP_PHASE2 * (size_t)npix + p] / ndet);
    const float tot_a = keep_finite(maps[NMC_EF_MAP_PHASE3 * (size_t)npix + p] / ndet);
    float xx_m = xx_a, xy_m = xy_a, ryx_m = ryx_a, ph_m = ph_a, path_m = path_a, sc_m = sc_a, tot_m = tot_a;
    float n_times = 1.0f;
    const float path_a_mm = (float)((double)(path_a * lambda) / (two * pi_ref));
    const int K = min(counts[p], kmax);
    for (int k = 0; k < K; ++k) {
      const nmc_speckle r = rec[(size_t)k * npix + p];
      const float nc = r.XX + r.XY;
      const float xx_c = keep_finite(nc > 0.0f ? r.XX / nc : 0.0f);
      const float xy_c = keep_finite(nc > 0.0f ? r.XY / nc : 0.0f);
      const float ryx_c = keep_finite(r.Ryx);
      const float ph_c = keep_finite(r.Phase), path_c = keep_finite(r.Path), sc_c = keep_finite(r.Scatt);
      const float d_path = wrap_ref(path_a - path_c), d_sc = wrap_ref(sc_a - sc_c);
      const float diff_lin = wrap_ref(d_path + d_sc);
      const float interf = (float)sin((double)diff_lin);
      const float path_c_mm = (float)((double)(path_c * lambda) / (two * pi_ref));
      const float dp = (path_c_mm - path_a_mm) / lc;
      float env = (float)exp((double)(-dp * dp));
      env = (!isfinite(env) || lc <= 0.01f) ? 0.0f : env;
      xx_m += (float)(((double)(xx_a + xx_c) + two * sqrt((double)(xx_a * xx_c)) * interf * env) / 4.0f);
      xy_m += (float)(((double)(xy_a + xy_c) + two * sqrt((double)(xy_a * xy_c)) * interf * env) / 4.0f);
      ryx_m += (float)(((double)(ryx_a + ryx_c) + two * sqrt((double)(ryx_a * ryx_c)) * interf * env) / 4.0f);
      ph_m += ph_c;
      path_m += path_c;
      sc_m += sc_c;
      tot_m += wrap_ref(ph_c + path_c + sc_c);
      n_times += 1.0f;
    }
    out[NMC_EF_MAP_RD * (size_t)npix + p] += ryx_m;
    out[NMC_EF_MAP_DET * (size_t)npix + p] += n_times;
    out[NMC_EF_MAP_XX * (size_t)npix + p] += xx_m;
    out[NMC_EF_MAP_XY * (size_t)npix + p] += xy_m;
    out[NMC_EF_MAP_PHASE0 * (size_t)npix + p] += ph_m;
    out[NMC_EF_MAP_PHASE1 * (size_t)npix + p] += path_m;
    out[NMC_EF_MAP_PHASE2 * (size_t)npix + p] += sc_m;
    out[NMC_EF_MAP_PHASE3 * (size_t)npix + p] += tot_m;
  }
}

cudaError_t cgemm(const float2* A, const float2* B, float2* C, int Mr, int N, int K, bool tb, cudaStream_t st) {
  const dim3 blk(16, 16), grd((N + 15) / 16, (Mr + 15) / 16);
  if (tb)
    cgemm_kernel<true><<<grd, blk, 0, st>>>(A, B, C, Mr, N, K);
  else
    cgemm_kernel<false><<<grd, blk, 0, st>>>(A, B, C, Mr, N, K);
  return cudaGetLastError();
}

double host_rfresnel(double n1, double n2, double ca1) {  // unpolarised, as helpers.metal:243-291
  if (n1 == n2) return 0.0;
  if (ca1 > 1.0 - 1e-12) {
    const double r = (n2 - n1) / (n2 + n1);
    return r * r;
  }
  if (ca1 < 1e-6) return 1.0;
  const double sa1 = std::sqrt(1.0 - ca1 * ca1), sa2 = n1 * sa1 / n2;
  if (sa2 >= 1.0) return 1.0;
  const double ca2 = std::sqrt(1.0 - sa2 * sa2);
  const double cap = ca1 * ca2 - sa1 * sa2, cam = ca1 * ca2 + sa1 * sa2;
  const double sap = sa1 * ca2 + ca1 * sa2, sam = sa1 * ca2 - ca1 * sa2;
  return 0.5 * sam * sam * (cam * cam + cap * cap) / (sap * sap * cam * cam);
}

bool build_cdf(const float* S, int n, std::vector<float>& cdf) {
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

}  // namespace
}  // namespace nmc

extern "C" nmc_status nmc_efield_run(int32_t device, const nmc_efield_config* cfg, const float* S_primary,
                                     const float* S_raman, const nmc_efield_setting* settings, int32_t n_settings,
                                     double* out, float* cone, double* pol_vs_scatt, float* maps,
                                     double* raman_depth, nmc_speckle* speckles, int32_t* speckle_counts) {
  using namespace nmc;
  if (!cfg || !S_primary || !settings || !out) return NMC_EINVAL;
  const nmc_efield_config& c = *cfg;
  if (n_settings < 1 || n_settings > kEfMaxSets) return NMC_EINVAL;
  const float vals[] = {c.mua, c.mus, c.wavelength_cm, c.n_medium, c.n_outside, c.mu_raman};
  for (float v : vals)
    if (!std::isfinite(v) || v < 0.f) return NMC_EINVAL;
  if (!(c.mua + c.mus > 0.f) || !(c.wavelength_cm > 0.f) || !(c.n_medium > 0.f) || !(c.n_outside > 0.f))
    return NMC_EINVAL;
  if (c.n_angles < 2 || c.n_angles > 100000) return NMC_EINVAL;
  if (c.mu_raman > 0.f && (!S_raman || !(c.raman_mua >= 0.f) || !(c.raman_mus >= 0.f) ||
                           !(c.raman_mua + c.raman_mus > 0.f) || !(c.raman_wavelength_cm > 0.f)))
    return NMC_EINVAL;
  if (cone && (c.cone_n < 2 || c.cone_n > 1024 || !(c.cone_half_angle > 0.f) || c.sep_n < 2 || c.sep_n > 4096 ||
               !(c.sep_half_width > 0.f)))
    return NMC_EINVAL;
  if (maps && (c.map_n < 1 || c.map_n > 1024 || !(c.map_dx > 0.f))) return NMC_EINVAL;
  if (raman_depth && (c.depth_bins < 1 || c.depth_bins > 4096 || !(c.depth_dz > 0.f))) return NMC_EINVAL;
  const int n = c.n_angles;
  std::vector<float> cdf0, cdf1;
  if (!build_cdf(S_primary, n, cdf0)) return NMC_EINVAL;
  const bool raman = c.mu_raman > 0.f;
  if (raman && !build_cdf(S_raman, n, cdf1)) return NMC_EINVAL;
  if (!raman) cdf1 = cdf0;
  std::vector<float> cdf(2 * n);
  std::copy(cdf0.begin(), cdf0.end(), cdf.begin());
  std::copy(cdf1.begin(), cdf1.end(), cdf.begin() + n);

  std::vector<EfSet> sets(n_settings);
  std::vector<unsigned long long> prefix(n_settings + 1, 0ull);
  for (int s = 0; s < n_settings; ++s) {
    const nmc_efield_setting& q = settings[s];
    if (!std::isfinite(q.pol_angle) || !std::isfinite(q.theta_in) || !std::isfinite(q.phi_in) ||
        q.theta_in < 0.f || q.theta_in >= 1.5707963f)
      return NMC_EINVAL;
    EfSet& d = sets[s];
    d = EfSet{};
    d.ex = std::cos(q.pol_angle);
    d.ey = std::sin(q.pol_angle);
    const double st = std::sin((double)q.theta_in) * c.n_outside / c.n_medium;
    const double ct = std::sqrt(1.0 - st * st);
    const double ux = st * std::cos((double)q.phi_in), uy = st * std::sin((double)q.phi_in), uz = ct;
    d.ux = (float)ux;
    d.uy = (float)uy;
    d.uz = (float)uz;
    double px, py, pz;
    if (st < 1e-9) {
      px = 0.0;
      py = 1.0;
      pz = 0.0;
    } else {  // s direction z x u
      const double r = 1.0 / std::sqrt(ux * ux + uy * uy);
      px = -uy * r;
      py = ux * r;
      pz = 0.0;
    }
    d.px = (float)px;
    d.py = (float)py;
    d.pz = (float)pz;
    const double qx = py * uz - pz * uy, qy = pz * ux - px * uz, qz = px * uy - py * ux;  // e_par
    double t[2][2], f = 0.0;
    for (int b = 0; b < 2; ++b) {
      double bx = b == 0 ? 1.0 : 0.0, by = b == 0 ? 0.0 : 1.0, bz = 0.0;
      const double du = bx * ux + by * uy + bz * uz;
      bx -= du * ux;
      by -= du * uy;
      bz -= du * uz;
      t[0][b] = bx * qx + by * qy + bz * qz;
      t[1][b] = bx * px + by * py + bz * pz;
      f += t[0][b] * t[0][b] + t[1][b] * t[1][b];
    }
    const double sc = std::sqrt(2.0 / f);
    d.t[0] = make_float2((float)(t[0][0] * sc), 0.f);
    d.t[1] = make_float2((float)(t[0][1] * sc), 0.f);
    d.t[2] = make_float2((float)(t[1][0] * sc), 0.f);
    d.t[3] = make_float2((float)(t[1][1] * sc), 0.f);
    d.w0 = (float)(1.0 - host_rfresnel(c.n_outside, c.n_medium, std::cos((double)q.theta_in)));
    d.first = 0;
    // photon counts are summed in FP64: keep the whole run exact there
    if (q.photons > (1ull << 53) - prefix[s]) return NMC_EINVAL;
    prefix[s + 1] = prefix[s] + q.photons;
  }
  nmc::DeviceScope dev(device);
  if (!dev.ok) return NMC_EDEVICE;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NMC_EDEVICE;
  std::vector<void*> allocs;
  auto dalloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (bytes == 0) return nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    cudaMemsetAsync(p, 0, bytes, st);
    return p;
  };
  auto done = [&](nmc_status s) {
    cudaStreamSynchronize(st);
    for (void* p : allocs) cudaFree(p);
    cudaStreamDestroy(st);
    return s;
  };
  const size_t ns = n_settings, SN = (size_t)c.sep_n * c.sep_n, MN = (size_t)c.map_n * c.map_n;
  float4* dS0 = (float4*)dalloc(sizeof(float4) * n);
  float4* dS1 = (float4*)dalloc(sizeof(float4) * n);
  float* dcdf = (float*)dalloc(sizeof(float) * 2 * n);
  EfSet* dsets = (EfSet*)dalloc(sizeof(EfSet) * ns);
  unsigned long long* dpre = (unsigned long long*)dalloc(8 * (ns + 1));
  double* dsums = (double*)dalloc(sizeof(double) * ns * NMC_EF_FIELDS);
  unsigned long long* dwork = (unsigned long long*)dalloc(16);
  double* dsep_d = cone ? (double*)dalloc(sizeof(double) * 2 * 2 * SN * ns) : nullptr;
  float* dsep = cone ? (float*)dalloc(sizeof(float) * 2 * 2 * SN * ns) : nullptr;
  double* dpvs = pol_vs_scatt ? (double*)dalloc(sizeof(double) * 4 * (NMC_EF_MAX_ORDER + 1) * ns) : nullptr;
  double* dmaps_d = maps ? (double*)dalloc(sizeof(double) * NMC_EF_MAPS * MN * ns) : nullptr;
  float* dmaps = maps ? (float*)dalloc(sizeof(float) * NMC_EF_MAPS * MN * ns) : nullptr;
  double* ddepth = raman_depth ? (double*)dalloc(sizeof(double) * c.depth_bins * ns) : nullptr;
  const bool spk = maps && c.speckle_max > 0 && (speckles || speckle_counts);
  if (spk && c.speckle_max > 100000u) return done(NMC_EINVAL);
  nmc_speckle* dspk = spk ? (nmc_speckle*)dalloc(sizeof(nmc_speckle) * c.speckle_max * MN * ns) : nullptr;
  int* dspkc = spk ? (int*)dalloc(sizeof(int) * MN * ns) : nullptr;
  if (!dS0 || !dS1 || !dcdf || !dsets || !dpre || !dsums || !dwork || (cone && (!dsep || !dsep_d)) ||
      (pol_vs_scatt && !dpvs) || (maps && (!dmaps || !dmaps_d)) || (raman_depth && !ddepth) || (spk && (!dspk || !dspkc)))
    return done(NMC_ENOMEM);
  if (cudaMemcpyAsync(dS0, S_primary, sizeof(float4) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dS1, raman ? S_raman : S_primary, sizeof(float4) * n, cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(dcdf, cdf.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dsets, sets.data(), sizeof(EfSet) * ns, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dpre, prefix.data(), 8 * (ns + 1), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return done(NMC_EDEVICE);

  EfParams P{};
  const double mut0 = (double)c.mua + c.mus + c.mu_raman;
  P.med[0].inv_mut = (float)(1.0 / mut0);
  P.med[0].surv = (float)((c.mus + c.mu_raman) / mut0);
  P.med[0].p_raman = (c.mus + c.mu_raman) > 0.f ? (float)(c.mu_raman / ((double)c.mus + c.mu_raman)) : 0.f;
  P.med[0].kmed = (float)(2.0 * 3.14159265358979323846 * c.n_medium / c.wavelength_cm);
  P.med[0].S = dS0;
  P.med[0].cdf_off = 0;
  const double mut1 = raman ? (double)c.raman_mua + c.raman_mus : mut0;
  P.med[1].inv_mut = (float)(1.0 / mut1);
  P.med[1].surv = raman ? (float)(c.raman_mus / mut1) : P.med[0].surv;
  P.med[1].p_raman = 0.f;
  P.med[1].kmed = raman ? (float)(2.0 * 3.14159265358979323846 * c.n_medium / c.raman_wavelength_cm)
                        : P.med[0].kmed;
  P.med[1].S = dS1;
  P.med[1].cdf_off = n;
  P.cdf = dcdf;
  P.n_angles = n;
  P.dtheta = (float)(3.14159265358979323846 / (n - 1));
  P.n_medium = c.n_medium;
  P.n_outside = c.n_outside;
  P.sets = dsets;
  P.prefix = dpre;
  P.nsets = n_settings;
  P.total = prefix[ns];
  P.k0 = (uint32_t)c.seed;
  P.k1 = (uint32_t)(c.seed >> 32);
  P.sums = dsums;
  P.sep = dsep_d;
  P.sep_n = c.sep_n;
  P.sep_inv = cone ? (float)(c.sep_n / (2.0 * c.sep_half_width)) : 0.f;
  P.sep_half = c.sep_half_width;
  P.pvs = dpvs;
  P.maps = dmaps_d;
  P.map_n = maps ? c.map_n : 1;
  P.map_inv = maps ? (float)(1.0 / c.map_dx) : 0.f;
  P.depth = ddepth;
  P.depth_bins = c.depth_bins;
  P.depth_inv = raman_depth ? (float)(1.0 / c.depth_dz) : 0.f;
  P.work = dwork;
  P.flags = (unsigned int*)(dwork + 1);
  P.step_cap = 20000000u;
  P.spk = dspk;
  P.spk_count = dspkc;
  P.spk_max = spk ? c.speckle_max : 0u;

  const bool fast = !(c.flags & NMC_FLAG_PRECISE_MATH);
  const void* f = fast ? (const void*)efield_kernel<true> : (const void*)efield_kernel<false>;
  const size_t smem = sizeof(float) * 2 * n;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                              cudaSuccess)
    return done(NMC_EINVAL);
  int per_sm = 0, nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, 256, smem) != cudaSuccess || per_sm < 1)
    return done(NMC_EDEVICE);
  const unsigned long long grid =
      std::max<unsigned long long>(1, std::min<unsigned long long>((unsigned long long)nsm * per_sm,
                                                                   (P.total + 255) / 256));
  void* args[] = {(void*)&P};
  if (P.total > 0 && cudaLaunchKernel(f, dim3((unsigned)grid), dim3(256), args, smem, st) != cudaSuccess)
    return done(NMC_EDEVICE);
  if (cone) to_f32<<<1024, 256, 0, st>>>(dsep_d, dsep, 2 * 2 * SN * ns);
  if (maps) to_f32<<<1024, 256, 0, st>>>(dmaps_d, dmaps, NMC_EF_MAPS * MN * ns);
  if (cone) {  // the 2-D Fourier sums, per setting and channel
    const int cn = c.cone_n, sn = c.sep_n;
    float2* W = (float2*)dalloc(sizeof(float2) * cn * sn);
    float2* T1 = (float2*)dalloc(sizeof(float2) * cn * sn);
    float2* dcone = (float2*)dalloc(sizeof(float2) * cn * cn * 2 * ns);
    if (!W || !T1 || !dcone) return done(NMC_ENOMEM);
    const float k0 = (float)(2.0 * 3.14159265358979323846 / c.wavelength_cm);
    twiddle_kernel<<<1024, 256, 0, st>>>(W, cn, sn, k0, c.cone_half_angle, c.sep_half_width);
    for (size_t s = 0; s < ns; ++s)
      for (int ch = 0; ch < 2; ++ch) {
        const float2* H = (const float2*)dsep + (s * 2 + ch) * SN;
        float2* C = dcone + (s * 2 + ch) * (size_t)cn * cn;
        if (cgemm(W, H, T1, cn, sn, sn, false, st) != cudaSuccess ||  // rows: theta_x
            cgemm(T1, W, C, cn, cn, sn, true, st) != cudaSuccess)     // columns: theta_y
          return done(NMC_EDEVICE);
      }
    if (cudaMemcpyAsync(cone, dcone, sizeof(float2) * cn * cn * 2 * ns, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return done(NMC_EDEVICE);
  }
  if (cudaMemcpyAsync(out, dsums, sizeof(double) * ns * NMC_EF_FIELDS, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      (pol_vs_scatt && cudaMemcpyAsync(pol_vs_scatt, dpvs, sizeof(double) * 4 * (NMC_EF_MAX_ORDER + 1) * ns,
                                       cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
      (maps && cudaMemcpyAsync(maps, dmaps, sizeof(float) * NMC_EF_MAPS * MN * ns, cudaMemcpyDeviceToHost, st) !=
                   cudaSuccess) ||
      (raman_depth && cudaMemcpyAsync(raman_depth, ddepth, sizeof(double) * c.depth_bins * ns,
                                      cudaMemcpyDeviceToHost, st) != cudaSuccess))
    return done(NMC_EDEVICE);
  if (spk && ((speckles && cudaMemcpyAsync(speckles, dspk, sizeof(nmc_speckle) * c.speckle_max * MN * ns,
                                           cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
              (speckle_counts &&
               cudaMemcpyAsync(speckle_counts, dspkc, sizeof(int) * MN * ns, cudaMemcpyDeviceToHost, st) !=
                   cudaSuccess)))
    return done(NMC_EDEVICE);
  unsigned int flags = 0;
  cudaMemcpyAsync(&flags, P.flags, sizeof flags, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return done(NMC_EDEVICE);
  if (spk && speckle_counts)  // arrivals -> records kept
    for (size_t k = 0; k < MN * ns; ++k) speckle_counts[k] = std::min<int32_t>(speckle_counts[k], (int32_t)c.speckle_max);
  return done((flags & NMC_DEVFLAG_STEPCAP) ? NMC_ESTEPCAP : NMC_OK);
}

extern "C" nmc_status nmc_speckle_mutual(int32_t device, int32_t nx, int32_t ny, const float* maps,
                                         const nmc_speckle* records, const int32_t* counts, int32_t max_records,
                                         float lambda, float lc, float* out_maps) {
  using namespace nmc;
  if (!maps || !counts || !out_maps || (max_records > 0 && !records)) return NMC_EINVAL;
  if (nx < 1 || ny < 1 || (size_t)nx * ny > (1u << 24) || max_records < 0 || max_records > 100000 ||
      !std::isfinite(lambda) || !std::isfinite(lc))
    return NMC_EINVAL;
  const size_t np = (size_t)nx * ny, nm = (size_t)NMC_EF_MAPS * np, nr = (size_t)max_records * np;
  nmc::DeviceScope dev(device);
  if (!dev.ok) return NMC_EDEVICE;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NMC_EDEVICE;
  float *dm = nullptr, *dout = nullptr;
  nmc_speckle* dr = nullptr;
  int* dc = nullptr;
  auto done = [&](nmc_status s) {
    cudaStreamSynchronize(st);
    cudaFree(dm);
    cudaFree(dout);
    cudaFree(dr);
    cudaFree(dc);
    cudaStreamDestroy(st);
    return s;
  };
  if (cudaMalloc((void**)&dm, nm * 4) != cudaSuccess || cudaMalloc((void**)&dout, nm * 4) != cudaSuccess ||
      cudaMalloc((void**)&dc, np * 4) != cudaSuccess ||
      (nr && cudaMalloc((void**)&dr, nr * sizeof(nmc_speckle)) != cudaSuccess))
    return done(NMC_ENOMEM);
  if (cudaMemcpyAsync(dm, maps, nm * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dout, out_maps, nm * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dc, counts, np * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      (nr && cudaMemcpyAsync(dr, records, nr * sizeof(nmc_speckle), cudaMemcpyHostToDevice, st) != cudaSuccess))
    return done(NMC_EDEVICE);
  const int grid = (int)std::min<size_t>((np + 127) / 128, 65535);
  speckle_mutual_kernel<<<grid, 128, 0, st>>>((int)np, dm, dr, dc, max_records, lambda, lc, dout);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(out_maps, dout, nm * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return done(NMC_EDEVICE);
  return done(NMC_OK);
}
