// layered.cu - multi-layer extension of the mcsub kernel: a stack of plane
// layers, each with its own mua, mus, HG g, refractive index and thickness
// (the last may be semi-infinite), between an ambient medium above and one
// below.  The reference declares MAXLAYERS = 100 (definitions.h:24) but its
// mcsub kernel (kernels.metal:59-319) has one semi-infinite layer; this
// kernel keeps that kernel's physics per layer:
//   HOP    s = -ln(xi) / mu_t of the current layer; a step that reaches a
//          layer boundary stops there and the rest of the dimensionless
//          step carries into the next layer (scaled by its mu_t);
//   CROSS  at a boundary the photon reflects with the unpolarised Fresnel
//          probability R(n_i, n_t, |uz|) (helpers.metal:243-291) by a random
//          draw, as the mcsub kernel does at its surface (kernels.metal:
//          183-214); otherwise it refracts (Snell) into the next layer, or
//          escapes into the ambient medium (Rd(r) above, Tt(r) below);
//   DROP   absorb = W mua / mu_t at each interaction (kernels.metal:224-234),
//          tallied in A(z), A(r, z) and per layer;
//   SPIN   Henyey-Greenstein with the layer's g (the reference's mcsub
//          kernel samples isotropically, kernels.metal:252; this kernel uses
//          the g it is given);
//   ROULETTE below 1e-4, chance 0.1 (kernels.metal:289-294).
// A launch is a normal pencil beam at the origin; the specular reflection
// at the top surface leaves W0 = 1 - R_sp.  Random numbers: Philox4x32-10,
// key (seed lo, seed hi), counter (photon lo, photon hi, interaction,
// 'LAYR'): x step, y cos theta, z psi, w roulette; boundary events draw their
// Fresnel choice from counter (photon lo, photon hi, event | 2^31, 'LAYR').
// With NMC_FLAG_LAYERED_REF_STREAMS the draws come from the reference's
// generator in MCSubKernel's order instead (seeding kernels.metal:91-95; a
// launch draw :113, then per hop the step :183, the Fresnel choice :191,
// cos theta :244, psi :255, the roulette draw :290), and with
// NMC_FLAG_LAYERED_ISOTROPIC cos theta = 2 xi - 1 as the reference samples
// it (:252): one semi-infinite layer then replays MCSubKernel's photons.
//
// Adjoint (ADJ): a photon scores once, when it escapes (G_rd[r bin] or
// G_tt[r bin] times its weight), so the per-layer derivatives of the loss
// accumulate directly from per-photon sums kept per layer: the geometric path
// L_l, the interactions n_l and Q_l = sum d ln p_HG(cos; g_l)/dg.  With
// implicit capture (weight x mus/mu_t per interaction, paths sampled with
// mu_t) the likelihood ratio of the path and the weight's own derivative give
//   d score/d mua_l = -score L_l,
//   d score/d mus_l = score (n_l / mus_l - L_l),
//   d score/d g_l   = score Q_l.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"
#include "nmc_abi.h"

namespace nmc {
namespace {

constexpr uint32_t kLayTag = 0x4C415952u;
constexpr int kMaxLayers = 100;  // MAXLAYERS, definitions.h:24
constexpr int kMaxAdjLayers = 16;  // per-photon sums of the adjoint live in local memory

__device__ __forceinline__ float dln_hg_dg(float g, float mu) {  // p = (1-g^2)/(2 (1+g^2-2g mu)^1.5)
  return -2.f * g / (1.f - g * g) - 3.f * (g - mu) / (1.f + g * g - 2.f * g * mu);
}

struct LayDev {
  float mua, mus, inv_mut, n, z0, z1;  // z1 = +inf for a semi-infinite last layer
  float g;
  PhaseConst ph;
};

struct LayParams {
  const LayDev* lay;
  int nl;
  float n_above, n_below, w0;
  int nr, nz;
  float idr, idz;
  unsigned long long* rd_r;  // nr + 1 (last = overflow), u64 fixed point
  unsigned long long* tt_r;  // nr + 1
  unsigned long long* a_z;   // nz + 1
  unsigned long long* a_rz;  // (nr + 1) * (nz + 1), or null
  unsigned long long* a_layer;  // nl
  int smem_az;   // A(z) privatised in shared memory (nz + 1 bins after the layer sums)
  double* sums;  // NMC_LAY_FIELDS
  unsigned long long first, n;
  uint32_t k0, k1;
  uint32_t rk[20];  // Philox round keys of (k0, k1)
  unsigned long long* work;
  unsigned int* flags;
  uint32_t step_cap;
  // adjoint
  const float* g_rd;  // nr + 1 upstream gradient of rd_r (may be null)
  const float* g_tt;  // nr + 1 upstream gradient of tt_r (may be null)
  double* grad;       // 3 * nl: d/dmua, d/dmus, d/dg
  // reference streams (REF kernels): photon p = (run p / batch + 1, index p % batch)
  unsigned long long batch;
  int iso;            // isotropic scattering (the reference's mcsub sampling)
};

template <bool FAST, bool ADJ, bool REF>
__global__ void __launch_bounds__(256) layered_kernel(const LayParams P) {
  using M = Math<FAST>;
  __shared__ LayDev s_lay[kMaxLayers];
  __shared__ double s_sum[NMC_LAY_FIELDS];
  __shared__ double s_grad[ADJ ? 3 * kMaxAdjLayers : 1];
  // absorbed weight per layer, then (if it fits) A(z): block-private u64
  // fixed-point sums, added to the global tallies once at the end; every
  // interaction deposits, and a handful of global addresses would serialise
  extern __shared__ unsigned long long s_tally[];
  unsigned long long* const s_al = s_tally;
  unsigned long long* const s_az = s_tally + P.nl;
  const int n_priv = P.nl + (P.smem_az ? P.nz + 1 : 0);
  for (int i = threadIdx.x; i < n_priv; i += blockDim.x) s_tally[i] = 0ull;
  for (int i = threadIdx.x; i < P.nl; i += blockDim.x) s_lay[i] = P.lay[i];
  if (threadIdx.x < NMC_LAY_FIELDS) s_sum[threadIdx.x] = 0.0;
  if (ADJ)
    for (int i = threadIdx.x; i < 3 * kMaxAdjLayers; i += blockDim.x) s_grad[i] = 0.0;
  __syncthreads();
  while (true) {
    const unsigned long long g = next_photon(P.work);
    if (g >= P.n) break;
    const unsigned long long pid = P.first + g;
    const uint32_t c0 = (uint32_t)pid, c1 = (uint32_t)(pid >> 32);
    float x = 0.f, y = 0.f, z = 0.f, ux = 0.f, uy = 0.f, uz = 1.f, w = P.w0, sleft = 0.f;
    int L = 0;
    uint32_t hop = 0, ev = 0;
    bool alive = true;
    float rd = 0.f, tt = 0.f;
    int dep_l = 0;        // the layer whose absorbed weight dep_w holds
    float dep_w = 0.f;    // merged while the photon stays in one layer
    float aL[ADJ ? kMaxAdjLayers : 1], aN[ADJ ? kMaxAdjLayers : 1], aQ[ADJ ? kMaxAdjLayers : 1];
    float score = 0.f;
    if (ADJ)
      for (int l = 0; l < P.nl; ++l) aL[l] = aN[l] = aQ[l] = 0.f;
    TausRng tr;
    uint4 r = make_uint4(0u, 0u, 0u, 0u);
    if (REF) {
      tr.init_photon(pid, P.batch, false, false);
      tr.next();  // the launch draw (radius 0: the beam stays on the axis)
    } else {
      r = philox4x32_10(make_uint4(c0, c1, 0u, kLayTag), RoundKeys{P.rk});
    }
    while (alive) {
      const LayDev& Ly = s_lay[L];
      if (sleft <= 0.f) sleft = M::neglog(REF ? tr.step_draw() : u01(r.x));
      // distance to the layer boundary ahead
      const float db = uz > 0.f ? (Ly.z1 - z) / uz : (uz < 0.f ? (Ly.z0 - z) / uz : INFINITY);
      const float s = Ly.inv_mut > 0.f ? sleft * Ly.inv_mut : INFINITY;
      if (s >= db) {  // reaches the boundary: CROSS
        x = fmaf(db, ux, x);
        y = fmaf(db, uy, y);
        z = uz > 0.f ? Ly.z1 : Ly.z0;
        if (ADJ) aL[L] += db;
        sleft = Ly.inv_mut > 0.f ? fmaxf(sleft - db / Ly.inv_mut, 0.f) : sleft;
        const bool down = uz > 0.f;
        const int Ln = down ? L + 1 : L - 1;
        const float nt = Ln < 0 ? P.n_above : (Ln >= P.nl ? P.n_below : s_lay[Ln].n);
        float uzt = 0.f;
        const float R = rfresnel(Ly.n, nt, fabsf(uz), &uzt);
        const float uf =
            REF ? tr.next() : u01(philox4x32_10(make_uint4(c0, c1, ev | 0x80000000u, kLayTag), RoundKeys{P.rk}).x);
        ++ev;
        if (uf <= R) {
          uz = -uz;  // reflected
        } else if (Ln < 0 || Ln >= P.nl) {  // escapes
          const float rr = sqrtf(x * x + y * y);
          const int ir = min((int)(rr * P.idr), P.nr);
          if (Ln < 0) {
            if (idx_ok(ir, (unsigned)P.nr + 1u, P.flags)) atomicAdd(P.rd_r + ir, to_fix(w));
            rd += w;
            if (ADJ && P.g_rd) score = w * __ldg(P.g_rd + ir);
          } else {
            if (idx_ok(ir, (unsigned)P.nr + 1u, P.flags)) atomicAdd(P.tt_r + ir, to_fix(w));
            tt += w;
            if (ADJ && P.g_tt) score = w * __ldg(P.g_tt + ir);
          }
          alive = false;
        } else {  // refracted into the next layer (Snell)
          const float ratio = Ly.n / nt;
          ux *= ratio;
          uy *= ratio;
          uz = down ? uzt : -uzt;
          L = Ln;
        }
        if (ev > P.step_cap) {
          atomicOr(P.flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
          alive = false;
        }
        continue;
      }
      // interaction inside the layer: HOP, DROP, SPIN, ROULETTE
      x = fmaf(s, ux, x);
      y = fmaf(s, uy, y);
      z = fmaf(s, uz, z);
      sleft = 0.f;
      if (ADJ) {
        aL[L] += s;
        aN[L] += 1.f;
      }
      const float absorb = w * Ly.mua * Ly.inv_mut;
      w -= absorb;
      if (absorb > 0.f) {
        const unsigned long long fa = to_fix(absorb);
        const int iz = min(max((int)(z * P.idz), 0), P.nz);
        if (idx_ok(iz, (unsigned)P.nz + 1u, P.flags)) atomicAdd((P.smem_az ? s_az : P.a_z) + iz, fa);
        if (L != dep_l) {
          if (dep_w > 0.f && idx_ok(dep_l, (unsigned)P.nl, P.flags)) atomicAdd(s_al + dep_l, to_fix(dep_w));
          dep_l = L;
          dep_w = 0.f;
        }
        dep_w += absorb;
        if (P.a_rz) {
          const int ir = min((int)(sqrtf(x * x + y * y) * P.idr), P.nr);
          if (idx_ok((size_t)ir * (P.nz + 1) + iz, (size_t)(P.nr + 1) * (P.nz + 1), P.flags))
            atomicAdd(P.a_rz + (size_t)ir * (P.nz + 1) + iz, fa);
        }
      }
      const float ucos = REF ? tr.next() : u01(r.y);
      const float cth = P.iso ? 2.f * ucos - 1.f : hg_sample<FAST>(Ly.ph, ucos);
      if (ADJ && Ly.ph.hg_mode == 0) aQ[L] += dln_hg_dg(Ly.g, cth);
      spin<FAST>(cth, REF ? tr.next() : u01(r.z), ux, uy, uz);
      if (w < kTHRESHOLD) {
        if ((REF ? tr.next() : u01(r.w)) <= kCHANCE)
          w /= kCHANCE;
        else
          alive = false;
      }
      ++hop;
      if (hop > P.step_cap) {
        atomicOr(P.flags, (unsigned int)NMC_DEVFLAG_STEPCAP);
        alive = false;
      }
      if (!REF) r = philox4x32_10(make_uint4(c0, c1, hop, kLayTag), RoundKeys{P.rk});
    }
    if (dep_w > 0.f && idx_ok(dep_l, (unsigned)P.nl, P.flags)) atomicAdd(s_al + dep_l, to_fix(dep_w));
    atomicAdd(&s_sum[NMC_LAY_PHOTONS], 1.0);
    atomicAdd(&s_sum[NMC_LAY_RD], (double)rd);
    atomicAdd(&s_sum[NMC_LAY_RD2], (double)rd * (double)rd);
    atomicAdd(&s_sum[NMC_LAY_TT], (double)tt);
    atomicAdd(&s_sum[NMC_LAY_TT2], (double)tt * (double)tt);
    atomicAdd(&s_sum[NMC_LAY_INTERACTIONS], (double)hop);
    if (ADJ && score != 0.f)
      for (int l = 0; l < P.nl; ++l) {
        atomicAdd(&s_grad[l], (double)(-score * aL[l]));
        atomicAdd(&s_grad[kMaxAdjLayers + l],
                  (double)(score * (s_lay[l].mus > 0.f ? aN[l] / s_lay[l].mus - aL[l] : -aL[l])));
        atomicAdd(&s_grad[2 * kMaxAdjLayers + l], (double)(score * aQ[l]));
      }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_priv; i += blockDim.x) {
    const unsigned long long v = s_tally[i];
    if (v) atomicAdd(i < P.nl ? P.a_layer + i : P.a_z + (i - P.nl), v);
  }
  if (ADJ)
    for (int i = threadIdx.x; i < 3 * P.nl; i += blockDim.x) {
      const int k = i / P.nl, l = i % P.nl;
      const double v = s_grad[k * kMaxAdjLayers + l];
      if (v != 0.0) atomicAdd(P.grad + i, v);
    }
  if (threadIdx.x < NMC_LAY_FIELDS && s_sum[threadIdx.x] != 0.0) atomicAdd(P.sums + threadIdx.x, s_sum[threadIdx.x]);
}

double host_fresnel_normal(double n1, double n2) {
  const double r = (n1 - n2) / (n1 + n2);
  return r * r;
}

}  // namespace
}  // namespace nmc

namespace {

nmc_status layered_impl(int32_t device, const nmc_layered_config* cfg, const nmc_layer* layers, uint64_t first,
                        uint64_t photons, double* out, double* rd_r, double* tt_r, double* a_z, double* a_rz,
                        double* a_layer, const float* g_rd, const float* g_tt, double* grad_mua, double* grad_mus,
                        double* grad_g) {
  using namespace nmc;
  const bool adj = g_rd || g_tt;
  if (!cfg || !layers || !out) return NMC_EINVAL;
  if (adj && cfg->n_layers > kMaxAdjLayers) return NMC_EINVAL;
  const bool ref = (cfg->flags & NMC_FLAG_LAYERED_REF_STREAMS) != 0;
  const bool iso = (cfg->flags & NMC_FLAG_LAYERED_ISOTROPIC) != 0;
  // the gradients follow the Philox streams and the Henyey-Greenstein phase
  if (adj && (ref || iso)) return NMC_EUNSUPPORTED;
  if (ref && cfg->seed == 0) return NMC_EINVAL;  // the dispatch batch
  // fixed-point tallies of one call stay below 2^63; more photons take more
  // calls (first += photons), whose results add up in the caller's arrays
  if (photons > (1ull << 31)) return NMC_EINVAL;
  const nmc_layered_config& c = *cfg;
  if (c.n_layers < 1 || c.n_layers > kMaxLayers || c.nr < 1 || c.nr > 65536 || c.nz < 1 || c.nz > 65536 ||
      !(c.dr > 0.f) || !(c.dz > 0.f) || !(c.n_above > 0.f) || !(c.n_below > 0.f) || !std::isfinite(c.n_above) ||
      !std::isfinite(c.n_below))
    return NMC_EINVAL;
  std::vector<LayDev> lay(c.n_layers);
  double z = 0.0;
  for (int i = 0; i < c.n_layers; ++i) {
    const nmc_layer& q = layers[i];
    const bool last = i == c.n_layers - 1;
    if (!std::isfinite(q.mua) || q.mua < 0.f || !std::isfinite(q.mus) || q.mus < 0.f || !std::isfinite(q.g) ||
        !(q.g > -1.f) || !(q.g < 1.f) || !(q.n > 0.f) || !std::isfinite(q.n) || !(q.thickness > 0.f) ||
        (!last && !std::isfinite(q.thickness)) || (!std::isfinite(q.thickness) && !(q.mua + q.mus > 0.f)))
      return NMC_EINVAL;
    LayDev& d = lay[i];
    d.mua = q.mua;
    d.mus = q.mus;
    d.inv_mut = q.mua + q.mus > 0.f ? (float)(1.0 / ((double)q.mua + q.mus)) : 0.f;
    d.n = q.n;
    d.g = q.g;
    d.z0 = (float)z;
    z += q.thickness;
    d.z1 = std::isfinite(q.thickness) ? (float)z : INFINITY;
    nmc_tissue_params tp{};
    tp.gv[1] = q.g;
    d.ph = phase_const(tp, 1);
  }
  nmc::DeviceScope dev(device);
  if (!dev.ok) return NMC_EDEVICE;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NMC_EDEVICE;
  std::vector<void*> allocs;
  auto dalloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
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
  const size_t nr1 = (size_t)c.nr + 1, nz1 = (size_t)c.nz + 1;
  LayDev* dlay = (LayDev*)dalloc(sizeof(LayDev) * c.n_layers);
  auto* drd = (unsigned long long*)dalloc(8 * nr1);
  auto* dtt = (unsigned long long*)dalloc(8 * nr1);
  auto* daz = (unsigned long long*)dalloc(8 * nz1);
  auto* darz = a_rz ? (unsigned long long*)dalloc(8 * nr1 * nz1) : nullptr;
  auto* dal = (unsigned long long*)dalloc(8 * c.n_layers);
  auto* dsum = (double*)dalloc(sizeof(double) * NMC_LAY_FIELDS);
  auto* dwork = (unsigned long long*)dalloc(16);
  auto* dgrd = g_rd ? (float*)dalloc(4 * nr1) : nullptr;
  auto* dgtt = g_tt ? (float*)dalloc(4 * nr1) : nullptr;
  auto* dgrad = adj ? (double*)dalloc(sizeof(double) * 3 * c.n_layers) : nullptr;
  if (!dlay || !drd || !dtt || !daz || (a_rz && !darz) || !dal || !dsum || !dwork || (g_rd && !dgrd) ||
      (g_tt && !dgtt) || (adj && !dgrad))
    return done(NMC_ENOMEM);
  if (cudaMemcpyAsync(dlay, lay.data(), sizeof(LayDev) * c.n_layers, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      (g_rd && cudaMemcpyAsync(dgrd, g_rd, 4 * nr1, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (g_tt && cudaMemcpyAsync(dgtt, g_tt, 4 * nr1, cudaMemcpyHostToDevice, st) != cudaSuccess))
    return done(NMC_EDEVICE);
  LayParams P{};
  P.lay = dlay;
  P.nl = c.n_layers;
  P.n_above = c.n_above;
  P.n_below = c.n_below;
  const double rsp = host_fresnel_normal(c.n_above, layers[0].n);
  P.w0 = (float)(1.0 - rsp);
  P.nr = c.nr;
  P.nz = c.nz;
  P.idr = (float)(1.0 / c.dr);
  P.idz = (float)(1.0 / c.dz);
  P.rd_r = drd;
  P.tt_r = dtt;
  P.a_z = daz;
  P.a_rz = darz;
  P.a_layer = dal;
  P.sums = dsum;
  P.first = first;
  P.n = photons;
  P.k0 = (uint32_t)c.seed;
  P.k1 = (uint32_t)(c.seed >> 32);
  philox_round_keys(P.k0, P.k1, P.rk);
  P.work = dwork;
  P.flags = (unsigned int*)(dwork + 1);
  P.step_cap = 20000000u;
  P.g_rd = dgrd;
  P.g_tt = dgtt;
  P.grad = dgrad;
  P.batch = ref ? c.seed : 1;
  P.iso = iso ? 1 : 0;
  const bool fast = !(c.flags & NMC_FLAG_PRECISE_MATH);
  const void* f =
      adj ? (fast ? (const void*)layered_kernel<true, true, false> : (const void*)layered_kernel<false, true, false>)
      : ref ? (fast ? (const void*)layered_kernel<true, false, true> : (const void*)layered_kernel<false, false, true>)
            : (fast ? (const void*)layered_kernel<true, false, false> : (const void*)layered_kernel<false, false, false>);
  // A(z) joins the per-layer sums in shared memory while both fit in 16 KB
  P.smem_az = (size_t)(c.n_layers + nz1) * 8 <= 16384 ? 1 : 0;
  const size_t smem = (size_t)(c.n_layers + (P.smem_az ? nz1 : 0)) * 8;
  int per_sm = 0, nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, 256, smem) != cudaSuccess || per_sm < 1)
    return done(NMC_EDEVICE);
  const unsigned long long grid =
      std::max<unsigned long long>(1, std::min<unsigned long long>((unsigned long long)nsm * per_sm,
                                                                   (photons + 255) / 256));
  void* args[] = {(void*)&P};
  if (photons > 0 && cudaLaunchKernel(f, dim3((unsigned)grid), dim3(256), args, smem, st) != cudaSuccess)
    return done(NMC_EDEVICE);
  std::vector<unsigned long long> hrd(nr1), htt(nr1), haz(nz1), hal(c.n_layers), harz(a_rz ? nr1 * nz1 : 0);
  std::vector<double> hgrad(adj ? 3 * c.n_layers : 0);
  unsigned int flags = 0;
  if (cudaMemcpyAsync(out, dsum, sizeof(double) * NMC_LAY_FIELDS, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(hrd.data(), drd, 8 * nr1, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(htt.data(), dtt, 8 * nr1, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(haz.data(), daz, 8 * nz1, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(hal.data(), dal, 8 * c.n_layers, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      (a_rz && cudaMemcpyAsync(harz.data(), darz, 8 * nr1 * nz1, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
      (adj && cudaMemcpyAsync(hgrad.data(), dgrad, sizeof(double) * 3 * c.n_layers, cudaMemcpyDeviceToHost, st) !=
                  cudaSuccess) ||
      cudaMemcpyAsync(&flags, P.flags, sizeof flags, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return done(NMC_EDEVICE);
  out[NMC_LAY_SPECULAR] = rsp * (double)photons;
  double a_tot = 0.0;
  for (int i = 0; i < c.n_layers; ++i) {
    const double v = (double)hal[i] * kUnfix;
    a_tot += v;
    if (a_layer) a_layer[i] += v;
  }
  out[NMC_LAY_A] = a_tot;
  for (size_t i = 0; i < nr1; ++i) {
    if (rd_r) rd_r[i] += (double)hrd[i] * kUnfix;
    if (tt_r) tt_r[i] += (double)htt[i] * kUnfix;
  }
  if (a_z)
    for (size_t i = 0; i < nz1; ++i) a_z[i] += (double)haz[i] * kUnfix;
  if (a_rz)
    for (size_t i = 0; i < nr1 * nz1; ++i) a_rz[i] += (double)harz[i] * kUnfix;
  for (int l = 0; adj && l < c.n_layers; ++l) {
    if (grad_mua) grad_mua[l] += hgrad[l];
    if (grad_mus) grad_mus[l] += hgrad[c.n_layers + l];
    if (grad_g) grad_g[l] += hgrad[2 * c.n_layers + l];
  }
  if (flags & NMC_DEVFLAG_BOUNDS) return done(NMC_EDEVICE);
  return done((flags & NMC_DEVFLAG_STEPCAP) ? NMC_ESTEPCAP : NMC_OK);
}

}  // namespace

extern "C" nmc_status nmc_layered_run(int32_t device, const nmc_layered_config* cfg, const nmc_layer* layers,
                                      uint64_t first, uint64_t photons, double* out, double* rd_r, double* tt_r,
                                      double* a_z, double* a_rz, double* a_layer) {
  return layered_impl(device, cfg, layers, first, photons, out, rd_r, tt_r, a_z, a_rz, a_layer, nullptr, nullptr,
                      nullptr, nullptr, nullptr);
}

extern "C" nmc_status nmc_layered_adjoint(int32_t device, const nmc_layered_config* cfg, const nmc_layer* layers,
                                          uint64_t first, uint64_t photons, const float* grad_rd_r,
                                          const float* grad_tt_r, double* out, double* rd_r, double* tt_r,
                                          double* grad_mua, double* grad_mus, double* grad_g) {
  if (!grad_rd_r && !grad_tt_r) return NMC_EINVAL;
  return layered_impl(device, cfg, layers, first, photons, out, rd_r, tt_r, nullptr, nullptr, nullptr, grad_rd_r,
                      grad_tt_r, grad_mua, grad_mus, grad_g);
}
