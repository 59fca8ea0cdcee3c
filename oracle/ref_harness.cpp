// ref_harness.cpp - runs the reference's own photon kernels on CPU cores.
//
// TEST INFRASTRUCTURE ONLY (the oracle's cross-check and the timed CPU
// baseline).  Nothing in the product links this file.
//
// The reference kernels (NMC/NMCCode/kernels.metal, which pulls in
// helpers.metal and definitions.h) are compiled in place, unmodified, behind
// the host shim in oracle/ref_shim; see oracle/Makefile.  Each call walks the
// photons (run, index) in the order main.m:159-168 dispatches them, on
// `nthreads` std::threads with private tally buffers, and sums the buffers in
// double.  The per-thread slab offsets the kernels use (index*BINS,
// index*Ny*Nx, ...) are folded into the base pointers handed to each call, so
// every photon writes into its worker's private slab.
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "kernels.metal"

// The shim maps Metal qualifiers to nothing; release the names for host code.
#undef thread
#undef device
#undef constant
#undef kernel

namespace refh {

// Pointer `p` shifted back by `off` elements, so that p_shifted[off + k]
// addresses p[k]; this reproduces the reference's per-thread slab offsets.
template <class T>
static T* shift_back(T* p, long off) {
  return reinterpret_cast<T*>(reinterpret_cast<uintptr_t>(p) -
                              static_cast<uintptr_t>(off) * sizeof(T));
}

template <class F>
static void parallel_photons(long n, int nthreads, F&& body) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > n) nthreads = n > 0 ? (int)n : 1;
  std::vector<std::thread> ts;
  for (int t = 0; t < nthreads; ++t) {
    long lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
    ts.emplace_back([=, &body] { body(t, lo, hi); });
  }
  for (auto& th : ts) th.join();
}

}  // namespace refh

extern "C" {

// sizeof of the reference structs, as this compiler lays them out.
int ref_sizeof_runparams() { return (int)sizeof(RunParams); }
int ref_sizeof_tissueparams() { return (int)sizeof(TissueParams); }
int ref_bins() { return BINS; }

// MCSubKernel (kernels.metal:59-319) for runs [run_lo, run_hi] x indices
// [0, batch).  J: BINS+1 doubles, F: (BINS+1)^2 doubles, SAE: 3 doubles
// (all +=).  per_photon_sae (optional): 3 floats per photon, photon order
// p = (run - run_lo) * batch + index.
int ref_mcsub(const RunParams* rp, const TissueParams* tp, int run_lo, int run_hi,
              int batch, int nthreads, double* J, double* F, double* SAE,
              float* per_photon_sae) {
  const long nrun = run_hi - run_lo + 1;
  const long n = nrun * batch;
  const int nJ = BINS + 1, nF = (BINS + 1) * (BINS + 1);
  std::vector<std::vector<double>> accJ(nthreads < 1 ? 1 : nthreads),
      accF(accJ.size()), accS(accJ.size());
  refh::parallel_photons(n, nthreads, [&](int t, long lo, long hi) {
    RunParams rpl = *rp;
    TissueParams tpl = *tp;
    std::vector<float> Jl(nJ, 0.f), Fl(nF, 0.f);
    std::vector<double>& aJ = accJ[t];
    std::vector<double>& aF = accF[t];
    std::vector<double>& aS = accS[t];
    aJ.assign(nJ, 0.0);
    aF.assign(nF, 0.0);
    aS.assign(3, 0.0);
    long since_flush = 0;
    for (long p = lo; p < hi; ++p) {
      int run = run_lo + (int)(p / batch);
      uint index = (uint)(p % batch);
      float sae[3] = {0.f, 0.f, 0.f};
      MCSubKernel(&rpl, &tpl, refh::shift_back(Jl.data(), (long)index * BINS),
                  refh::shift_back(Fl.data(), (long)index * BINS * BINS),
                  refh::shift_back(sae, (long)index * 3), &run, index);
      for (int k = 0; k < 3; ++k) aS[k] += sae[k];
      if (per_photon_sae)
        for (int k = 0; k < 3; ++k) per_photon_sae[p * 3 + k] = sae[k];
      if (++since_flush == 64 || p + 1 == hi) {
        for (int k = 0; k < nJ; ++k) { aJ[k] += Jl[k]; Jl[k] = 0.f; }
        for (int k = 0; k < nF; ++k) { aF[k] += Fl[k]; Fl[k] = 0.f; }
        since_flush = 0;
      }
    }
  });
  for (size_t t = 0; t < accJ.size(); ++t) {
    if (accJ[t].empty()) continue;
    for (int k = 0; k < nJ; ++k) J[k] += accJ[t][k];
    for (int k = 0; k < nF; ++k) F[k] += accF[t][k];
    for (int k = 0; k < 3; ++k) SAE[k] += accS[t][k];
  }
  return 0;
}

// MCXYZKernel (kernels.metal:321-754).  F3D: Nx*Ny*Nz doubles, Rd2D and
// DetPhot2D: Nx*Ny doubles, rd_slots: batch doubles (all +=).
// per_photon_rd (optional): the Rd_loc each photon adds to Rd[index].
int ref_mcxyz(const RunParams* rp, const TissueParams* tp, const unsigned char* V,
              int run_lo, int run_hi, int batch, int nthreads, double* F3D,
              double* Rd2D, double* DetPhot2D, double* rd_slots,
              float* per_photon_rd) {
  const long nrun = run_hi - run_lo + 1;
  const long n = nrun * batch;
  const long nvox = (long)rp->Nx * rp->Ny * rp->Nz;
  const long n2d = (long)rp->Nx * rp->Ny;
  const int nt = nthreads < 1 ? 1 : nthreads;
  // atomic_float is a double-backed accumulator in the shim, so the kernel's
  // relaxed atomics accumulate in double here.
  std::vector<std::vector<double>> aF(nt), aR(nt), aP(nt), aSlots(nt);
  refh::parallel_photons(n, nthreads, [&](int t, long lo, long hi) {
    RunParams rpl = *rp;
    TissueParams tpl = *tp;
    std::vector<metal::atomic_float> f3d(nvox), r2d(n2d);
    std::vector<metal::atomic_int> p2d(n2d);
    std::vector<double> slots(batch, 0.0);
    float tseed = 0.f;
    for (long p = lo; p < hi; ++p) {
      int run = run_lo + (int)(p / batch);
      uint index = (uint)(p % batch);
      metal::atomic_float rd_loc{};
      MCXYZKernel(&rpl, &tpl, (char*)V, f3d.data(), refh::shift_back(&rd_loc, (long)index),
                  refh::shift_back(r2d.data(), (long)index * n2d),
                  refh::shift_back(p2d.data(), (long)index * n2d), &run, &tseed, index);
      slots[index] += (double)rd_loc.v;
      if (per_photon_rd) per_photon_rd[p] = (float)rd_loc.v;
    }
    aF[t].resize(nvox);
    for (long k = 0; k < nvox; ++k) aF[t][k] = f3d[k].v;
    aR[t].resize(n2d);
    aP[t].resize(n2d);
    for (long k = 0; k < n2d; ++k) { aR[t][k] = r2d[k].v; aP[t][k] = (double)p2d[k].v; }
    aSlots[t] = slots;
  });
  for (int t = 0; t < nt; ++t) {
    if (aF[t].empty()) continue;
    for (long k = 0; k < nvox; ++k) F3D[k] += aF[t][k];
    for (long k = 0; k < n2d; ++k) { Rd2D[k] += aR[t][k]; DetPhot2D[k] += aP[t][k]; }
    for (int k = 0; k < batch; ++k) rd_slots[k] += aSlots[t][k];
  }
  return 0;
}

// MCXYZKernelTT (kernels.metal:757-1118).  `run_value` < 0 reproduces the
// reference host, whose mis-bound buffer makes the kernel read 0 as
// iRunNum on every dispatch (MetalMC.m:462-473); otherwise the real run
// number is passed.  Rd2D is indexed ix*Ny+iy from unclamped indices
// (kernels.metal:978-985); callers use boundaryflag 1 so that indices stay
// within one row of the grid, and the buffer here carries Ny+1 guard cells
// on each side.
int ref_mcxyz_tt(const RunParams* rp, const TissueParams* tp, const unsigned char* V,
                 int run_lo, int run_hi, int batch, int nthreads, int run_value,
                 double* F3D, double* Rd2D, double* rd_slots, float* per_photon_rd) {
  const long nrun = run_hi - run_lo + 1;
  const long n = nrun * batch;
  const long nvox = (long)rp->Nx * rp->Ny * rp->Nz;
  const long n2d = (long)rp->Nx * rp->Ny;
  const long guard = rp->Ny + 1;
  const int nt = nthreads < 1 ? 1 : nthreads;
  std::vector<std::vector<double>> aF(nt), aR(nt), aSlots(nt);
  refh::parallel_photons(n, nthreads, [&](int t, long lo, long hi) {
    RunParams rpl = *rp;
    TissueParams tpl = *tp;
    std::vector<float> f3d(nvox, 0.f), r2d(n2d + 2 * guard, 0.f);
    std::vector<double> accF(nvox, 0.0), accR(n2d, 0.0), slots(batch, 0.0);
    long since_flush = 0;
    for (long p = lo; p < hi; ++p) {
      int run = run_value < 0 ? 0 : run_lo + (int)(p / batch);
      uint index = (uint)(p % batch);
      float rd_loc = 0.f;
      MCXYZKernelTT(&rpl, &tpl, (char*)V, f3d.data(), refh::shift_back(&rd_loc, (long)index),
                    r2d.data() + guard, &run, index);
      slots[index] += rd_loc;
      if (per_photon_rd) per_photon_rd[p] = rd_loc;
      if (++since_flush == 256 || p + 1 == hi) {
        for (long k = 0; k < nvox; ++k) { accF[k] += f3d[k]; f3d[k] = 0.f; }
        for (long k = 0; k < n2d; ++k) { accR[k] += r2d[guard + k]; r2d[guard + k] = 0.f; }
        since_flush = 0;
      }
    }
    aF[t] = std::move(accF);
    aR[t] = std::move(accR);
    aSlots[t] = std::move(slots);
  });
  for (int t = 0; t < nt; ++t) {
    if (aF[t].empty()) continue;
    for (long k = 0; k < nvox; ++k) F3D[k] += aF[t][k];
    for (long k = 0; k < n2d; ++k) Rd2D[k] += aR[t][k];
    for (int k = 0; k < batch; ++k) rd_slots[k] += aSlots[t][k];
  }
  return 0;
}

// The reference generator (helpers.metal:319-371): `n` draws after seeding
// with (s1, s2, s3).
void ref_taus_draws(unsigned s1, unsigned s2, unsigned s3, int n, float* out) {
  RandomGen g(s1, s2, s3);
  for (int k = 0; k < n; ++k) out[k] = g.rand();
}

// Fresnel::RFresnel (helpers.metal:243-291).
float ref_rfresnel(float n1, float n2, float ca1, float* ca2) {
  return Fresnel::RFresnel(n1, n2, ca1, ca2);
}

}  // extern "C"
