// engine.h - parameter blocks and launch entry points of the transport
// kernels, shared by the kernel translation units and the C-ABI runtime.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "nmc_abi.h"
#include "nmc_device.cuh"

namespace nmc {

// Makes `device` current for the life of an entry point and gives the
// caller's current device back on exit, so a handle on one GPU works from a
// thread whose current device is another, and the library never changes the
// caller's current device.
struct DeviceScope {
  int prev = -1;
  bool ok = false;
  explicit DeviceScope(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = cudaSetDevice(device) == cudaSuccess;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// One detection event recorded by the adjoint's forward pass.
struct AdjEvent {
  unsigned int photon;  // photon index within the launch
  unsigned int bin;     // radial bin
  float w;              // detected weight
  float pad;
};

// Voxel kernels (MCXYZKernel kernels.metal:321-754 and MCXYZKernelTT
// :757-1118).  Photon positions are kept as an integer voxel-lattice cell
// (k = floor(x / d), unbounded) plus an FP32 offset inside the cell.
// Per-set sums of a voxel sweep (u64 fixed point 2^-32 for weights).
struct XyzSweepSums {
  unsigned long long photons, substeps, scatters, A, rd;
  double rd2;
};

struct XyzParams {
  int Nx, Ny, Nz;
  float dx, dy, dz, idx, idy, idz;
  float dxmax, dymax, dzmax;  // largest float below dx, dy, dz
  int hx, hy, ox, oy;         // Nx/2, Ny/2 rounded down; Nx, Ny odd
  float hdx, hdy;             // dx/2, dy/2
  int ksurf;                  // zsurf = ksurf * dz + fsurf
  float fsurf;
  int boundaryflag, det_state;
  int launchflag, mcflag;
  float xs, ys, zs, ux0, uy0, uz0, radius, waist, zfocus, n1, n2;
  float r_min, r_max, na;
  int det_everything;         // detector accepts every exit (skips the geometry test)
  const uint8_t* V;
  float4 core[NMC_NTISS];     // mua, mus, 1/mus, g
  PhaseConst phase[NMC_NTISS];
  uint32_t flags;
  int fast_math;              // SFU approximations (Math<true>)
  uint32_t step_cap;
  uint32_t per_fetch;         // photons a thread takes from the queue at a time (>= 1)
  unsigned long long* F3D;
  unsigned long long* Rd2D;
  unsigned int* Det2D;
  unsigned long long* rd_slots;
  unsigned long long nslots;
  DevSums* sums;
  unsigned long long first, n;
  RngParams rng;
  TraceParams trace;
  // media with per-voxel optical properties (no reference counterpart)
  const float4* vox;          // (mua, mus, 1/mus, g) per voxel
  // radial reflectance Rd(r) at the detection plane, u64 fixed point
  unsigned long long* rd_r;   // rd_bins + 1 entries (last = overflow), may be null
  int rd_bins;
  float rd_idr;
  // perturbation Monte Carlo adjoint
  int adj_pass;               // 0: record detection events, 1: accumulating replay, 2: score replay
  AdjEvent* ev;
  unsigned long long* ev_count;
  unsigned int ev_cap;
  const float* adj_D;         // per photon score (accumulating replay)
  float* adj_Dw;              // per photon score (written by the score replay)
  const float* adj_G;         // upstream gradient per radial bin (replays)
  const float* adj_GF;        // upstream gradient per voxel of F3D, or null (replays)
  double* gL;                 // per voxel: sum D * charged path length (absorption)
  double* gM;                 // per voxel: d ln p(path)/dmus terms weighted by D
  double* gQ;                 // per voxel: sum D * dln p_HG / dg over scatterings
  // record pass with a deposit list (for a fluence loss): every merged
  // deposit (voxel, weight) of a photon, in chunks of kDepChunk records taken
  // by the threads from a pool; a chunk starts with a header record
  // (0xFFFFFFFF, photon index) and every photon's records follow its header
  uint2* dl_pool;             // dl_chunks * kDepChunk records, or null: no list
  unsigned int dl_chunks;
  unsigned int* dl_fill;      // records written per chunk
  unsigned long long* dl_next;  // chunks taken (may pass dl_chunks: the list is then incomplete)
  // batched sweep over tissue tables (one table per set, e.g. per wavelength)
  const float4* sw_core;               // n_sets * NMC_NTISS (mua, mus, 1/mus, g)
  const PhaseConst* sw_phase;          // n_sets * NMC_NTISS
  const unsigned long long* sw_prefix; // n_sets + 1 budget prefix sums, in queue order
  const unsigned long long* sw_first;  // id of each queue slot's first photon
  const unsigned int* sw_order;        // the set each queue slot runs
  XyzSweepSums* sw_sums;               // n_sets
  int sw_nsets;
};

// kRecord: kVoxel plus the adjoint's detection-event list (its forward pass);
// kScore: the adjoint's score replay (per photon total score, no tallies);
// kAdjoint: the adjoint's accumulating replay.
constexpr unsigned int kDepChunk = 256;  // deposit-list records per chunk

enum XyzMode { kTissue = 0, kVoxel = 1, kAdjoint = 2, kSweep = 3, kRecord = 4, kScore = 5 };

// Layered semi-infinite kernel (MCSubKernel kernels.metal:59-319).
struct SubParams {
  float mua, mus, mut, albedo, n1, n2;
  float dr, dz, idr, idz;
  int bins;
  int mcflag, boundaryflag;
  float radius, waist, zfocus, xs, ys, zs;
  PhaseConst phase;  // tissue 1
  int phase_kind;    // SubPhase
  int fast_math;
  int skip_F;        // no F(r,z) tally
  int global_tallies;  // F(r,z), J(r) straight to global memory (no shared-memory privatisation)
  uint32_t per_fetch;  // photons a thread takes from the queue at a time (>= 1)
  unsigned long long* J;  // fixed point 2^-32, BINS+1
  unsigned long long* F;  // (BINS+1)^2
  DevSums* sums;
  unsigned long long first, n;
  RngParams rng;
  TraceParams trace;
  uint32_t step_cap;
};

enum SubPhase { kPhaseHG = 0, kPhaseIsoRef = 1, kPhaseTT = 2 };

// One parameter set of a batched sweep, as the kernel reads it.
struct __align__(16) SweepSetDev {
  float mut, albedo, n1, n2, rsp;
  unsigned int id;           // the set's index (its key offset and its tallies)
  unsigned long long first;  // id of the set's first photon
  PhaseConst ph;
};

struct SweepParams {
  int nsets;
  const SweepSetDev* sets;           // in queue order
  const unsigned long long* prefix;  // nsets + 1 prefix sums of the budgets, in queue order
  unsigned long long total;
  int bins;
  float idr;
  int mcflag, boundaryflag;
  float radius, waist, zfocus, xs, ys, zs;
  unsigned long long* J;     // nsets x (bins + 1), may be null
  unsigned long long* sums;  // nsets x 5
  double* e2;                // nsets
  unsigned long long* work;
  unsigned int* flags;
  uint32_t k0, k1;
  int phase_kind, fast;
  uint32_t step_cap;
};

cudaError_t launch_sweep(const SweepParams& p, int grid, int block, cudaStream_t stream);
cudaError_t sweep_occupancy(const SweepParams& p, int block, int* blocks_per_sm);

// Parameter blocks from the reference's configuration (params.cu); device
// pointers are left for the caller to set.
PhaseConst phase_const(const nmc_tissue_params& tp, int t);
// Tissue t of the table has usable optical properties: finite mua >= 0,
// finite mus > 0, finite g and finite two-term phase terms (gf, af, gb, ab,
// CC), the same test for every entry point that takes a tissue table.
bool tissue_usable(const nmc_tissue_params& tp, int t);
RngParams rng_params(const nmc_ext& e, int sim);
void fill_xyz(XyzParams& p, const nmc_run_params& rp, const nmc_tissue_params& tp, const nmc_ext& e,
              int sim);
void fill_sub(SubParams& p, const nmc_run_params& rp, const nmc_tissue_params& tp, const nmc_ext& e);

// Launchers (blocking is up to the caller; all work goes on `stream`).
cudaError_t launch_mcxyz(const XyzParams& p, bool two_term, bool trace, int grid, int block,
                         cudaStream_t stream);
cudaError_t mcxyz_occupancy(bool two_term, bool trace, int block, int* blocks_per_sm);
// per-voxel media (mode kVoxel or kAdjoint), Philox streams, one-term HG
cudaError_t launch_mcxyz_voxel(const XyzParams& p, int mode, bool trace, int grid, int block,
                               cudaStream_t stream);
cudaError_t mcxyz_voxel_occupancy(int mode, bool trace, int block, int* blocks_per_sm);
// D[photon] += G[bin] * w over recorded events
cudaError_t launch_mcxyz_sweep(const XyzParams& p, bool two_term, int grid, int block, cudaStream_t stream);
cudaError_t mcxyz_sweep_occupancy(bool two_term, int block, int* blocks_per_sm);
cudaError_t launch_adjoint_scores(const AdjEvent* ev, unsigned int n_ev, const float* G, float* D,
                                  cudaStream_t stream);
// D[photon] += sum GF[voxel] * deposit over the record pass's deposit list
cudaError_t launch_deposit_scores(const uint2* pool, const unsigned int* fill, unsigned int n_chunks,
                                  const float* GF, float* D, unsigned long long n_photons, cudaStream_t stream);

cudaError_t launch_mcsub(const SubParams& p, bool trace, int grid, int block, cudaStream_t stream);
cudaError_t mcsub_occupancy(const SubParams& p, bool trace, int block, int* blocks_per_sm);
size_t mcsub_smem_bytes(int bins);

// u64 fixed point (2^-32) -> float / double, element-wise.
cudaError_t launch_unfix_f32(const unsigned long long* src, float* dst, size_t n, double scale,
                             cudaStream_t stream);
cudaError_t launch_unfix_f64(const unsigned long long* src, double* dst, size_t n, double scale,
                             cudaStream_t stream);

}  // namespace nmc
