/*
 * nmc_abi.h - C ABI of the GB300 photon-transport engine (mcsub / mcxyz /
 * mcxyz two-term hop-drop-spin-roulette loop and its tallies).
 *
 * The reference drives its GPU kernels through an Objective-C class
 * (NMC/NMCCode/MetalMC.h:25-31):
 *
 *   initWithDevice:kernel_type      -> nmc_create
 *   prepareData:run_params:tiss:v   -> nmc_prepare
 *   setNumRunsSeed:                 -> nmc_set_num_runs_seed
 *   sendComputeCommand              -> nmc_send_compute_command
 *   getComputeResults: (16 arrays)  -> nmc_get_compute_results
 *
 * Everything here is plain C: pointers, sizes and POD structs, no CUDA or
 * torch types.  Every entry point returns an nmc_status and never exits the
 * process (the reference calls exit(1) on bad input, mcio.h:163).
 *
 * The two configuration PODs are byte-identical to the reference's
 * `struct RunParams` (172 bytes) and `struct TissueParams` (608 bytes)
 * (NMC/NMCCode/definitions.h:186-218); they carry an nmc_ prefix so that a
 * caller may include this header next to the reference's definitions.h and
 * pass `(const nmc_run_params*)&runParams`.
 */
#ifndef NMC_ABI_H
#define NMC_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NMC_ABI_VERSION 1

/* definitions.h:57-58 (Ntiss, STRLEN) */
#define NMC_NTISS 19
#define NMC_STRLEN 32

/* Reference compile-time constants kept as defaults (definitions.h:16-82). */
#define NMC_PHOTON_TOTAL_DEFAULT 100000u /* PHOTON_TOTAL */
#define NMC_PHOTON_BATCH_DEFAULT 10000u  /* PHOTON_BATCH */
#define NMC_MCSUB_BINS_DEFAULT 101       /* BINS (bins 1..BINS, BINS = overflow) */
#define NMC_MCSUB_DR_DEFAULT 0.0020f     /* dr_mcsub */
#define NMC_MCSUB_DZ_DEFAULT 0.0020f     /* dz_mcsub */

/* Simulation kinds: same values as enum MC_SIM_TYPE (definitions.h:151-164). */
typedef enum nmc_sim_type {
  NMC_SIM_MCSUB = 0,
  NMC_SIM_MCXYZ = 1,
  NMC_SIM_MCXYZ_TT = 2,
  NMC_SIM_POLARIZATION_CBS_ELECTRIC_FIELDS = 3,
  NMC_SIM_POLARIZATION_MUELLER_STOKES = 4,
  NMC_SIM_RAMAN = 5
} nmc_sim_type;

/* Detection side: enum MC_PH_PACKETS_DETECTION_STATE (definitions.h:168-172). */
enum { NMC_DET_REFLECTANCE = 0, NMC_DET_TRANSMITTANCE = 1 };

/* struct RunParams, definitions.h:186-209.  Enums are 4-byte ints. */
typedef struct nmc_run_params {
  char myname[NMC_STRLEN];
  int32_t mcflag, launchflag, boundaryflag, speckleflag, semiflag;
  float xfocus, yfocus, zfocus;
  float ux0, uy0, uz0;
  float radius, det_radius, xd;
  float waist;
  float zsurf;
  float n1, n2;
  float na, lambda, lc;
  int32_t det_state; /* enum MC_PH_PACKETS_DETECTION_STATE */
  int32_t ph_quant;  /* enum MC_PH_PACKETS_QUANTITY */
  float dx, dy, dz;
  int32_t Nx, Ny, Nz, Nt;
  float xs, ys, zs;
  float time_min;
  int32_t mckernelflag; /* enum MC_SIM_TYPE */
} nmc_run_params;

/* struct TissueParams, definitions.h:211-218.  Index 0 is unused by the
 * reference's readers (tissue ids are 1..Nt, mcio.h:128). */
typedef struct nmc_tissue_params {
  float muav[NMC_NTISS];
  float musv[NMC_NTISS];
  float gv[NMC_NTISS];
  float gf[NMC_NTISS], af[NMC_NTISS], gb[NMC_NTISS], ab[NMC_NTISS], CC[NMC_NTISS];
} nmc_tissue_params;

#if defined(__cplusplus)
static_assert(sizeof(nmc_run_params) == 172, "RunParams must stay 172 bytes");
static_assert(offsetof(nmc_run_params, n1) == 96, "RunParams.n1 offset");
static_assert(offsetof(nmc_run_params, det_state) == 116, "RunParams.det_state offset");
static_assert(offsetof(nmc_run_params, dx) == 124, "RunParams.dx offset");
static_assert(offsetof(nmc_run_params, Nx) == 136, "RunParams.Nx offset");
static_assert(offsetof(nmc_run_params, xs) == 152, "RunParams.xs offset");
static_assert(offsetof(nmc_run_params, time_min) == 164, "RunParams.time_min offset");
static_assert(offsetof(nmc_run_params, mckernelflag) == 168, "RunParams.mckernelflag offset");
static_assert(sizeof(nmc_tissue_params) == 608, "TissueParams must stay 608 bytes");
#elif defined(__STDC_VERSION__) && __STDC_VERSION__ >= 201112L
_Static_assert(sizeof(nmc_run_params) == 172, "RunParams must stay 172 bytes");
_Static_assert(sizeof(nmc_tissue_params) == 608, "TissueParams must stay 608 bytes");
#endif

/* ---------------------------------------------------------------- status */
typedef enum nmc_status {
  NMC_OK = 0,
  NMC_EINVAL = 1,      /* bad argument or configuration */
  NMC_EIO = 2,         /* file missing, short or malformed */
  NMC_EDEVICE = 3,     /* CUDA error or missing device */
  NMC_ETIMEOUT = 4,    /* host wait exceeded nmc_ext.timeout_s */
  NMC_ESTEPCAP = 5,    /* a photon hit the device-side step cap */
  NMC_ENOMEM = 6,      /* host or device allocation failed */
  NMC_EUNSUPPORTED = 7,/* kind or option not built */
  NMC_ESTATE = 8       /* call out of order (e.g. run before prepare) */
} nmc_status;

/* ---------------------------------------------------------- extensions */
/* Random number streams. */
enum {
  /* Philox4x32-10, key = (seed lo, seed hi), counter = (photon id lo,
   * photon id hi, block #, 0x4E4D4321).  Each photon owns one stream, so
   * results do not depend on thread mapping. */
  NMC_RNG_PHILOX = 0,
  /* The reference's Tausworthe/xorshift generator with its own per-thread
   * seeding (helpers.metal:319-371, kernels.metal:91-95,339-343,772); photon
   * id p maps to (run = p / photons_per_dispatch + 1, index = p %
   * photons_per_dispatch) exactly as main.m:159-168 dispatches them. */
  NMC_RNG_TAUS_REF = 1
};

/* Phase function of the mcsub kernel. */
enum {
  NMC_PHASE_HG = 0,            /* Henyey-Greenstein with gv[1] */
  NMC_PHASE_ISOTROPIC_REF = 1, /* what MCSubKernel actually samples (kernels.metal:252) */
  NMC_PHASE_TWO_TERM = 2       /* two-term HG with gf/af/gb/ab/CC[1] (kernels.metal:1053-1070) */
};

/* Reference behaviours that are switchable (default = reference behaviour). */
enum {
  /* Two-term kernel: replay the run-1 RNG streams on every dispatch, as the
   * reference does because its host binds DetPhot2D where the kernel reads
   * iRunNum (MetalMC.m:462-473 vs kernels.metal:757-768). */
  NMC_FLAG_TT_REPLAY_RUN1 = 1u << 0,
  /* Disable the mcxyz MIN_VALUE / MAX_SCATT kill (kernels.metal:747). */
  NMC_FLAG_NO_HARD_KILL = 1u << 1,
  /* Use CUDA's correctly rounded / 1-ulp log, exp, sin/cos, reciprocal and
   * pow in the photon step instead of the SFU approximations. */
  NMC_FLAG_PRECISE_MATH = 1u << 2,
  /* Skip the fluence tally (mcsub F(r,z)) when only Rd, J and the totals
   * are wanted. */
  NMC_FLAG_SKIP_FLUENCE = 1u << 3,
  /* mcsub: deposit F(r,z) and J(r) straight into the global u64 tallies
   * instead of privatising them per block in shared memory. */
  NMC_FLAG_GLOBAL_TALLIES = 1u << 4,
  /* Layered runs: draw from the reference's generator in MCSubKernel's
   * order (kernels.metal:91-95 seeding; a launch draw, then per hop the step,
   * the Fresnel choice at a boundary, cos theta, psi and, below THRESHOLD,
   * the roulette draw: :113-290).  Photon p is (run p / batch + 1, index
   * p % batch) of the reference's dispatch loop, with batch = the config's
   * `seed` (PHOTON_BATCH = 10000, definitions.h:17, in the reference).  With
   * one semi-infinite layer these are the reference kernel's own photons. */
  NMC_FLAG_LAYERED_REF_STREAMS = 1u << 5,
  /* Layered runs: isotropic scattering, which is what MCSubKernel samples
   * (kernels.metal:252 overwrites its Henyey-Greenstein cos theta). */
  NMC_FLAG_LAYERED_ISOTROPIC = 1u << 6,
  /* Voxel handles: leave the L2 cache's persisting set-aside alone.  By
   * default nmc_prepare marks the handle's u64 fluence tally (8 bytes per
   * voxel) as persisting in L2 on the handle's stream, and raises the
   * device's persisting set-aside (cudaLimitPersistingL2CacheSize, a setting
   * of this process's context) to that size, capped by the device, while
   * the handle lives; nmc_destroy puts the previous value back.  Without it
   * the L2 writes the tally's lines back to DRAM under the transport's
   * atomics (about 29 GB per 1e8 photons on a 200^3 grid); with it the
   * transport's DRAM traffic is the map plus one touch of the tally.  Pass
   * this flag when the application manages L2 persistence itself. */
  NMC_FLAG_NO_L2_PERSIST = 1u << 7
};

typedef struct nmc_ext {
  uint32_t size;                 /* sizeof(nmc_ext); set by nmc_ext_defaults */
  uint32_t rng;                  /* NMC_RNG_* */
  uint64_t seed;                 /* Philox key */
  uint32_t phase;                /* NMC_PHASE_* (mcsub only) */
  uint32_t flags;                /* NMC_FLAG_* */
  uint64_t photons_per_dispatch; /* PHOTON_BATCH */
  uint64_t photons_total;        /* PHOTON_TOTAL (CLI and normalisation) */
  /* mcsub geometry and beam: compile-time #defines in the reference
   * (definitions.h:30-54), run-time here. */
  int32_t sub_bins;              /* BINS: bins 1..BINS, BINS = overflow */
  float sub_dr, sub_dz;
  int32_t sub_mcflag;            /* 0 collimated, 1 Gaussian focus, 2 isotropic point */
  int32_t sub_boundaryflag;      /* 0 infinite, 1 air/tissue surface */
  float sub_radius, sub_waist, sub_zfocus, sub_xs, sub_ys, sub_zs;
  /* launch shape; 0 = chosen by the runtime */
  int32_t block_size;
  int32_t blocks_per_sm;
  double timeout_s;              /* host wait limit per call */
  /* voxel and mcsub kernels: consecutive photons a thread takes from the
   * work queue at a time, rounded down to a power of two up to 64 (0 or 1:
   * one); results do not depend on it */
  uint32_t photons_per_fetch;
  uint32_t reserved[7];
} nmc_ext;

/* Totals since nmc_prepare / nmc_reset.  Sums are un-normalised weights. */
typedef struct nmc_summary {
  uint64_t photons;      /* photons completed */
  uint64_t substeps;     /* mcsub hops / mcxyz voxel sub-steps, counted on the device */
  uint64_t scatters;     /* SPIN events */
  double S, A, E;        /* specular, absorbed, escaped weight (SAE of MCSubKernel) */
  double rd_sum;         /* sum over photons of detected weight */
  double rd_sumsq;       /* sum over photons of (detected weight)^2 */
  double kernel_ms;      /* device time of transport launches (CUDA events) */
  uint32_t launches;     /* transport kernel launches */
  uint32_t device_flags; /* NMC_DEVFLAG_* raised by kernels */
} nmc_summary;

enum {
  NMC_DEVFLAG_STEPCAP = 1u << 0,
  NMC_DEVFLAG_BADTISSUE = 1u << 1,
  NMC_DEVFLAG_REPLAY = 1u << 2, /* an adjoint replay did not reproduce a photon's recorded detections */
  NMC_DEVFLAG_BOUNDS = 1u << 3  /* checked build only: an index fell outside its buffer (access skipped) */
};

/* FP64 tallies readable with nmc_get_tally_f64. */
typedef enum nmc_tally {
  NMC_TALLY_J = 0,        /* mcsub escaping flux J[ir], BINS+1 values (index 0 unused) */
  NMC_TALLY_F = 1,        /* mcsub F[ir*BINS+iz], (BINS+1)^2 values */
  NMC_TALLY_F3D = 2,      /* mcxyz deposition, Nx*Ny*Nz, index iz*Ny*Nx + ix*Ny + iy */
  NMC_TALLY_RD2D = 3,     /* mcxyz detected weight map, Nx*Ny, index ix*Ny + iy */
  NMC_TALLY_DETPHOT2D = 4,/* mcxyz detected photon counts, Nx*Ny */
  NMC_TALLY_RD_SLOTS = 5, /* per dispatch slot Rd (kernels.metal:753), photons_per_dispatch */
  NMC_TALLY_RD_R = 6      /* radial Rd(r) at the detection plane, bins + 1 (last = overflow) */
} nmc_tally;

/* Per-photon record written by nmc_run_traced (parity tests). */
typedef struct nmc_photon_record {
  uint32_t n_scatt;   /* SPIN events */
  uint32_t n_sub;     /* mcsub hops / mcxyz voxel sub-steps */
  uint32_t fate;      /* NMC_FATE_* */
  uint32_t n_detect;  /* detection events */
  float w_final;      /* weight when the photon died */
  float absorbed;     /* sum of dropped weight (including outside the grid) */
  float detected;     /* escaped (mcsub E) or detected (mcxyz Rd_loc) weight */
  float x, y, z;      /* final position */
} nmc_photon_record;

enum {
  NMC_FATE_ALIVE = 0,
  NMC_FATE_ESCAPED = 1,   /* mcsub escape through the surface */
  NMC_FATE_ROULETTE = 2,  /* lost the roulette */
  NMC_FATE_MINWEIGHT = 3, /* W < MIN_VALUE (kernels.metal:747) */
  NMC_FATE_MAXSCATT = 4,  /* num_scatt > MAX_SCATT (kernels.metal:747) */
  NMC_FATE_BOUNDARY = 5,  /* left the grid (boundaryflag 1/2) or z < 0 (two-term) */
  NMC_FATE_STEPCAP = 6    /* device-side step cap (not a reference behaviour) */
};

/* ------------------------------------------------------------- lifecycle */
typedef struct nmc_handle nmc_handle;

/* Defaults equal to the reference's compile-time constants. */
void nmc_ext_defaults(nmc_ext* ext);

/* ABI version of the loaded library (NMC_ABI_VERSION). */
int32_t nmc_abi_version(void);

/* Replaces -[MetalMC initWithDevice::] (MetalMC.h:26, MetalMC.m:96-177):
 * selects the transport kernel for `sim_type` (an nmc_sim_type) on CUDA
 * device `device`.  Kinds whose reference kernel is an empty stub
 * (kernels.metal:1122-1202) return NMC_EUNSUPPORTED. */
nmc_status nmc_create(int32_t sim_type, int32_t device, nmc_handle** out);

/* Replaces -[MetalMC prepareData:::] (MetalMC.h:27, MetalMC.m:179-383):
 * copies the run and tissue parameters and, for the voxel kinds, the
 * Nx*Ny*Nz uint8 tissue map (index iz*Ny*Nx + ix*Ny + iy) to the device and
 * clears all tallies.  `v` may be NULL for mcsub. */
nmc_status nmc_prepare(nmc_handle* h, const nmc_run_params* rp,
                       const nmc_tissue_params* tp, const uint8_t* v);

/* Swaps the tissue table of a prepared handle (e.g. the next wavelength)
 * without re-sending the map; tallies are kept (nmc_reset clears them).
 * The tissues the map uses must have finite mua >= 0, mus > 0 and phase
 * terms, as in nmc_prepare. */
nmc_status nmc_set_tissue_params(nmc_handle* h, const nmc_tissue_params* tp);

/* Extension knobs (RNG, phase function, mcsub bins and beam, launch shape).
 * Call before nmc_prepare or between runs; defaults from nmc_ext_defaults. */
nmc_status nmc_set_ext(nmc_handle* h, const nmc_ext* ext);

/* Replaces -[MetalMC setNumRunsSeed::] (MetalMC.h:30, MetalMC.m:498-505).
 * The next nmc_send_compute_command simulates photons
 * [(run-1)*photons_per_dispatch, run*photons_per_dispatch).  The reference
 * never reads time_seed (its kernels seed from run and thread index only);
 * it is accepted and ignored. */
nmc_status nmc_set_num_runs_seed(nmc_handle* h, int32_t run, float time_seed);

/* Replaces -[MetalMC sendComputeCommand] (MetalMC.h:28, MetalMC.m:385-496):
 * one blocking dispatch of photons_per_dispatch photons. */
nmc_status nmc_send_compute_command(nmc_handle* h);

/* Simulates photons [first_photon, first_photon + n_photons) with one
 * persistent launch and waits for it.  Tallies accumulate. */
nmc_status nmc_run(nmc_handle* h, uint64_t first_photon, uint64_t n_photons);

/* Same as nmc_run but returns as soon as the work is queued on the handle's
 * stream; nmc_synchronize waits for it. */
nmc_status nmc_run_async(nmc_handle* h, uint64_t first_photon, uint64_t n_photons);
nmc_status nmc_synchronize(nmc_handle* h);

/* nmc_run that also writes one nmc_photon_record per photon into `recs`
 * (n_photons entries) and, when `events` is not NULL, the (x, y, z, W)
 * state after each of the first `k_events` SPIN events of every photon
 * (n_photons * k_events * 4 floats, unused entries NaN). */
nmc_status nmc_run_traced(nmc_handle* h, uint64_t first_photon, uint64_t n_photons,
                          nmc_photon_record* recs, float* events, uint32_t k_events);

/* Replaces -[MetalMC getComputeResults:...] (MetalMC.h:29, MetalMC.m:508-824):
 * ADDS (+=) the device tallies accumulated since nmc_prepare / nmc_reset into
 * the caller's arrays, in the reference's layouts:
 *   J          BINS+1 floats, J[ir], ir = 1..BINS
 *   F          (BINS+1)*(BINS+1) floats, F[ir*BINS + iz], ir, iz = 1..BINS
 *              (the reference sizes these BINS and BINS*BINS and writes one
 *              bin past them, kernels.metal:202-234; here they are sized to
 *              hold every index the formula produces)
 *   F3D        Nx*Ny*Nz floats, F3D[iz*Ny*Nx + ix*Ny + iy]
 *   SAE        3 floats: specular, absorbed, escaped weight (mcsub)
 *   Rd         photons_per_dispatch floats, per dispatch slot
 *   Rd2D       Nx*Ny floats, DetPhot2D Nx*Ny ints, index ix*Ny + iy
 *   Pol*, Phase*, PolVsScatt: outputs of the empty polarisation kernel;
 *              left untouched.
 * Any pointer may be NULL; arrays a kind does not produce are left untouched. */
nmc_status nmc_get_compute_results(nmc_handle* h, float* J, float* F, float* F3D,
                                   float* SAE, float* Rd, float* Rd2D,
                                   int32_t* DetPhot2D, float* PolXX, float* PolXY,
                                   float* PolYX, float* PolYY, float* Phase0,
                                   float* Phase1, float* Phase2, float* Phase3,
                                   float* PolVsScatt);

/* Totals, sums and timing since nmc_prepare / nmc_reset. */
nmc_status nmc_get_summary(nmc_handle* h, nmc_summary* out);

/* Copies one FP64 tally (see nmc_tally for sizes and layouts) into `out`,
 * which holds `n` doubles; n must equal the tally's size. */
nmc_status nmc_get_tally_f64(nmc_handle* h, int32_t which, double* out, size_t n);

/* Number of doubles in tally `which` for the prepared configuration. */
size_t nmc_tally_size(nmc_handle* h, int32_t which);

/* Clears all tallies and counters; keeps the prepared inputs. */
nmc_status nmc_reset(nmc_handle* h);

/* Tallies accumulate as 64-bit fixed point on the device (32 fractional
 * bits: integer sums, the same whatever the thread order).  Before a bin
 * could wrap, the library folds every tally into an FP64 carry, in stream
 * order: by default after each 2^31 photons, and a longer run is launched in
 * pieces of that size.  Results read back include the carries.  This sets
 * the interval in photons, in [1, 2^31] (no counterpart in the reference,
 * whose float atomics lose precision instead). */
nmc_status nmc_set_fold_interval(nmc_handle* h, uint64_t photons);

/* The cudaStream_t the handle launches on (for timing and overlap). */
void* nmc_stream(nmc_handle* h);

/* Text of the last error on this handle ("" if none). */
const char* nmc_last_error(const nmc_handle* h);

/* Frees the handle and its device memory. */
void nmc_destroy(nmc_handle* h);

/* ------------------------------------------ per-voxel media and adjoint */
/* Gives every voxel its own absorption, scattering and HG anisotropy
 * (Nx*Ny*Nz floats each, index iz*Ny*Nx + ix*Ny + iy; g may be NULL to use
 * gv[1] everywhere).  No reference counterpart: the reference indexes at
 * most 18 tissue types through the uint8 map (definitions.h:57).  From this
 * call on, an NMC_SIM_MCXYZ handle ignores its tissue map (Philox streams,
 * one-term HG).  Requires mua >= 0, mus > 0, -1 < g < 1, all finite. */
nmc_status nmc_set_voxel_props(nmc_handle* h, const float* mua, const float* mus, const float* g);

/* Adds a radial reflectance tally Rd(r): detected weight binned by the
 * distance from the z axis where it leaves the detection plane, `bins` bins
 * of width `dr` plus one overflow bin (NMC_TALLY_RD_R). */
nmc_status nmc_set_radial_tally(nmc_handle* h, int32_t bins, float dr);

/* Perturbation Monte Carlo adjoint of the radial reflectance for per-voxel
 * media.  nmc_adjoint_forward runs photons [first, first+n) like nmc_run and
 * also records every detection event (photon, radial bin, weight); up to
 * `event_capacity` events are kept (NMC_EINVAL if more occurred).
 * nmc_adjoint_backward takes the upstream gradient dL/dRdr[b] of the
 * un-normalised radial tally (bins + 1 floats) and replays the detected
 * photons of the last forward to return, per voxel,
 *   grad_mua = dL/dmua, grad_mus = dL/dmus, grad_g = dL/dg
 * (Nx*Ny*Nz doubles each, any may be NULL), the path-length and
 * likelihood-ratio estimator of the same photons. */
nmc_status nmc_adjoint_forward(nmc_handle* h, uint64_t first, uint64_t n, uint64_t event_capacity);
/* As nmc_adjoint_forward, and also keeps the deposit list of the photons:
 * every (voxel, absorbed weight) the run adds to NMC_TALLY_F3D, merged per
 * visit of a photon to a voxel, room for `deposit_capacity` records of 8
 * bytes (about 0.7 records per voxel sub-step; 0 keeps none) plus one
 * 2 KB chunk per thread of the launch.  With the list
 * a backward with a deposit gradient gets each photon's total score from it
 * instead of replaying every photon for it.  A list that outgrows its
 * capacity is dropped, and that backward replays the scores as without one.
 * No reference counterpart. */
nmc_status nmc_adjoint_forward_ex(nmc_handle* h, uint64_t first, uint64_t n, uint64_t event_capacity,
                                  uint64_t deposit_capacity);
/* 1 if the last adjoint forward kept a complete deposit list, else 0. */
int32_t nmc_adjoint_deposit_list_complete(nmc_handle* h);
nmc_status nmc_adjoint_backward(nmc_handle* h, const float* grad_rd_r, double* grad_mua,
                                double* grad_mus, double* grad_g);
/* As nmc_adjoint_backward, with the upstream gradient of the absorbed-weight
 * tally too (NMC_TALLY_F3D of the forward's photons, Nx*Ny*Nz floats; the
 * fluence is that tally / (mua * photons * voxel volume), whose chain rule
 * stays with the caller).  Either gradient may be NULL, not both.  With a
 * deposit gradient the detected photons are not enough: every photon is
 * replayed, after its total score is summed from the forward's deposit list
 * (nmc_adjoint_forward_ex) or, without one, from a first replay. */
nmc_status nmc_adjoint_backward_ex(nmc_handle* h, const float* grad_rd_r, const float* grad_absorbed,
                                   double* grad_mua, double* grad_mus, double* grad_g);

/* ---------------------------------- polarised E-field, CBS cone and Raman */
/* The reference's NMC_SIM_POLARIZATION_CBS_ELECTRIC_FIELDS and NMC_SIM_RAMAN
 * kernels are empty (kernels.metal:1122-1202); nmc_create still refuses those
 * kinds.  These entry points are this engine's own polarised transport for a
 * semi-infinite slab of spheres; the per-pixel outputs mirror the buffers the
 * reference host allocates for that kind (MetalMC.m:206-328: PolXX/XY/YX/YY,
 * Rd2D, DetPhot2D, Phase0-3 maps and PolVsScatt[4][MAX_SCATT_POL]). */

/* Mie amplitudes of a homogeneous sphere (size parameter x = 2 pi n_medium a
 * / lambda, relative index m = m_re + i m_im): S is n_angles x 4 floats
 * (Re S1, Im S1, Re S2, Im S2) at theta_j = j pi / (n_angles - 1); efficiencies
 * and the asymmetry g.  Any output may be NULL. */
nmc_status nmc_mie(double x, double m_re, double m_im, int32_t n_angles, float* S, double* q_ext,
                   double* q_sca, double* g);

typedef struct nmc_efield_config {
  float mua, mus;             /* primary wavelength, cm^-1 */
  float wavelength_cm;        /* primary vacuum wavelength */
  float raman_mua, raman_mus; /* at the Raman wavelength, cm^-1 */
  float raman_wavelength_cm;
  float mu_raman;             /* conversion coefficient, cm^-1 (0: none) */
  float n_medium, n_outside;  /* refractive indices */
  int32_t n_angles;           /* rows of both S tables (>= 2) */
  int32_t cone_n;             /* backscattering cone grid, cone_n x cone_n (2..1024) */
  float cone_half_angle;      /* rad, in air */
  int32_t sep_n;              /* first-to-last scattering separation histogram, bins per axis (2..4096) */
  float sep_half_width;       /* cm */
  int32_t map_n;              /* exit maps, map_n x map_n pixels centred on the beam (1..1024) */
  float map_dx;               /* cm per pixel */
  int32_t depth_bins;         /* Raman conversion depth histogram (1..4096) */
  float depth_dz;             /* cm per bin */
  uint64_t seed;
  uint32_t flags;             /* NMC_FLAG_PRECISE_MATH */
  uint32_t speckle_max;       /* speckle records kept per exit-map pixel (0: none; the
                                 reference's MAX_SPECKLES_PER_PIXEL is 1000) */
} nmc_efield_config;

typedef struct nmc_efield_setting {
  float pol_angle;         /* azimuth of the incident linear polarisation (rad, from x) */
  float theta_in, phi_in;  /* incidence direction in air (rad; 0 = normal) */
  uint32_t pad;
  uint64_t photons;
} nmc_efield_setting;
#ifdef __cplusplus
static_assert(sizeof(nmc_efield_config) == 88, "nmc_efield_config layout");
static_assert(sizeof(nmc_efield_setting) == 24, "nmc_efield_setting layout");
#endif

/* Per-setting results of nmc_efield_run, NMC_EF_FIELDS doubles per setting.
 * "co" / "cross": analyser parallel / perpendicular to the incident
 * polarisation; "multi": photons scattered at least twice, the part that
 * interferes with its time-reversed path; "interf": the interference term at
 * exact backscattering, sum of w Re(E conj(E_reversed)). */
enum {
  NMC_EF_PHOTONS = 0, NMC_EF_SPECULAR, NMC_EF_RD, NMC_EF_RD2, NMC_EF_CO, NMC_EF_CROSS,
  NMC_EF_MULTI_CO, NMC_EF_MULTI_CROSS, NMC_EF_INTERF_CO, NMC_EF_INTERF_CROSS, NMC_EF_SEP_OUTSIDE,
  NMC_EF_RAMAN_N, NMC_EF_RAMAN_RD, NMC_EF_RAMAN_CO, NMC_EF_RAMAN_CROSS, NMC_EF_SCATTERS,
  NMC_EF_FIELDS
};
/* Exit maps, map_n^2 floats each, index ix*map_n + iy. */
enum {
  NMC_EF_MAP_XX = 0, NMC_EF_MAP_XY, NMC_EF_MAP_YX, NMC_EF_MAP_YY, NMC_EF_MAP_RD, NMC_EF_MAP_DET,
  NMC_EF_MAP_PHASE0, NMC_EF_MAP_PHASE1, NMC_EF_MAP_PHASE2, NMC_EF_MAP_PHASE3, NMC_EF_MAPS
};
#define NMC_EF_MAX_ORDER 150 /* PolVsScatt orders 0..150, MAX_SCATT_POL (definitions.h:25) */

/* One detected photon at an exit-map pixel, struct SPECKLE of
 * definitions.h:220-229 (same fields, same order): Phase = arg of the
 * co-polarised amplitude, Path = path phase 2 pi n L / lambda (wrapped),
 * Scatt = arg of the cross-polarised amplitude, Total = Phase + Path
 * (wrapped), XX / XY = intensity of an x-polarised input in the x / y
 * analyser, Ryx = the photon's weight. */
typedef struct nmc_speckle {
  float Phase, Path, Scatt, Total, XX, XY, Ryx;
} nmc_speckle;
#ifdef __cplusplus
static_assert(sizeof(nmc_speckle) == 28, "nmc_speckle layout (struct SPECKLE)");
#endif

/* Runs every setting's photons in one persistent launch on `device`.
 * S_primary / S_raman: n_angles x 4 Mie tables at the two wavelengths.
 * Outputs (any but `out` may be NULL), per setting s:
 *   out[s*NMC_EF_FIELDS + k];
 *   cone[((s*2 + c)*cone_n + i)*cone_n + j] as complex (2 floats): the
 *     interference field of channel c (0 co, 1 cross) at angles
 *     (theta_x, theta_y) = (-h + (i + 0.5) 2h/cone_n, -h + (j + 0.5) 2h/cone_n);
 *     the cone intensity is multi + Re(cone);
 *   pol_vs_scatt[(s*4 + ch)*(NMC_EF_MAX_ORDER+1) + n]: XX, XY, YX, YY
 *     intensity escaping after n scatterings (n capped);
 *   maps[(s*NMC_EF_MAPS + m)*map_n*map_n + ...];
 *   raman_depth[s*depth_bins + b]: weight converted at depth b*dz.
 * At most 2^53 photons over all settings (counts are summed in FP64);
 * NMC_EINVAL beyond. */
nmc_status nmc_efield_run(int32_t device, const nmc_efield_config* cfg, const float* S_primary,
                          const float* S_raman, const nmc_efield_setting* settings, int32_t n_settings,
                          double* out, float* cone, double* pol_vs_scatt, float* maps, double* raman_depth,
                          nmc_speckle* speckles, int32_t* speckle_counts);
/* (speckles: with speckle_max > 0 and maps, records of the first
 * speckle_max photons reaching each pixel, at
 * ((s*speckle_max + k)*map_n + ix)*map_n + iy; speckle_counts[s*map_n^2 +
 * ix*map_n + iy] how many; both may be NULL.) */

/* The reference's speckle mutual-interference post-processing
 * (MetalMC.m:628-742) on the GPU: for each pixel of an nx x ny map, the
 * pixel's mean (from the accumulated maps and photon counts) interferes with
 * each of its `counts[p]` speckle records (records[k*nx*ny + p], p = ix*ny +
 * iy, k < max_records) with the path-difference coherence envelope
 * exp(-((path_k - path_mean) lambda / (2 pi lc))^2) (0 when lc <= 0.01);
 * the mutual sums are added (+=) to out_maps (NMC_EF_MAPS maps of nx*ny,
 * XX, XY, Rd, Det and Phase0-3 updated as the reference updates them).
 * `maps` holds the accumulated maps in the same layout.  Host pointers. */
nmc_status nmc_speckle_mutual(int32_t device, int32_t nx, int32_t ny, const float* maps,
                              const nmc_speckle* records, const int32_t* counts, int32_t max_records,
                              float lambda, float lc, float* out_maps);

/* ------------------------------------------------------ layered mcsub */
/* A stack of plane layers (MAXLAYERS = 100, definitions.h:24, declared by
 * the reference but unused): the mcsub kernel's hop / drop / spin /
 * roulette per layer, Fresnel reflection or Snell refraction at every
 * boundary, escape into the ambient media above (Rd) and below (Tt).
 * thickness is in cm; the last layer may be semi-infinite (INFINITY), then
 * it needs mua + mus > 0.  Normal pencil beam at the origin. */
typedef struct nmc_layer {
  float mua, mus, g, n, thickness;
} nmc_layer;

typedef struct nmc_layered_config {
  int32_t n_layers;            /* 1..100 */
  float n_above, n_below;      /* ambient refractive indices */
  int32_t nr;                  /* Rd(r), Tt(r), A(r,z): nr bins of dr + one overflow bin */
  float dr;
  int32_t nz;                  /* A(z): nz bins of dz + one overflow bin */
  float dz;
  uint32_t flags;              /* NMC_FLAG_PRECISE_MATH, NMC_FLAG_LAYERED_REF_STREAMS,
                                  NMC_FLAG_LAYERED_ISOTROPIC */
  uint64_t seed;               /* Philox key; the dispatch batch with
                                  NMC_FLAG_LAYERED_REF_STREAMS */
} nmc_layered_config;
#ifdef __cplusplus
static_assert(sizeof(nmc_layer) == 20, "nmc_layer layout");
static_assert(sizeof(nmc_layered_config) == 40, "nmc_layered_config layout");
#endif

/* Per-run sums of nmc_layered_run (weights, not yet divided by photons). */
enum {
  NMC_LAY_PHOTONS = 0, NMC_LAY_SPECULAR, NMC_LAY_RD, NMC_LAY_RD2, NMC_LAY_TT, NMC_LAY_TT2, NMC_LAY_A,
  NMC_LAY_INTERACTIONS, NMC_LAY_FIELDS
};

/* Photons [first, first + photons) through the stack on `device` (at most
 * 2^31 per call; results add up over calls); out holds
 * NMC_LAY_FIELDS doubles; rd_r, tt_r (nr+1), a_z (nz+1), a_rz ((nr+1)*(nz+1),
 * index ir*(nz+1) + iz) and a_layer (n_layers) are added to (+=) and may be
 * NULL.  Host pointers. */
nmc_status nmc_layered_run(int32_t device, const nmc_layered_config* cfg, const nmc_layer* layers,
                           uint64_t first, uint64_t photons, double* out, double* rd_r, double* tt_r,
                           double* a_z, double* a_rz, double* a_layer);

/* The same run with per-layer gradients of L = sum_b grad_rd_r[b] rd_r[b] +
 * sum_b grad_tt_r[b] tt_r[b] (un-normalised tallies; either gradient may be
 * NULL, not both): grad_mua, grad_mus, grad_g (n_layers each, +=) from the
 * path length, interaction count and d ln p_HG/dg each photon collects per
 * layer (perturbation Monte Carlo; at most 16 layers). */
nmc_status nmc_layered_adjoint(int32_t device, const nmc_layered_config* cfg, const nmc_layer* layers,
                               uint64_t first, uint64_t photons, const float* grad_rd_r, const float* grad_tt_r,
                               double* out, double* rd_r, double* tt_r, double* grad_mua, double* grad_mus,
                               double* grad_g);

/* -------------------------------------------------------------- autotune */
/* One launch configuration the autotuner timed. */
typedef struct nmc_tune_entry {
  int32_t block_size, blocks_per_sm;
  uint32_t flags;             /* NMC_FLAG_GLOBAL_TALLIES or 0 */
  uint32_t photons_per_fetch; /* photons a thread takes from the queue at a time */
  float ms;                   /* kernel time of the tuning run */
} nmc_tune_entry;

typedef struct nmc_tune_result {
  nmc_tune_entry best, fallback; /* chosen; the defaults (block 0 / blocks 0) */
  int32_t n_tried;
  nmc_tune_entry tried[48];
} nmc_tune_result;
#ifdef __cplusplus
static_assert(sizeof(nmc_tune_result) == 1004, "nmc_tune_result layout");
#endif

/* Times the handle's kernel on photons [0, photons) under each candidate
 * launch configuration (block size; resident blocks per SM, i.e. photons in
 * flight per SM; photons a thread takes from the work queue at a time; for
 * mcsub, tallies privatised in shared memory or not), keeps the fastest in
 * the handle's nmc_ext (block_size, blocks_per_sm, photons_per_fetch, flags) and
 * clears the tallies.  Results do not depend on the configuration: every
 * photon's stream is a function of its id only.  No reference counterpart
 * (the reference dispatches 1e4 threads in threadgroups of the pipeline's
 * maximum, MetalMC.m:485-495). */
nmc_status nmc_autotune(nmc_handle* h, uint64_t photons, nmc_tune_result* out);

/* ------------------------------------------------------- batched sweeps */
/* One parameter set of a batched sweep (e.g. one wavelength) on the mcsub
 * geometry (semi-infinite medium, the handle's nmc_ext beam, bins and phase
 * function).  Replaces one `nmc` process per wavelength
 * (NMC-samples/example3.ipynb cell 5 rewrites _H.mci and relaunches nmc for
 * every wavelength). */
typedef struct nmc_sweep_set {
  float mua, mus;           /* cm^-1 */
  float g;                  /* HG anisotropy (phase NMC_PHASE_HG) */
  float gf, af, gb, ab, cc; /* two-term parameters (NMC_PHASE_TWO_TERM) */
  float n1, n2;             /* tissue / outside refractive index */
  uint32_t pad;
  uint64_t photons;         /* photon budget of this set */
  uint64_t first_photon;    /* id of the set's first photon (0, or where a
                               previous sweep of this set stopped) */
} nmc_sweep_set;

/* Per-set results of nmc_run_sweep, NMC_SWEEP_FIELDS doubles per set. */
enum {
  NMC_SWEEP_PHOTONS = 0,  /* photons completed */
  NMC_SWEEP_HOPS = 1,     /* hops (steps) */
  NMC_SWEEP_S = 2,        /* specular weight */
  NMC_SWEEP_A = 3,        /* absorbed weight */
  NMC_SWEEP_E = 4,        /* escaped weight */
  NMC_SWEEP_E2 = 5,       /* sum over photons of escaped weight squared */
  NMC_SWEEP_RD = 6,       /* Rd = (S + E) / photons, as main.m:238-242 */
  NMC_SWEEP_RD_SE = 7,    /* standard error of Rd */
  NMC_SWEEP_FIELDS = 8
};

/* Runs every set's photon budget in one persistent launch on a handle made
 * with NMC_SIM_MCSUB (nmc_prepare called; its tissue layer is replaced by
 * the sets).  Photons of set s use Philox key (seed lo, seed hi + s), so set
 * s reproduces a plain run with seed + (s << 32).  `out` holds n_sets *
 * NMC_SWEEP_FIELDS doubles; `J` (optional) n_sets * (BINS+1) doubles of the
 * escaping flux J[ir] per set (un-normalised).  At most 2^31 photons per set
 * and call (the per-set fixed-point sums stay below 2^63).  The launch hands the sets
 * out in decreasing estimated cost per photon (mu_t / mu_a), which shortens
 * its tail and changes no result. */
nmc_status nmc_run_sweep(nmc_handle* h, const nmc_sweep_set* sets, int32_t n_sets, double* out,
                         double* J);

/* Batched sweep on a voxel tissue map: set s runs photons[s] photons with
 * its own tissue table tables[s] (all 19 entries as in nmc_prepare; the
 * handle's map, geometry, beam and kernel kind stay) in one persistent
 * launch on a handle made with NMC_SIM_MCXYZ or NMC_SIM_MCXYZ_TT.  Photons
 * of set s are ids first_photon[s] .. first_photon[s] + photons[s] - 1
 * (first_photon may be NULL: all 0) under Philox key (seed lo, seed hi + s),
 * so set s reproduces a plain run of those ids with seed + (s << 32).
 * Replaces one `nmc` process per wavelength on the skin-vessel map
 * (NMC-samples/example3.ipynb cell 5).  `out` holds n_sets *
 * NMC_SWEEP_FIELDS doubles: HOPS counts voxel sub-steps, S is 0, E the
 * detected weight, RD = E / photons (the run's Total Rd, main.m:294-305).
 * No map tallies (F3D, Rd2D) are kept.  At most 2^31 photons per set and
 * call.  The launch hands the sets out in
 * decreasing estimated cost per photon (sum over the map's tissues of
 * voxels * (mus + 1/d) / mua), which shortens its tail and changes no
 * result. */
nmc_status nmc_run_sweep_tissues(nmc_handle* h, const nmc_tissue_params* tables, const uint64_t* photons,
                                 const uint64_t* first_photon, int32_t n_sets, double* out);

/* Measurement support (no counterpart in the reference): FP32 FMA lanes per
 * second and MUFU (ex2) lanes per second sustained on `device`, the issue
 * ceilings that bound the transport kernels. */
nmc_status nmc_probe_issue_peaks(int32_t device, double* ffma_lanes_per_s,
                                 double* mufu_lanes_per_s);

/* Largest grid nmc_mcxyz_run_noalloc accepts. */
#define NMC_NOALLOC_MAX_VOXELS 2097152u /* Nx*Ny*Nz, e.g. 128^3 */
#define NMC_NOALLOC_MAX_MAP 65536u      /* Nx*Ny, e.g. 256^2 */
/* Most photons nmc_mcxyz_run_noalloc takes in one call (its fixed-point
 * sums are not folded within a call). */
#define NMC_NOALLOC_MAX_PHOTONS 2147483648ull /* 2^31 */

/* Voxel transport that allocates no memory.  No counterpart in the
 * reference.
 *
 * For callers that cannot let a library call cudaMalloc: an application
 * that hands out device memory only from its own pool, a plugin living
 * inside another runtime's fixed memory budget, or a real-time loop where an
 * allocation may neither stall nor fail.  The caller owns every buffer it
 * passes, all on the current device: the uint8 tissue map `d_v`
 * (Nx*Ny*Nz, index iz*Ny*Nx + ix*Ny + iy) and the outputs `d_F3D`
 * (Nx*Ny*Nz floats), `d_Rd2D` (Nx*Ny floats, may be NULL), `d_DetPhot2D`
 * (Nx*Ny counts, may be NULL) and `d_totals` (8 doubles, may be NULL:
 * photons, sub-steps, SPIN events, absorbed weight, detected weight, sum of
 * squared detected weight per photon, device flags, 0).  Outputs are
 * overwritten with the tallies of photons [first_photon, first_photon +
 * n_photons), unnormalised, exactly as nmc_run followed by
 * nmc_get_tally_f64 would give them for a fresh handle.  rp->mckernelflag
 * selects MCXYZ or MCXYZ_TT; `ext` gives the RNG, seed and flags.
 *
 * The library's working memory for this call (u64 tallies, photon counter,
 * totals; about 17 MB) is one fixed array in device memory that every GPU
 * loading the library holds until the process exits; grids beyond
 * NMC_NOALLOC_MAX_VOXELS voxels or NMC_NOALLOC_MAX_MAP columns are rejected
 * with NMC_EINVAL, and so are calls of more than NMC_NOALLOC_MAX_PHOTONS
 * photons (2^31: the u64 fixed-point sums and u32 counts of one call are
 * never folded into FP64 the way nmc_run folds them, so a larger call could
 * wrap) or whose photon ids would pass 2^64; these size checks come before
 * any device call.  The launch shape follows ext->block_size and
 * ext->blocks_per_sm as nmc_run's does.  Every call reuses that array and clears it first, so
 * calls whose GPU work overlaps (two streams, two host threads) race and
 * must be serialised by the caller.  The first call on a device looks up the
 * array's device address (once per device, with that device current); make
 * that first call before any stream capture.  The call checks the tissue
 * map on the GPU and waits on `stream` for that check once, then queues the
 * transport and the output conversion on `stream` and returns. */
nmc_status nmc_mcxyz_run_noalloc(const nmc_run_params* rp, const nmc_tissue_params* tp,
                                 const nmc_ext* ext, const uint8_t* d_v,
                                 uint64_t first_photon, uint64_t n_photons, float* d_F3D,
                                 float* d_Rd2D, uint32_t* d_DetPhot2D, double* d_totals,
                                 void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NMC_ABI_H */
