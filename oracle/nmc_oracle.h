/*
 * nmc_oracle.h - C API of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain CPU restatement of the
 * reference's photon kernels (NMC/NMCCode/kernels.metal MCSubKernel,
 * MCXYZKernel, MCXYZKernelTT and the helpers.metal routines they call), run
 * in FP64 (or FP32) with either the Philox streams the GPU engine uses or the
 * reference's own Tausworthe generator.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU baseline call it; the product never links it.
 */
#ifndef NMC_ORACLE_H
#define NMC_ORACLE_H

#include <stdint.h>

#include "nmc_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output accumulators (+=).  Any array pointer may be NULL.  Sizes as in
 * nmc_tally: J BINS+1, F (BINS+1)^2, F3D Nx*Ny*Nz, Rd2D / DetPhot2D Nx*Ny,
 * rd_slots photons_per_dispatch. */
typedef struct orc_out {
  double* J;
  double* F;
  double* F3D;
  double* Rd2D;
  double* DetPhot2D;
  double* rd_slots;
  double S, A, E;          /* specular / absorbed / escaped weight */
  double rd_sum, rd_sumsq; /* per-photon detected weight */
  double photons, substeps, scatters;
} orc_out;

/* Simulates photons [first, first + n) of kind `sim_type` (nmc_sim_type
 * MCSUB / MCXYZ / MCXYZ_TT) with `real_bits` 64 (double) or 32 (float)
 * arithmetic on `nthreads` host threads.  `recs` (n entries) and `events`
 * (n * k_events * 4 floats) are optional per-photon traces with the same
 * meaning as nmc_run_traced.  Returns 0 or an nmc_status. */
int orc_run(int sim_type, int real_bits, const nmc_run_params* rp,
            const nmc_tissue_params* tp, const uint8_t* v, const nmc_ext* ext,
            uint64_t first, uint64_t n, int nthreads, orc_out* out,
            nmc_photon_record* recs, float* events, uint32_t k_events);

/* Philox4x32-10 block function (Salmon et al., SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* First `n` uniforms of photon `photon_id`'s stream for `ext`'s RNG choice
 * (Philox: counter/key layout of nmc_abi.h; Taus: the reference's generator
 * seeded as kernels.metal:91-95 for run/index derived from photon_id). */
void orc_uniforms(const nmc_ext* ext, int sim_type, uint64_t photon_id, int n, double* out);

/* Fresnel reflectance (helpers.metal:243-291) in double. */
double orc_rfresnel(double n1, double n2, double ca1, double* ca2);

/* Two-term cos(theta) sample (kernels.metal:1058-1070) for a given uniform
 * pair, in double. */
double orc_tt_costheta(double gf, double af, double gb, double ab, double cc,
                       double u_choice, double u_sample);

/* Henyey-Greenstein cos(theta) sample (kernels.metal:696-703) in double. */
double orc_hg_costheta(double g, double u);

/* The engine's multi-layer model (nmc_layered_run) restated on the CPU, same
 * Philox layout, or the reference's streams and isotropic phase under the
 * config's NMC_FLAG_LAYERED_* flags; out (NMC_LAY_FIELDS) and the tallies are
 * added to (+=) and may be NULL except out; per_photon (may be NULL) gets
 * (escaped up, escaped down, absorbed) weight per photon, 3 doubles each.
 * Returns 0, NMC_EINVAL or NMC_ESTEPCAP. */
int orc_layered_run(int real_bits, const nmc_layered_config* cfg, const nmc_layer* layers, uint64_t first,
                    uint64_t n, int nthreads, double* out, double* rd_r, double* tt_r, double* a_z,
                    double* a_layer, double* per_photon);

/* The engine's polarised E-field model (nmc_efield_run) restated on the CPU,
 * same Philox layout: per setting the NMC_EF_FIELDS sums into `out` (+=;
 * n_settings * NMC_EF_FIELDS doubles; SEP_OUTSIDE only with `cone`).
 * Returns 0 or NMC_EINVAL. */
int orc_efield_run(int real_bits, const nmc_efield_config* cfg, const float* S_primary, const float* S_raman,
                   const nmc_efield_setting* settings, int n_settings, int cone, int nthreads, double* out);

/* MetalMC.m:628-742 speckle mutual interference (see nmc_speckle_mutual). */
void orc_speckle_mutual(int nx, int ny, const float* maps, const nmc_speckle* rec, const int32_t* counts,
                        int kmax, float lambda, float lc, float* out);

#ifdef __cplusplus
}
#endif
#endif
