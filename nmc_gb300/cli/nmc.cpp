// nmc.cpp - the `nmc` command-line program over the GB300 engine.
//
// Drop-in for the reference's `nmc` executable (NMC/NMCCode/main.m:19-564 with
// the file routines of mcio.h:16-389), which the sample notebooks run as a
// subprocess: `nmc <name>` reads <name>_H.mci (one value per line, read with
// fgets into a 32-byte buffer as mcio.h:16-171 does) and <name>_T.bin (raw
// uint8 tissue map), writes <name>_props.m, runs PHOTON_TOTAL photons in
// PHOTON_BATCH dispatches, and writes the reference's outputs with its
// normalisations and printf formats:
//   mcsub:  <name>_Rd.dat ("%0.4f", S + E) and mcOUT0.dat (run parameters,
//           S/A/E, r row, J row, F(z, r) table; main.m:203-262, mcio.h:327-389);
//   mcxyz:  <name>_F.bin (fluence rate, float32, F3D / (dx dy dz N mua[v]),
//           non-finite -> 0), <name>_Rd.dat, <name>_Ryx.dat and
//           <name>_DetPhot2D.dat (tab text, rows of Ny values taken at
//           j + i*Nx as main.m:519-561 does).
// The reference's own generator and stream schedule are the default
// (NMC_RNG_TAUS_REF), so the photons are the reference's.  They run in one
// persistent launch: photon (run r, index i) of the reference's dispatch loop
// (main.m:144-187) is photon (r - 1) * batch + i here and draws the same
// stream, and the tallies are integer sums, so the files equal the loop's bit
// for bit while the GPU waits for one tail instead of one per dispatch.
// Options:
//   --photons N     photons (default PHOTON_TOTAL = 100000, multiple of the batch)
//   --batch B       photons per dispatch (default PHOTON_BATCH = 10000)
//   --philox S      the engine's Philox streams with seed S instead
//   --dispatch      run the reference's loop of photons / batch blocking dispatches
//   --persistent    one persistent launch (the default)
//   --device D      CUDA device (default 0)
//   --dry-run       parse the inputs, print them and write _props.m only
// Besides the reference's files it writes <name>_report.json: photons, kernel
// time, photons/s, Rd with its standard error, sub-steps and scatterings per
// photon (the reference only prints a rate, main.m:199).
// Exit status 0, or 1 with a message (the reference exits 1 on unknown kinds).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nmc_abi.h"

namespace {

constexpr double kPi = 3.1415926;  // PI of definitions.h:60

// One line as fgets(buf, 32, fid) returns it (at most 31 characters, the
// newline kept if it fits), so long lines split exactly as in the reference.
bool next_field(FILE* f, char* buf) {
  return std::fgets(buf, 32, f) != nullptr;
}

bool read_mci(const std::string& name, nmc_run_params& rp, nmc_tissue_params& tp) {
  std::memset(&rp, 0, sizeof rp);
  std::memset(&tp, 0, sizeof tp);
  std::snprintf(rp.myname, sizeof rp.myname, "%s", name.c_str());
  const std::string fn = name + "_H.mci";
  FILE* f = std::fopen(fn.c_str(), "r");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", fn.c_str());
    return false;
  }
  char buf[32];
  bool ok = true;
  auto F = [&](float* v) { ok = ok && next_field(f, buf) && std::sscanf(buf, "%f", v) == 1; };
  auto I = [&](int32_t* v) { ok = ok && next_field(f, buf) && std::sscanf(buf, "%d", v) == 1; };
  F(&rp.time_min);
  I(&rp.Nx);
  I(&rp.Ny);
  I(&rp.Nz);
  F(&rp.dx);
  F(&rp.dy);
  F(&rp.dz);
  I(&rp.mcflag);
  I(&rp.launchflag);
  I(&rp.boundaryflag);
  F(&rp.xs);
  F(&rp.ys);
  F(&rp.zs);
  F(&rp.xfocus);
  F(&rp.yfocus);
  F(&rp.zfocus);
  F(&rp.ux0);
  F(&rp.uy0);
  F(&rp.uz0);
  F(&rp.radius);
  F(&rp.waist);
  F(&rp.zsurf);
  F(&rp.det_radius);
  F(&rp.xd);
  F(&rp.n1);
  F(&rp.n2);
  F(&rp.na);
  F(&rp.lambda);
  F(&rp.lc);
  I(&rp.speckleflag);
  I(&rp.semiflag);
  int32_t det = 0;
  I(&det);
  rp.det_state = det;
  I(&rp.mckernelflag);
  I(&rp.Nt);
  if (ok && (rp.Nt < 0 || rp.Nt >= NMC_NTISS)) {
    std::fprintf(stderr, "Nt = %d out of range\n", rp.Nt);
    ok = false;
  }
  for (int i = 1; ok && i <= rp.Nt; ++i) {
    F(&tp.muav[i]);
    F(&tp.musv[i]);
    if (rp.mckernelflag == NMC_SIM_MCXYZ_TT) {
      F(&tp.gf[i]);
      F(&tp.af[i]);
      F(&tp.gb[i]);
      F(&tp.ab[i]);
      F(&tp.CC[i]);
    } else {
      F(&tp.gv[i]);
    }
  }
  std::fclose(f);
  if (!ok) std::fprintf(stderr, "%s: missing or malformed line\n", fn.c_str());
  return ok;
}

// The file names use the whole <name>; rp.myname keeps its first 31
// characters (the reference copies argv[1] into char[32], mcio.h:22).
void save_props(const std::string& name, const nmc_run_params& rp, const nmc_tissue_params& tp) {  // mcio.h:298-325
  const std::string fn = name + "_props.m";
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) return;
  for (long i = 1; i <= rp.Nt; i++) {
    std::fprintf(f, "muav(%ld) = %0.4f;\n", i, tp.muav[i]);
    std::fprintf(f, "musv(%ld) = %0.4f;\n", i, tp.musv[i]);
    if (rp.mckernelflag == NMC_SIM_MCXYZ_TT) {
      std::fprintf(f, "gf(%ld) = %0.4f;\n\n", i, tp.gf[i]);
      std::fprintf(f, "af(%ld) = %0.4f;\n\n", i, tp.af[i]);
      std::fprintf(f, "gb(%ld) = %0.4f;\n\n", i, tp.gb[i]);
      std::fprintf(f, "ab(%ld) = %0.4f;\n\n", i, tp.ab[i]);
      std::fprintf(f, "CC(%ld) = %0.4f;\n\n", i, tp.CC[i]);
    } else {
      std::fprintf(f, "gv(%ld) = %0.4f;\n\n", i, tp.gv[i]);
    }
  }
  std::fclose(f);
}

void print_params(const nmc_run_params& rp, const nmc_tissue_params& tp) {
  std::printf("name = %s\n", rp.myname);
  std::printf("time_min = %0.2f min\n", rp.time_min);
  std::printf("Nx = %d, dx = %0.4f [mm]\n", rp.Nx, rp.dx);
  std::printf("Ny = %d, dy = %0.4f [mm]\n", rp.Ny, rp.dy);
  std::printf("Nz = %d, dz = %0.4f [mm]\n", rp.Nz, rp.dz);
  std::printf("xs = %0.4f [mm]\nys = %0.4f [mm]\nzs = %0.4f [mm]\n", rp.xs, rp.ys, rp.zs);
  std::printf("mcflag = %d\nlaunchflag = %d\nboundaryflag = %d\nzsurf = %0.4f\n", rp.mcflag, rp.launchflag,
              rp.boundaryflag, rp.zsurf);
  std::printf("n1 = %0.4f\nn2 = %0.4f\nmckernelflag = %d\n", rp.n1, rp.n2, rp.mckernelflag);
  std::printf("# of tissues available, Nt = %d\n", rp.Nt);
  for (int i = 1; i <= rp.Nt; i++) {
    std::printf("muav[%d] = %0.4f\nmusv[%d] = %0.4f\n", i, tp.muav[i], i, tp.musv[i]);
    if (rp.mckernelflag == NMC_SIM_MCXYZ_TT)
      std::printf("gf(%d) = %0.4f; af(%d) = %0.4f; gb(%d) = %0.4f; ab(%d) = %0.4f; CC(%d) = %0.4f;\n", i,
                  tp.gf[i], i, tp.af[i], i, tp.gb[i], i, tp.ab[i], i, tp.CC[i]);
    else
      std::printf("  gv[%d] = %0.4f\n", i, tp.gv[i]);
  }
}

int die(nmc_handle* h, const char* what) {
  std::fprintf(stderr, "%s failed: %s\n", what, h ? nmc_last_error(h) : "");
  if (h) nmc_destroy(h);
  return 1;
}

void save_mcout(const float* J, const float* F, double S, double A, double E, double mua, double mus, double g,
                double n1, double n2, int bins, double dr, double dz, double nph) {  // mcio.h:327-389
  FILE* t = std::fopen("mcOUT0.dat", "w+");
  if (!t) return;
  std::fprintf(t, "%0.3e\tmua, absorption coefficient [1/mm]\n", mua);
  std::fprintf(t, "%0.4f\tmus, scattering coefficient [1/mm]\n", mus);
  std::fprintf(t, "%0.4f\tg, anisotropy [-]\n", g);
  std::fprintf(t, "%0.4f\tn1, refractive index of tissue\n", n1);
  std::fprintf(t, "%0.4f\tn2, refractive index of outside medium\n", n2);
  std::fprintf(t, "%d\tmcflag\n", 0);
  std::fprintf(t, "%0.4f\tradius, radius of flat beam or 1/e radius of Gaussian beam [mm]\n", 0.0);
  std::fprintf(t, "%0.4f\twaist, 1/e waist of focus [mm]\n", 0.10);
  std::fprintf(t, "%0.4f\txs, x position of isotropic source [mm]\n", 0.0);
  std::fprintf(t, "%0.4f\tys, y\n", 0.0);
  std::fprintf(t, "%0.4f\tzs, z\n", 0.0);
  std::fprintf(t, "%d\tNR\n", bins);
  std::fprintf(t, "%d\tNZ\n", bins);
  std::fprintf(t, "%0.5f\tdr\n", dr);
  std::fprintf(t, "%0.5f\tdz\n", dz);
  std::fprintf(t, "%0.1e\tNphotons\n", nph);
  std::fprintf(t, "%1.6e\tSpecular reflectance\n", S);
  std::fprintf(t, "%1.6e\tAbsorbed fraction\n", A);
  std::fprintf(t, "%1.6e\tEscaping fraction\n", E);
  std::fprintf(t, "%0.1f", 0.0);
  for (long ir = 1; ir <= bins; ir++) {
    const double r2 = dr * ir, r1 = dr * (ir - 1);
    std::fprintf(t, "\t%1.5f", 2.0 / 3 * (r2 * r2 + r2 * r1 + r1 * r1) / (r1 + r2));
  }
  std::fprintf(t, "\n%0.1f", 0.0);
  for (long ir = 1; ir <= bins; ir++) std::fprintf(t, "\t%1.12e", J[ir]);
  std::fprintf(t, "\n");
  for (long iz = 1; iz <= bins; iz++) {
    std::fprintf(t, "%1.5f", (iz - 0.5) * dz);
    for (long ir = 1; ir <= bins; ir++) std::fprintf(t, "\t %1.6e", F[ir * bins + iz]);
    std::fprintf(t, "\n");
  }
  std::fclose(t);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("USAGE: nmc name [--photons N] [--batch B] [--philox SEED] [--dispatch] [--device D] "
                "[--dry-run]\nwhich will load the files name_H.mci and name_T.bin\n"
                "and run the Monte Carlo program.\n");
    return 0;
  }
  const std::string name = argv[1];
  uint64_t photons = NMC_PHOTON_TOTAL_DEFAULT, batch = NMC_PHOTON_BATCH_DEFAULT, seed = 0;
  bool philox = false, persistent = true, dry = false;
  int device = 0;
  for (int i = 2; i < argc; ++i) {
    const std::string a = argv[i];
    auto val = [&](const char* what) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", what);
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "--photons") photons = std::strtoull(val("--photons"), nullptr, 10);
    else if (a == "--batch") batch = std::strtoull(val("--batch"), nullptr, 10);
    else if (a == "--philox") { philox = true; seed = std::strtoull(val("--philox"), nullptr, 10); }
    else if (a == "--persistent") persistent = true;
    else if (a == "--dispatch") persistent = false;
    else if (a == "--device") device = std::atoi(val("--device"));
    else if (a == "--dry-run") dry = true;
    else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      return 1;
    }
  }
  if (batch == 0 || photons == 0 || photons % batch) {
    std::fprintf(stderr, "--photons must be a positive multiple of --batch\n");
    return 1;
  }
  nmc_run_params rp;
  nmc_tissue_params tp;
  if (!read_mci(name, rp, tp)) return 1;
  const int kind = rp.mckernelflag;
  if (kind != NMC_SIM_MCSUB && kind != NMC_SIM_MCXYZ && kind != NMC_SIM_MCXYZ_TT) {
    std::printf("Unknown or unsupported kernel. quit.\n");
    return 1;
  }
  std::vector<uint8_t> v;
  {
    const size_t nv = (size_t)std::max(rp.Nx, 0) * std::max(rp.Ny, 0) * std::max(rp.Nz, 0);
    const std::string fn = name + "_T.bin";
    FILE* f = std::fopen(fn.c_str(), "rb");
    if (f) {
      v.resize(nv);
      const size_t got = std::fread(v.data(), 1, nv, f);
      std::fclose(f);
      if (got != nv) {
        std::fprintf(stderr, "%s holds %zu bytes, expected Nx*Ny*Nz = %zu\n", fn.c_str(), got, nv);
        return 1;
      }
    } else if (kind != NMC_SIM_MCSUB) {
      std::fprintf(stderr, "cannot open %s\n", fn.c_str());
      return 1;
    }
  }
  print_params(rp, tp);
  save_props(name, rp, tp);
  if (dry) return 0;

  nmc_handle* h = nullptr;
  if (nmc_create(kind, device, &h) != NMC_OK) return die(h, "nmc_create");
  nmc_ext ext;
  nmc_ext_defaults(&ext);
  ext.photons_per_dispatch = batch;
  ext.photons_total = photons;
  ext.rng = philox ? NMC_RNG_PHILOX : NMC_RNG_TAUS_REF;
  ext.seed = seed;
  if (nmc_set_ext(h, &ext) != NMC_OK) return die(h, "nmc_set_ext");
  if (nmc_prepare(h, &rp, &tp, v.empty() ? nullptr : v.data()) != NMC_OK) return die(h, "nmc_prepare");
  if (persistent) {
    const nmc_status st = nmc_run(h, 0, photons);
    if (st != NMC_OK && st != NMC_ESTEPCAP) return die(h, "nmc_run");
  } else {
    const int runs = (int)(photons / batch);
    for (int run = 1; run <= runs; ++run) {
      if (nmc_set_num_runs_seed(h, run, 0.f) != NMC_OK) return die(h, "nmc_set_num_runs_seed");
      const nmc_status st = nmc_send_compute_command(h);
      if (st != NMC_OK && st != NMC_ESTEPCAP) return die(h, "nmc_send_compute_command");
    }
  }
  nmc_summary sm;
  nmc_get_summary(h, &sm);
  std::printf("Total execution time (GPU):%f\nSimulation rate %d [photons/sec]\n", sm.kernel_ms * 1e-3,
              (int)(photons / std::max(sm.kernel_ms * 1e-3, 1e-9)));
  const double N = (double)photons;

  if (kind == NMC_SIM_MCSUB) {  // main.m:203-262
    const int B = ext.sub_bins;
    std::vector<float> J(B + 1, 0.f), Fz((size_t)(B + 1) * (B + 1), 0.f);
    float SAE[3] = {0.f, 0.f, 0.f};
    if (nmc_get_compute_results(h, J.data(), Fz.data(), nullptr, SAE, nullptr, nullptr, nullptr, nullptr, nullptr,
                                nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr) != NMC_OK)
      return die(h, "nmc_get_compute_results");
    const float mua = tp.muav[1];
    // the reference's dr_mcsub / dz_mcsub are double literals (definitions.h:52-53)
    const double dr = ext.sub_dr == NMC_MCSUB_DR_DEFAULT ? 0.0020 : (double)ext.sub_dr;
    const double dz = ext.sub_dz == NMC_MCSUB_DZ_DEFAULT ? 0.0020 : (double)ext.sub_dz;
    for (int ir = 1; ir <= B; ir++) {
      const float r = (float)((ir - 0.5) * dr);
      J[ir] /= 2.0 * kPi * r * dr * N;
      for (int iz = 1; iz <= B; iz++) Fz[(size_t)ir * B + iz] /= 2.0 * kPi * r * dr * dz * N * mua;
    }
    for (float& x : SAE) x /= (float)photons;  // float / int, as main.m:238-240
    const float R = SAE[0], A = SAE[1], E = SAE[2];
    const float total_rd = E + R;
    std::printf("Escaping fraction is: %lg\n", (double)E);
    std::printf("Absorbed fraction is: %lg\n", (double)A);
    std::printf("Reflectance is: %lg\n", (double)R);
    std::printf("Total is: %lg\n", (double)(E + A + R));
    std::printf("Rd is: %lg\n", (double)total_rd);
    const std::string fn = name + "_Rd.dat";
    std::printf("saving %s\n", fn.c_str());
    if (FILE* f = std::fopen(fn.c_str(), "w")) {
      std::fprintf(f, "%0.4f\n", total_rd);
      std::fclose(f);
    }
    save_mcout(J.data(), Fz.data(), R, A, E, tp.muav[1], tp.musv[1], tp.gv[1], rp.n1, rp.n2, B, dr, dz, N);
  } else {  // main.m:473-561
    const size_t nv = (size_t)rp.Nx * rp.Ny * rp.Nz, n2d = (size_t)rp.Nx * rp.Ny;
    std::vector<float> F3D(nv, 0.f), Rd(batch, 0.f), Rd2D(n2d, 0.f);
    std::vector<int32_t> Det(n2d, 0);
    if (nmc_get_compute_results(h, nullptr, nullptr, F3D.data(), nullptr, Rd.data(), Rd2D.data(), Det.data(),
                                nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                nullptr) != NMC_OK)
      return die(h, "nmc_get_compute_results");
    const float temp = (float)rp.dx * rp.dy * rp.dz * (float)N;
    for (size_t i = 0; i < nv; i++) {
      const float mua = tp.muav[v[i]];
      const float val = F3D[i] / (temp * mua);
      F3D[i] = (!std::isnan(val) && !std::isinf(val)) ? val : 0.0f;
    }
    std::string fn = name + "_F.bin";
    std::printf("saving %s\n", fn.c_str());
    if (FILE* f = std::fopen(fn.c_str(), "wb")) {
      std::fwrite(F3D.data(), sizeof(float), nv, f);
      std::fclose(f);
    }
    float total_rd = 0.f;
    for (float r : Rd)
      if (!std::isnan(r) && !std::isinf(r)) total_rd += r;
    total_rd /= (float)N;
    std::printf("Total Rd = %0.8f\n", total_rd);
    fn = name + "_Rd.dat";
    std::printf("saving %s\n", fn.c_str());
    if (FILE* f = std::fopen(fn.c_str(), "w")) {
      std::fprintf(f, "%0.4f\n", total_rd);
      std::fclose(f);
    }
    // rows of Ny values at j + i*Nx (the reference's indexing, equal to
    // i*Ny + j only when Nx == Ny; out-of-range indices read as 0 here)
    auto table = [&](const std::string& suffix, auto&& cell) {
      const std::string tn = name + suffix;
      std::printf("saving %s\n", tn.c_str());
      FILE* f = std::fopen(tn.c_str(), "wb");
      if (!f) return;
      for (int i = 0; i < rp.Nx; i++) {
        for (int j = 0; j < rp.Ny; j++) cell(f, (size_t)j + (size_t)i * rp.Nx);
        std::fprintf(f, "\n");
      }
      std::fclose(f);
    };
    table("_Ryx.dat", [&](FILE* f, size_t idx) {
      const float val = idx < n2d ? Rd2D[idx] : 0.f;
      std::fprintf(f, "\t %1.6e", (!std::isnan(val) && !std::isinf(val)) ? val : 0.0);
    });
    table("_DetPhot2D.dat", [&](FILE* f, size_t idx) { std::fprintf(f, "\t %d", idx < n2d ? Det[idx] : 0); });
  }
  {  // structured run report
    const double rd = kind == NMC_SIM_MCSUB ? (sm.S + sm.E) / N : sm.rd_sum / N;
    const double m = (kind == NMC_SIM_MCSUB ? sm.E : sm.rd_sum) / N;
    const double se = std::sqrt(std::max(0.0, sm.rd_sumsq / N - m * m) / N);
    const std::string fn = name + "_report.json";
    if (FILE* f = std::fopen(fn.c_str(), "w")) {
      std::fprintf(f,
                   "{\"name\": \"%s\", \"kind\": %d, \"photons\": %llu, \"rng\": \"%s\", "
                   "\"kernel_ms\": %.6f, \"photons_per_s\": %.6e, \"Rd\": %.9f, \"Rd_se\": %.9f, "
                   "\"substeps_per_photon\": %.6f, \"scatters_per_photon\": %.6f, \"device_flags\": %u}\n",
                   rp.myname, kind, (unsigned long long)photons, philox ? "philox4x32-10" : "reference", sm.kernel_ms,
                   photons / std::max(sm.kernel_ms * 1e-3, 1e-12), rd, se, (double)sm.substeps / N,
                   (double)sm.scatters / N, sm.device_flags);
      std::fclose(f);
    }
  }
  nmc_destroy(h);
  return 0;
}
