"""Shared simulation set-ups for the tests and the benchmark.

Geometries follow the reference's sample notebooks (NMC-samples/example0.ipynb
cells 2-4: homogeneous cube; example2.ipynb cells 3-4: skin with a blood
vessel) and the workload list the benchmark quotes (mcsub semi-infinite
medium; 200^3 skin-vessel voxel grid).
"""
from __future__ import annotations

import math

import numpy as np

from nmc_gb300 import abi

# Tissue ids of the skin-vessel map (index 0 unused, mcio.h:128)
AIR, EPIDERMIS, DERMIS, BLOOD = 1, 2, 3, 4


def mcsub_case(g: float = 0.9, phase: int = abi.PHASE_HG, rng: int = abi.RNG_PHILOX, seed: int = 0,
               bins: int = 101, dr: float = 0.01, dz: float = 0.01, mua: float = 1.0, mus: float = 100.0,
               n1: float = 1.37, n2: float = 1.0, tt=None):
    """Semi-infinite medium, normal pencil beam: mua=1, mus=100 /cm, g=0.9,
    n 1.37/1.0, Rd(r) 100 bins + overflow of 0.01 cm, F(r,z) 100x100 of 0.01 cm."""
    rp = abi.run_params(myname="mcsub", n1=n1, n2=n2, mckernelflag=abi.SIM_MCSUB, Nt=1)
    kw = {}
    if tt is not None:
        gf, af, gb, ab, cc = tt
        kw = dict(gf=[gf], af=[af], gb=[gb], ab=[ab], cc=[cc])
    tp = abi.tissue_params(mua=[mua], mus=[mus], g=[g], **kw)
    ext = abi.ext_defaults(rng=rng, seed=seed, phase=phase, sub_bins=bins, sub_dr=dr, sub_dz=dz)
    return rp, tp, ext


def homogeneous_case(N: int = 200, d: float = 0.02, rng: int = abi.RNG_PHILOX, seed: int = 0):
    """example0.ipynb cells 2-4: homogeneous cube, uniform beam r=1.2,
    mua=1, mus=100, g=0.9, n 1.4/1.001, boundaryflag 2, zsurf=0."""
    rp = abi.run_params(myname="test", Nx=N, Ny=N, Nz=N, dx=d, dy=d, dz=d, mcflag=0, launchflag=0,
                        boundaryflag=2, xs=0.0, ys=0.0, zs=0.0, xfocus=0.0, yfocus=0.0, zfocus=1e12,
                        ux0=0.7, uy0=0.4, uz0=math.sqrt(1 - 0.49 - 0.16), radius=1.2, waist=1.2,
                        zsurf=0.0, det_radius=5.0, xd=0.0, n1=1.4, n2=1.001, na=90.0, det_state=0,
                        mckernelflag=abi.SIM_MCXYZ, Nt=1)
    tp = abi.tissue_params(mua=[1.0], mus=[100.0], g=[0.9])
    v = np.ones(N * N * N, np.uint8)
    ext = abi.ext_defaults(rng=rng, seed=seed)
    return rp, tp, v, ext


def skin_vessel_map(N: int = 200, d: float = 0.005, zsurf: float = 0.01, epi: float = 0.006,
                    vessel_z: float = 0.05, vessel_r: float = 0.01, Ny: int | None = None,
                    Nz: int | None = None) -> np.ndarray:
    """uint8 tissue map, index iz*Ny*Nx + ix*Ny + iy (kernels.metal:482).
    Air above zsurf, one epidermis layer of thickness `epi` below it (rounded
    to voxels as example2.ipynb cell 4 does), dermis below, and a blood
    vessel cylinder along x of radius vessel_r centred at depth vessel_z."""
    Nx = N
    Ny = Ny or N
    Nz = Nz or N
    T = np.full((Nz, Nx, Ny), DERMIS, np.uint8)  # [iz, ix, iy]
    n_air = int(round(zsurf / d))
    T[:n_air] = AIR
    e1 = int(round(zsurf / d)) + 1
    e2 = min(int(round((zsurf + epi) / d)), Nz)
    if e2 >= e1:
        T[e1 - 1:e2] = EPIDERMIS
    yc = (np.arange(Ny) + 0.5 - Ny / 2.0) * d
    zc = (np.arange(Nz) + 0.5) * d
    inside = (yc[None, :] ** 2 + (zc[:, None] - vessel_z) ** 2) <= vessel_r ** 2  # [iz, iy]
    for iz in range(Nz):
        T[iz][:, inside[iz]] = BLOOD
    return T.reshape(-1)


def skin_vessel_case(N: int = 200, d: float = 0.005, rng: int = abi.RNG_PHILOX, seed: int = 0,
                     n2: float = 1.0, tissue_n: float = 1.37):
    """Skin-vessel workload: 200^3 @ 0.005 cm, air 0.01 cm, epidermis 0.006 cm
    (mua 20, mus 300, g 0.9), dermis (mua 0.5, mus 200, g 0.9), vessel along x
    r 0.01 cm at depth 0.05 cm (mua 230, mus 200, g 0.9), n = 1.37; uniform
    collimated beam r = 0.03 cm launched just below zsurf (example2.ipynb
    cell 3: zs = zsurf + 1e-4), boundaryflag 2, detector accepting all exits."""
    zsurf = 0.01
    rp = abi.run_params(myname="skinvessel", Nx=N, Ny=N, Nz=N, dx=d, dy=d, dz=d, mcflag=0, launchflag=0,
                        boundaryflag=2, xs=0.0, ys=0.0, zs=zsurf + 0.0001, xfocus=0.0, yfocus=0.0,
                        zfocus=float("inf"), ux0=0.7, uy0=0.4, uz0=math.sqrt(1 - 0.49 - 0.16),
                        radius=0.03, waist=0.03, zsurf=zsurf, det_radius=15.0, xd=0.0,
                        n1=tissue_n, n2=n2, na=90.0, det_state=0, mckernelflag=abi.SIM_MCXYZ, Nt=4)
    tp = abi.tissue_params(mua=[0.0001, 20.0, 0.5, 230.0], mus=[1.0, 300.0, 200.0, 200.0],
                           g=[1.0, 0.9, 0.9, 0.9])
    v = skin_vessel_map(N, d, zsurf)
    ext = abi.ext_defaults(rng=rng, seed=seed)
    return rp, tp, v, ext


def match_fraction(a, b, rel=1e-3, abs_=1e-6, fields=("detected", "absorbed")):
    """Fraction of photons whose fate, SPIN count and weight fields agree."""
    ok = (a["fate"] == b["fate"]) & (a["n_scatt"] == b["n_scatt"])
    for f in fields:
        x = a[f].astype(np.float64)
        y = b[f].astype(np.float64)
        ok &= np.abs(x - y) <= abs_ + rel * np.maximum(np.abs(x), np.abs(y))
    return float(np.mean(ok)), ok


def spectral_sweep_sets(n_wavelengths: int = 351, seed: int = 2024, budget_lo: float = 1e5,
                        budget_hi: float = 1e7, n1: float = 1.37, n2: float = 1.0):
    """Batched spectral sweep on the mcsub geometry: wavelengths 400-750 nm;
    reduced scattering mus' = a (lambda / 500 nm)^-b with a in [10, 40] /cm and
    b in [0.8, 2.0] (seeded); mua a seeded sum of 3-6 Gaussians (amplitudes
    0.05-2 /cm, centres 400-750 nm, widths 10-60 nm) over 0.01 /cm; two-term
    phase function g_f = 0.9, backward branch g_b = 0.3 sampled and negated
    (mean cosine -0.3), alpha = 0.5 (HG shape per branch), forward weight 0.9;
    mus = mus' / (1 - g_eff) with g_eff = 0.9*0.9 + 0.1*(-0.3) = 0.78; budgets
    log-uniform in [1e5, 1e7] photons.  Returns (wavelengths, list of
    abi.SweepSet)."""
    rng = np.random.default_rng(seed)
    lam = np.linspace(400.0, 750.0, n_wavelengths)
    a = rng.uniform(10.0, 40.0)
    b = rng.uniform(0.8, 2.0)
    k = int(rng.integers(3, 7))
    amp = rng.uniform(0.05, 2.0, k)
    cen = rng.uniform(400.0, 750.0, k)
    wid = rng.uniform(10.0, 60.0, k)
    mua = 0.01 + (amp[None, :] * np.exp(-((lam[:, None] - cen[None, :]) ** 2) / (2 * wid[None, :] ** 2))).sum(1)
    gf, af, gb, ab, cc = 0.9, 0.5, 0.3, 0.5, 0.9
    g_eff = cc * gf + (1 - cc) * (-gb)
    mus = a * (lam / 500.0) ** (-b) / (1.0 - g_eff)
    budgets = np.exp(rng.uniform(np.log(budget_lo), np.log(budget_hi), n_wavelengths)).astype(np.int64)
    sets = []
    for i in range(n_wavelengths):
        sets.append(abi.SweepSet(mua=float(mua[i]), mus=float(mus[i]), g=g_eff, gf=gf, af=af, gb=gb, ab=ab,
                                 cc=cc, n1=n1, n2=n2, pad=0, photons=int(budgets[i])))
    return lam, sets


def smooth_noise(shape, seed: int, sigma: float) -> np.ndarray:
    """Seeded white noise smoothed by a periodic Gaussian of `sigma` voxels
    (FFT), rescaled to [0, 1]."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kk = sum(np.meshgrid(*[(2 * np.pi * f) ** 2 for f in k], indexing="ij"))
    s = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-0.5 * sigma ** 2 * kk)))
    return (s - s.min()) / (s.max() - s.min())


def adjoint_case(N: int = 64, d: float = 0.01, seed: int = 7, sigma: float = 4.0, bins: int = 128,
                 dr: float = 0.005):
    """Per-voxel medium for the adjoint: N^3 voxels of d cm; mua log-uniform
    over smoothed seeded noise in [0.1, 5] /cm, mus linear in [50, 300] /cm
    (an independent noise field), g = 0.85 everywhere; tissue n = 1.4 under
    air; normal pencil beam at the origin of the top face (launchflag 1);
    photons leaving the grid are killed (boundaryflag 1); Rd(r) in `bins`
    bins of `dr` cm plus overflow.  Returns (rp, tp, v, ext, mua, mus, g,
    bins, dr) with the property arrays shaped [iz, ix, iy]."""
    rp = abi.run_params(myname="adjoint", Nx=N, Ny=N, Nz=N, dx=d, dy=d, dz=d, mcflag=0, launchflag=1,
                        boundaryflag=1, xs=0.0, ys=0.0, zs=0.0, xfocus=0.0, yfocus=0.0, zfocus=float("inf"),
                        ux0=0.0, uy0=0.0, uz0=1.0, radius=0.0, waist=0.0, zsurf=0.0, det_radius=15.0, xd=0.0,
                        n1=1.4, n2=1.0, na=90.0, det_state=0, mckernelflag=abi.SIM_MCXYZ, Nt=1)
    tp = abi.tissue_params(mua=[1.0], mus=[100.0], g=[0.85])
    v = np.ones(N * N * N, np.uint8)
    ext = abi.ext_defaults(rng=abi.RNG_PHILOX, seed=seed)
    ua = smooth_noise((N, N, N), seed, sigma)
    us = smooth_noise((N, N, N), seed + 1, sigma)
    mua = (0.1 * 50.0 ** ua).astype(np.float32)
    mus = (50.0 + 250.0 * us).astype(np.float32)
    g = np.full((N, N, N), 0.85, np.float32)
    return rp, tp, v, ext, mua, mus, g, bins, dr


# Two-term phase function of the spectral sweeps: forward HG lobe g_f = 0.9,
# backward lobe g_b = 0.3 sampled and negated (mean cosine -0.3), HG shape
# (alpha = 0.5) per lobe, forward weight 0.9.
TT_SWEEP = dict(gf=0.9, af=0.5, gb=0.3, ab=0.5, cc=0.9)
# seeded absorption amplitude ranges (1/cm) per tissue of the skin-vessel map
SWEEP_MUA_RANGE = {EPIDERMIS: (1.0, 20.0), DERMIS: (0.05, 2.0), BLOOD: (10.0, 250.0)}


def skin_vessel_spectral_tables(n_wavelengths: int = 351, seed: int = 2024, budget_lo: float = 1e5,
                                budget_hi: float = 1e7):
    """Spectral sweep on the skin-vessel map: wavelengths 400-750 nm; per
    tissue (epidermis, dermis, blood) mus' = a (lambda / 500 nm)^-b with a in
    [10, 40] /cm and b in [0.8, 2.0], and mua a sum of 3-6 Gaussians (centres
    400-750 nm, widths 10-60 nm, amplitudes in SWEEP_MUA_RANGE) over 0.01 /cm,
    all seeded; two-term phase TT_SWEEP with mus = mus' / (1 - g_eff),
    g_eff = 0.9*0.9 - 0.1*0.3 = 0.78; air mua 1e-4, mus 1; budgets
    log-uniform in [budget_lo, budget_hi].  Returns (wavelengths, list of
    abi.TissueParams, budgets)."""
    rng = np.random.default_rng(seed)
    lam = np.linspace(400.0, 750.0, n_wavelengths)
    g_eff = TT_SWEEP["cc"] * TT_SWEEP["gf"] - (1 - TT_SWEEP["cc"]) * TT_SWEEP["gb"]
    mua = {}
    mus = {}
    for t in (EPIDERMIS, DERMIS, BLOOD):
        a = rng.uniform(10.0, 40.0)
        b = rng.uniform(0.8, 2.0)
        k = int(rng.integers(3, 7))
        lo, hi = SWEEP_MUA_RANGE[t]
        amp = rng.uniform(lo, hi, k)
        cen = rng.uniform(400.0, 750.0, k)
        wid = rng.uniform(10.0, 60.0, k)
        mua[t] = 0.01 + (amp[None, :] * np.exp(-((lam[:, None] - cen[None, :]) ** 2)
                                                / (2 * wid[None, :] ** 2))).sum(1)
        mus[t] = a * (lam / 500.0) ** (-b) / (1.0 - g_eff)
    budgets = np.exp(rng.uniform(np.log(budget_lo), np.log(budget_hi), n_wavelengths)).astype(np.int64)
    tables = []
    for i in range(n_wavelengths):
        tables.append(abi.tissue_params(
            mua=[1e-4, mua[EPIDERMIS][i], mua[DERMIS][i], mua[BLOOD][i]],
            mus=[1.0, mus[EPIDERMIS][i], mus[DERMIS][i], mus[BLOOD][i]],
            g=[1.0, g_eff, g_eff, g_eff],
            **{k: [v] * 4 for k, v in TT_SWEEP.items()}))
    return lam, tables, budgets


def cbs_case(n_settings: int = 8, photons: int = 12_500_000, cone_n: int = 256, cone_half_angle: float = 5e-3,
             sep_n: int = 1024, sep_half_width: float = 0.512, mu_raman: float = 1e-4, seed: int = 5):
    """Polarised E-field / CBS / Raman case: monodisperse spheres a = 0.5 um,
    n 1.59 in water (1.33), lambda 633 nm, number density for mus = 100 /cm,
    mua 0.01 /cm; semi-infinite slab under air; Mie S1, S2 on 1801 angles;
    Raman conversion at mu_raman to 700 nm (the same spheres' table at 700 nm,
    density unchanged, mua 0.01); backscattering cone on cone_n^2 angles
    within +-cone_half_angle; settings: linear polarisation at 0, 45, 90,
    135 degrees, each at normal incidence and at 10 degrees (n_settings of
    them, photons each).  Returns (config, S_633, S_700, settings)."""
    from nmc_gb300 import efield

    m633 = efield.sphere_suspension(0.5, 1.59, 1.33, 633.0, 100.0)
    x700 = 2 * math.pi * 1.33 * 0.5 / 0.700
    m700 = efield.mie(x700, complex(1.59 / 1.33, 0.0), 1801)
    mus700 = m633["number_density"] * m700["q_sca"] * math.pi * (0.5e-4) ** 2
    cfg = abi.EfieldConfig(mua=0.01, mus=100.0, wavelength_cm=633e-7, raman_mua=0.01, raman_mus=mus700,
                           raman_wavelength_cm=700e-7, mu_raman=mu_raman, n_medium=1.33, n_outside=1.0,
                           n_angles=1801, cone_n=cone_n, cone_half_angle=cone_half_angle, sep_n=sep_n,
                           sep_half_width=sep_half_width, map_n=64, map_dx=0.01, depth_bins=100, depth_dz=0.01,
                           seed=seed, flags=0, speckle_max=0)
    settings = []
    for k in range(n_settings):
        pol = (k % 4) * math.pi / 4
        th = 0.0 if k < 4 else math.radians(10.0)
        settings.append(abi.EfieldSetting(pol_angle=pol, theta_in=th, phi_in=0.0, pad=0, photons=photons))
    return cfg, m633["table"], m700["table"], settings


def hg_amplitude_table(g: float, n_angles: int = 1801) -> np.ndarray:
    """S1 = S2 = sqrt(p_HG(theta)), real: a scatterer whose unpolarised phase
    function is Henyey-Greenstein (the scalar limit of the E-field kernel)."""
    th = np.linspace(0.0, math.pi, n_angles)
    p = (1 - g * g) / (1 + g * g - 2 * g * np.cos(th)) ** 1.5
    a = np.sqrt(p).astype(np.float32)
    return np.stack([a, np.zeros_like(a), a, np.zeros_like(a)], axis=1)


def notebook_skinvessel_map(N: int = 200, d: float = 0.0005, zsurf: float = 0.01) -> np.ndarray:
    """The sample notebooks' skin-vessel label volume (example2/3 cell 4):
    dermis (4), air (1) above zsurf, epidermis (5) for 0.006 cm below it,
    blood (3) in a cylinder along y of radius 0.01 cm at x = 0, z = N/2 d;
    in the engine's voxel order (the notebooks write T(y, x, z) in Fortran
    order, which is the same order)."""
    x = (np.arange(1, N + 1) - N / 2.0) * d
    z = np.arange(1, N + 1) * d
    T = np.full((N, N, N), 4, np.uint8)  # [iy, ix, iz]
    a = int(round(zsurf / d))
    if a >= 1:
        T[:, :, :a] = 1
    e1 = max(int(round(zsurf / d)) + 1, 1)
    e2 = min(int(round((zsurf + 0.006) / d)), N)
    if e2 >= e1:
        T[:, :, e1 - 1:e2] = 5
    inside = (x[:, None] ** 2 + (z[None, :] - N / 2.0 * d) ** 2) <= 0.01 ** 2  # [ix, iz]
    T[:, inside] = 3
    return np.ascontiguousarray(T.transpose(2, 1, 0)).reshape(-1)


def write_notebook_mci(path: str, tissues, N: int = 200, d: float = 0.0005):
    """_H.mci exactly as example2/3 cell 5 writes it (skin vessel, "%.4f")."""
    import math as _m

    vals = [f"{10.0:.2f}", f"{N}", f"{N}", f"{N}", f"{d:.4f}", f"{d:.4f}", f"{d:.4f}", "0", "0", "2",
            f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0101:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{_m.inf:.4f}",
            f"{0.7:.4f}", f"{0.4:.4f}", f"{_m.sqrt(1 - 0.49 - 0.16):.4f}", f"{0.03:.4f}", f"{0.03:.4f}",
            f"{0.01:.4f}", f"{15.0:.4f}", f"{0.0:.4f}", f"{1.4:.4f}", f"{1.001:.4f}", f"{90.0:.4f}",
            f"{532e-6:.4f}", f"{0.001:.4f}", "0", "1", "0", "1", f"{len(tissues)}"]
    for mua, mus, g in tissues:
        vals += [f"{mua:.4f}", f"{mus:.4f}", f"{g:.4f}"]
    with open(path, "w") as f:
        f.write("\n".join(vals) + "\n")


def example1_mus(n_runs: int = 10) -> list[float]:
    """The scattering coefficients example1 cell 4 sweeps: n_runs log-spaced
    values from 0.1 to 1e7 (its get_log_scale)."""
    f = math.exp(math.log(1e7 / 0.1) / max(n_runs - 1, 1))
    return [0.1 * f ** i for i in range(n_runs)]


def write_example1_mci(path: str, mus: float, N: int = 200, d: float = 0.02):
    """_H.mci exactly as example1 cell 3 writes it for one run of its sweep
    (cell 2: homogeneous tissue 1, mua 10, g 0.9, point collimated source at
    the origin (mcflag 4), boundaryflag 0, zsurf 0, n1 1.001, n2 1.4)."""
    vals = [f"{1:.2f}", f"{N}", f"{N}", f"{N}", f"{d:.4f}", f"{d:.4f}", f"{d:.4f}", "4", "0", "0",
            f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{1e12:.4f}",
            f"{0.7:.4f}", f"{0.4:.4f}", f"{math.sqrt(1 - 0.49 - 0.16):.4f}", f"{1.0:.4f}", f"{1.0:.4f}",
            f"{0.0:.4f}", f"{5.0:.4f}", f"{0.0:.4f}", f"{1.001:.4f}", f"{1.4:.4f}", f"{90.0:.4f}",
            f"{640e-6:.4f}", f"{0.001:.4f}", "0", "1", "0", "1", "1", f"{10.0:.4f}", f"{mus:.4f}", f"{0.9:.4f}"]
    with open(path, "w") as f:
        f.write("\n".join(vals) + "\n")


def example0_params():
    """RunParams and TissueParams as `nmc` reads them from example0's _H.mci
    (cell 2: homogeneous 200^3 at 0.02, uniform beam of radius 1.2 at the
    origin, boundaryflag 2, zsurf 0, mua 1, mus 100, g 0.9, n1 1.4, n2 1.001)."""
    rp = abi.run_params(myname="test", Nx=200, Ny=200, Nz=200, dx=0.02, dy=0.02, dz=0.02, mcflag=0, launchflag=0,
                        boundaryflag=2, xs=0.0, ys=0.0, zs=0.0, xfocus=0.0, yfocus=0.0, zfocus=1e12, ux0=0.7,
                        uy0=0.4, uz0=0.5916, radius=1.2, waist=1.2, zsurf=0.0, det_radius=5.0, xd=0.0, n1=1.4,
                        n2=1.001, na=90.0, lambda_=0.0006, lc=0.001, semiflag=1, det_state=0,
                        mckernelflag=abi.SIM_MCXYZ, Nt=1)
    return rp, abi.tissue_params(mua=[1.0], mus=[100.0], g=[0.9])


def write_example0_mci(path: str):
    """_H.mci exactly as example0 cell 3 writes it."""
    vals = [f"{1.0:.2f}", "200", "200", "200", f"{0.02:.4f}", f"{0.02:.4f}", f"{0.02:.4f}", "0", "0", "2",
            f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{0.0:.4f}", f"{1e12:.4f}",
            f"{0.7:.4f}", f"{0.4:.4f}", f"{math.sqrt(1 - 0.49 - 0.16):.4f}", f"{1.2:.4f}", f"{1.2:.4f}",
            f"{0.0:.4f}", f"{5.0:.4f}", f"{0.0:.4f}", f"{1.4:.4f}", f"{1.001:.4f}", f"{90.0:.4f}",
            f"{640e-6:.4f}", f"{0.001:.4f}", "0", "1", "0", "1", "1", f"{1.0:.4f}", f"{100.0:.4f}", f"{0.9:.4f}"]
    with open(path, "w") as f:
        f.write("\n".join(vals) + "\n")


# Three-layer skin stack for the layered model: (mua, mus, g, n, thickness),
# cm^-1 and cm: epidermis 0.01, dermis 0.2, semi-infinite subcutis.
LAYERED_SKIN3 = [(3.0, 200.0, 0.8, 1.4, 0.01), (0.3, 150.0, 0.85, 1.4, 0.2), (0.1, 100.0, 0.9, 1.44, math.inf)]


# Media and modes of the per-photon parity tests over the launch, boundary and
# detection branches (kernels.metal:366-463, :556-637, :646-672).
def modes_medium(Nx=40, Ny=40, Nz=40, dx=0.01, dy=0.01, dz=0.01, **run):
    """Air above zsurf = 2 dz, tissue (mua 1, mus 80, g 0.85) below, a
    spherical inclusion (mua 5, mus 120, g 0.9) of radius 0.06 cm at depth 0.1."""
    zsurf = 2 * dz
    base = dict(myname="modes", Nx=Nx, Ny=Ny, Nz=Nz, dx=dx, dy=dy, dz=dz, mcflag=0, launchflag=0,
                boundaryflag=2, xs=0.0, ys=0.0, zs=zsurf + 1e-4, xfocus=0.0, yfocus=0.0, zfocus=float("inf"),
                ux0=0.0, uy0=0.0, uz0=1.0, radius=0.03, waist=0.03, zsurf=zsurf, det_radius=15.0, xd=0.0,
                n1=1.37, n2=1.0, na=90.0, det_state=0, mckernelflag=abi.SIM_MCXYZ, Nt=3)
    base.update(run)
    rp = abi.run_params(**base)
    tp = abi.tissue_params(mua=[0.0001, 1.0, 5.0], mus=[1.0, 80.0, 120.0], g=[1.0, 0.85, 0.9])
    T = np.full((Nz, Nx, Ny), 2, np.uint8)
    T[:2] = 1
    x = (np.arange(Nx) + 0.5 - Nx / 2) * dx
    y = (np.arange(Ny) + 0.5 - Ny / 2) * dy
    z = (np.arange(Nz) + 0.5) * dz
    inc = (x[None, :, None] ** 2 + y[None, None, :] ** 2 + (z[:, None, None] - 0.1) ** 2) <= 0.06 ** 2
    T[inc] = 3
    return rp, tp, T.reshape(-1)


PARITY_MODES = {
    "gaussian-beam": dict(mcflag=1, radius=0.02, waist=0.02, zfocus=0.1),
    "isotropic-point": dict(mcflag=2, xs=0.0, ys=0.0, zs=0.1),
    "rectangle": dict(mcflag=3, radius=0.05),
    "point-collimated": dict(mcflag=4),
    "manual-direction": dict(launchflag=1, xs=0.01, ys=-0.02, zs=0.0201, ux0=0.3, uy0=0.2,
                             uz0=math.sqrt(1 - 0.13)),
    "boundary-0": dict(boundaryflag=0),
    "boundary-1": dict(boundaryflag=1),
    "transmittance": dict(det_state=1, Nz=16, zsurf=0.16, boundaryflag=1),
    "ring-detector": dict(xd=0.05, det_radius=0.02, na=30.0),
    "odd-noncubic-grid": dict(Nx=41, Ny=37, Nz=29, dx=0.011, dy=0.009, dz=0.0125),
}
