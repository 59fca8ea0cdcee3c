"""Per-voxel media and the perturbation Monte Carlo adjoint of Rd(r).

The adjoint's gradients are checked against central finite differences with
common random numbers (the same photon streams at mu -/+ delta) on 32 voxels
around the beam entry of a 64^3 heterogeneous medium, batch by batch, so that
each comparison carries its own standard error.  mua is pathwise (the
trajectories do not depend on it) and must agree to 1e-3 relative; mus and g
are likelihood-ratio estimates and must agree within 4.5 standard errors of
the batch means, voxel by voxel and summed.  Two losses: one on Rd(r) alone
(the detected photons are replayed once) and one on Rd(r) plus the absorbed
weight of a block of voxels (every photon is replayed, after its total score
is summed from the forward's deposit list or, without one, from a first
replay).
"""
import time

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu

VOXELS = [(iz, ix, iy) for iz in range(4) for ix in (30, 31, 32, 33) for iy in (31, 32)]


def _engine(gpu, case):
    rp, tp, v, ext, mua, mus, g, bins, dr = case
    e = gpu.Engine(abi.SIM_MCXYZ, 0, ext)
    e.prepare_data(rp, tp, v)
    e.set_radial_tally(bins, dr)
    e.set_voxel_props(mua, mus, g)
    return e


@pytest.fixture(scope="module")
def case():
    return cases.adjoint_case()


def _upstream(bins):
    G = np.random.default_rng(3).uniform(0.5, 1.5, bins + 1).astype(np.float32)
    G[-1] = 0.0  # overflow bin carries no loss
    return G


def _crn_check(gpu, case, voxels, G, GF, B, nb):
    """pMC gradients of G . Rd(r) + GF . absorbed against CRN central
    differences, per batch of nb photons (B batches)."""
    rp, tp, v, ext, mua, mus, g, bins, dr = case
    N = rp.Nx
    flat = np.array([iz * N * N + ix * N + iy for iz, ix, iy in voxels])
    G64 = G.astype(np.float64)
    GF64 = None if GF is None else GF.astype(np.float64)

    def loss(e):
        out = float(G64 @ e.tally(abi.TALLY_RD_R))
        if GF64 is not None:
            out += float(GF64 @ e.tally(abi.TALLY_F3D))
        return out

    with _engine(gpu, case) as e:
        pm = {k: np.zeros((B, len(flat))) for k in "asg"}
        for b in range(B):
            e.reset()
            e.adjoint_forward(b * nb, nb)
            ga, gs, gg = e.adjoint_backward(G, GF)
            pm["a"][b], pm["s"][b], pm["g"][b] = ga[flat], gs[flat], gg[flat]
        fd = {k: np.zeros((B, len(flat))) for k in "asg"}
        for k, arr, step in (("a", mua, lambda x: 0.02 * x), ("s", mus, lambda x: 0.02 * x),
                             ("g", g, lambda x: 0.01)):
            for j, fi in enumerate(flat):
                base = float(arr.ravel()[fi])
                h = step(base)
                sides = []
                for sgn in (1.0, -1.0):
                    a2 = arr.copy().ravel()
                    a2[fi] = base + sgn * h
                    props = {"a": (a2, mus, g), "s": (mua, a2, g), "g": (mua, mus, a2)}[k]
                    e.set_voxel_props(*[p.ravel() for p in props])
                    sc = []
                    for b in range(B):
                        e.reset()
                        e.run(b * nb, nb)
                        sc.append(loss(e))
                    sides.append(np.array(sc))
                fd[k][:, j] = (sides[0] - sides[1]) / (2.0 * h)
    for k in "asg":
        d = pm[k] - fd[k]
        se = d.std(0, ddof=1) / np.sqrt(B)
        P, F = pm[k].mean(0), fd[k].mean(0)
        t = d.mean(0) / se
        tot = d.sum(1)
        t_tot = tot.mean() / (tot.std(ddof=1) / np.sqrt(B))
        print(f"{k}: corr {np.corrcoef(P, F)[0, 1]:.4f} max|t| {np.abs(t).max():.2f} total t {t_tot:.2f}")
        if k == "a":
            # pathwise: same trajectories, differences are the fast exp's
            # slope and roulette flips
            assert np.all(np.abs(P - F) <= np.maximum(4.5 * se, 1e-3 * np.abs(F))), (P, F)
        else:
            assert np.all(np.abs(t) <= 4.5), (k, t)
            assert abs(t_tot) <= 4.5
            assert np.corrcoef(P, F)[0, 1] >= 0.97


def test_adjoint_rd_matches_crn_finite_differences(gpu, case):
    _crn_check(gpu, case, VOXELS, _upstream(case[7]), None, B=16, nb=500_000)


def test_adjoint_rd_and_fluence_match_crn_finite_differences(gpu, case):
    # loss on Rd(r) and on the absorbed weight of a block under the beam
    N = case[0].Nx
    GF = np.zeros((N, N, N), np.float32)
    GF[2:8, 28:36, 28:36] = 1.0
    voxels = [(iz, ix, iy) for iz in range(0, 8, 2) for ix in (30, 31, 32, 33) for iy in (31, 32)]
    _crn_check(gpu, case, voxels, _upstream(case[7]), GF.ravel(), B=16, nb=250_000)


def test_deposit_list_gives_the_score_replay_gradients(gpu, case):
    # With the record pass's deposit list a fluence-loss backward sums each
    # photon's total score from the list instead of replaying it; the
    # gradients are those of the score replay up to float summation order.
    # A list whose capacity runs out is dropped and the backward replays.
    rng = np.random.default_rng(5)
    G = _upstream(case[7])
    GF = rng.uniform(0.5, 1.5, case[0].Nx * case[0].Ny * case[0].Nz).astype(np.float32)
    n = 100_000
    with _engine(gpu, case) as e:
        e.adjoint_forward(0, n)
        assert not e.deposit_list_complete
        ref = e.adjoint_backward(G, GF)
        e.adjoint_forward(0, n, deposit_capacity=800 * n)
        assert e.deposit_list_complete
        lst = e.adjoint_backward(G, GF)
        e.adjoint_forward(0, n, deposit_capacity=1000)  # far too small: dropped
        assert not e.deposit_list_complete
        small = e.adjoint_backward(G, GF)
    for a, b, c in zip(ref, lst, small):
        scale = np.abs(a).max()
        np.testing.assert_allclose(b, a, rtol=0, atol=1e-5 * scale)
        np.testing.assert_allclose(c, a, rtol=0, atol=1e-5 * scale)


def test_adjoint_is_linear_in_the_upstream_gradient(gpu, case):
    bins = case[7]
    G1 = _upstream(bins)
    G2 = np.zeros(bins + 1, np.float32)
    G2[5:40] = 1.0
    with _engine(gpu, case) as e:
        e.adjoint_forward(0, 200_000)
        r1 = e.adjoint_backward(G1)
        r2 = e.adjoint_backward(G2)
        r12 = e.adjoint_backward(G1 + G2)
    for a, b, c in zip(r1, r2, r12):
        scale = np.abs(a).max() + np.abs(b).max()
        np.testing.assert_allclose(a + b, c, rtol=0, atol=1e-4 * scale)


def test_radial_tally_and_events(gpu, case):
    with _engine(gpu, case) as e:
        n = 200_000
        e.adjoint_forward(0, n)
        rd = e.tally(abi.TALLY_RD_R)
        sm = e.summary()
        assert rd.size == case[7] + 1
        # the radial bins hold every detected weight
        assert rd.sum() == pytest.approx(sm["rd_sum"], rel=1e-5)
        # the record pass tallies like a plain run of the same photons (the
        # two kernels are compiled apart: a rare photon may round differently)
        e.reset()
        e.run(0, n)
        plain = e.tally(abi.TALLY_RD_R)
        print("record vs plain: max bin difference", np.abs(plain - rd).max() / rd.max())
        np.testing.assert_allclose(plain, rd, rtol=0, atol=1e-3 * rd.max())
        # too small an event list is an error, and the handle stays usable
        e.reset()
        with pytest.raises(gpu.NMCError):
            e.adjoint_forward(0, n, event_capacity=100)
        with pytest.raises(gpu.NMCError):
            e.adjoint_backward(_upstream(case[7]))
        e.adjoint_forward(0, 1000)
        e.adjoint_backward(_upstream(case[7]))


def test_voxel_media_match_the_tissue_map(gpu):
    # the same medium given as a tissue map and as per-voxel properties; a
    # beam of finite radius (no photon starts exactly on a voxel face, where
    # the two modes' same-voxel rules differ)
    rp, tp, v, ext = cases.skin_vessel_case(N=64, d=0.005)
    gv = [0.9, 0.9, 0.9, 0.9]
    mua_t, mus_t = [0.0001, 20.0, 0.5, 230.0], [1.0, 300.0, 200.0, 200.0]
    tp = abi.tissue_params(mua=mua_t, mus=mus_t, g=gv)
    vi = v.astype(np.int64) - 1
    mua = np.asarray(mua_t, np.float32)[vi]
    mus = np.asarray(mus_t, np.float32)[vi]
    g = np.asarray(gv, np.float32)[vi]
    n = 20_000
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        recs_t, _ = e.run_traced(0, n)
        e.set_voxel_props(mua, mus, g)
        recs_v, _ = e.run_traced(0, n)
    frac, _ = cases.match_fraction(recs_t, recs_v)
    print("per-photon agreement", frac)
    assert frac >= 0.97


def test_autograd_function(gpu, case):
    torch = pytest.importorskip("torch")
    from nmc_gb300.autograd import fluence, radial_reflectance, transport

    rp, tp, v, ext, mua, mus, g, bins, dr = case
    N = rp.Nx
    n = 200_000
    w = torch.linspace(1.0, 0.0, bins + 1, dtype=torch.float64)
    wf = torch.zeros((N, N, N), dtype=torch.float64)
    wf[1:6, 30:34, 30:34] = 1.0
    with _engine(gpu, case) as e:
        ta = torch.tensor(mua, dtype=torch.float64, requires_grad=True)
        ts = torch.tensor(mus, dtype=torch.float64, requires_grad=True)
        tg = torch.tensor(g, dtype=torch.float64, requires_grad=True)
        rd, ab = transport(ta, ts, tg, e, 0, n)
        assert rd.shape == (bins + 1,) and ab.shape == (N, N, N)
        # another forward on the same handle before backward: the first is
        # recorded again
        radial_reflectance(ta * 1.1, ts, tg, e, 0, n)
        ((rd * w).sum() + (ab * wf).sum()).backward()
        e.set_voxel_props(mua, mus, g)
        e.reset()
        e.adjoint_forward(0, n, deposit_capacity=600 * n)  # as transport() records by default
        rd_direct = e.tally(abi.TALLY_RD_R) / n
        ab_direct = e.tally(abi.TALLY_F3D) / n
        ga, gs, gg = e.adjoint_backward((w.numpy() / n).astype(np.float32),
                                        (wf.numpy().ravel() / n).astype(np.float32))
    np.testing.assert_allclose(rd.detach().numpy(), rd_direct, rtol=1e-6)
    np.testing.assert_allclose(ab.detach().numpy().ravel(), ab_direct, rtol=1e-6)
    for t, ref in ((ta, ga), (ts, gs), (tg, gg)):
        # the per-photon scores are float sums whose order varies between
        # runs (atomics), hence the absolute floor
        np.testing.assert_allclose(t.grad.numpy().ravel(), ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    # the fluence normalisation differentiates through torch
    ta2 = torch.tensor(mua, dtype=torch.float64, requires_grad=True)
    phi = fluence(ab.detach(), ta2, 0.01 ** 3)
    phi.sum().backward()
    assert torch.all(ta2.grad <= 0)


def test_adjoint_costs_at_most_three_forwards(gpu, case):
    # forward + adjoint against a plain forward of the same photons, best of
    # three host-timed calls each: for a loss on Rd(r), and for Rd(r) plus the
    # absorbed weight (the forward keeps its deposit list, so every photon is
    # replayed once)
    G = _upstream(case[7])
    GF = np.ones(case[0].Nx ** 3, np.float32)
    n = 2_000_000

    def best(fn):
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    with _engine(gpu, case) as e:
        fwd = lambda: e.run(0, n)  # noqa: E731
        adj = lambda: (e.adjoint_forward(0, n), e.adjoint_backward(G))  # noqa: E731
        adj_f = lambda: (e.adjoint_forward(0, n, deposit_capacity=600 * n), e.adjoint_backward(G, GF))  # noqa: E731
        fwd(), adj(), adj_f()  # warm-up (and the lists' first allocation)
        t_fwd, t_adj, t_adj_f = best(fwd), best(adj), best(adj_f)
        assert e.deposit_list_complete
    print(f"forward {t_fwd * 1e3:.1f} ms; record + backward: Rd {t_adj * 1e3:.1f} ms ({t_adj / t_fwd:.2f}x), "
          f"Rd + absorbed {t_adj_f * 1e3:.1f} ms ({t_adj_f / t_fwd:.2f}x)")
    assert t_adj <= 3.0 * t_fwd
    assert t_adj_f <= 3.0 * t_fwd


def test_adjoint_satisfies_the_scaling_identity(gpu):
    # A homogeneous semi-infinite medium under a pencil beam has no length
    # scale of its own, so total Rd is unchanged when every mua and mus is
    # scaled by the same factor: sum_v (mua_v dRd/dmua_v + mus_v dRd/dmus_v) = 0.
    # The pathwise mua gradient and the likelihood-ratio mus gradient come from
    # different estimators and must cancel in that sum, within its statistics.
    N, d = 48, 0.01
    rp, tp, v, ext, _, _, _, bins, dr = cases.adjoint_case(N=N, d=d)
    rp.boundaryflag = 2  # photons beyond the sides and the bottom continue in the edge voxels' medium
    mua = np.full((N, N, N), 1.0, np.float32)
    mus = np.full((N, N, N), 100.0, np.float32)
    g = np.full((N, N, N), 0.85, np.float32)
    G = np.ones(bins + 1, np.float32)  # the loss is the total detected weight
    B, per = 8, 200_000
    a, s = [], []
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.set_radial_tally(bins, dr)
        e.set_voxel_props(mua, mus, g)
        for b in range(B):
            e.reset()
            e.adjoint_forward(b * per, per)
            ga, gs, _ = e.adjoint_backward(G)
            a.append(float((mua.ravel() * ga.ravel()).sum()) / per)
            s.append(float((mus.ravel() * gs.ravel()).sum()) / per)
    a, s = np.array(a), np.array(s)
    tot = a + s
    se = tot.std(ddof=1) / np.sqrt(B)
    print(f"mua . dRd/dmua {a.mean():.5f}, mus . dRd/dmus {s.mean():.5f}, sum {tot.mean():.2e} +- {se:.1e}")
    assert abs(tot.mean()) <= 3.5 * se + 1e-5
    assert abs(a.mean()) >= 20 * se  # each side on its own is far from zero
