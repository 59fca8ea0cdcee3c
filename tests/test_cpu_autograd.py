"""The torch plumbing of nmc_gb300.autograd on the CPU, with an engine
stand-in whose tallies are linear in the voxel properties: rd_r = n (W mua +
V mus) and absorbed = n mua / 2 (un-normalised, as the engine's tallies are).
Its adjoint returns the exact gradients of L = G . rd_r + GF . absorbed, so
the torch gradients must equal the analytic ones: this checks the per-photon
scaling, the reshaping, needs_input_grad and the re-recording of a forward
when the handle ran another one in between."""
import numpy as np
import pytest
import torch

from nmc_gb300 import abi, autograd

SHAPE = (2, 3, 2)
NV = int(np.prod(SHAPE))
NB = 4


class LinearEngine:
    sim_type = abi.SIM_MCXYZ

    def __init__(self, seed=0):
        r = np.random.default_rng(seed)
        self.W, self.V = r.normal(size=(NB, NV)), r.normal(size=(NB, NV))
        self.forwards = 0
        self.props = None

    def set_voxel_props(self, mua, mus, g):
        self.props = (np.asarray(mua, np.float64), np.asarray(mus, np.float64), np.asarray(g, np.float64))

    def reset(self):
        self.rd = self.ab = None

    def adjoint_forward(self, first, n, cap, deposit_capacity=0):
        self.forwards += 1
        self.n = n
        mua, mus, _ = self.props
        self.rd = n * (self.W @ mua + self.V @ mus)
        self.ab = n * 0.5 * mua
        self.recorded = self.props

    def tally(self, which):
        return {abi.TALLY_RD_R: self.rd, abi.TALLY_F3D: self.ab}[which].copy()

    def adjoint_backward(self, G, GF):
        assert self.recorded is self.props  # gradients of the recorded forward
        G = np.zeros(NB) if G is None else np.asarray(G, np.float64)
        GF = np.zeros(NV) if GF is None else np.asarray(GF, np.float64)
        n = self.n
        return n * (self.W.T @ G + 0.5 * GF), n * (self.V.T @ G), np.zeros(NV)


def _props(seed=1):
    r = np.random.default_rng(seed)
    mk = lambda lo, hi: torch.tensor(r.uniform(lo, hi, SHAPE), dtype=torch.float64, requires_grad=True)
    return mk(0.1, 5.0), mk(50.0, 300.0), mk(0.8, 0.9)


def test_forward_is_per_photon_and_shaped():
    e = LinearEngine()
    mua, mus, g = _props()
    rd, ab = autograd.transport(mua, mus, g, e, n=1000)
    assert rd.shape == (NB,) and ab.shape == SHAPE and rd.dtype == torch.float64
    m, s = mua.detach().numpy().ravel(), mus.detach().numpy().ravel()
    np.testing.assert_allclose(rd.detach().numpy(), e.W @ m + e.V @ s, rtol=1e-5)
    np.testing.assert_allclose(ab.detach().numpy().ravel(), 0.5 * m, rtol=1e-6)


def test_gradients_equal_analytic():
    e = LinearEngine()
    mua, mus, g = _props()
    rd, ab = autograd.transport(mua, mus, g, e, n=1000)
    c = torch.linspace(-1.0, 2.0, NB, dtype=torch.float64)
    d = torch.linspace(0.5, 1.5, NV, dtype=torch.float64).reshape(SHAPE)
    ((c * rd).sum() + (d * ab).sum()).backward()
    np.testing.assert_allclose(mua.grad.numpy().ravel(), e.W.T @ c.numpy() + 0.5 * d.numpy().ravel(), rtol=1e-5)
    np.testing.assert_allclose(mus.grad.numpy().ravel(), e.V.T @ c.numpy(), rtol=1e-5)
    np.testing.assert_array_equal(g.grad.numpy(), np.zeros(SHAPE))


def test_backward_records_again_after_another_forward():
    e = LinearEngine()
    mua, mus, g = _props(1)
    rd1, _ = autograd.transport(mua, mus, g, e, n=500)
    other = _props(2)
    autograd.transport(*other, e, n=500)  # the handle now holds another forward
    assert e.forwards == 2
    rd1.sum().backward()
    assert e.forwards == 3  # the first forward was recorded again for its backward
    np.testing.assert_allclose(mua.grad.numpy().ravel(), e.W.T @ np.ones(NB), rtol=1e-5)


def test_zero_upstream_gives_zero_gradients():
    e = LinearEngine()
    mua, mus, g = _props()
    rd, ab = autograd.transport(mua, mus, g, e, n=100)
    (0.0 * rd.sum()).backward()
    for t in (mua, mus, g):
        np.testing.assert_array_equal(t.grad.numpy(), np.zeros(SHAPE))


def test_only_voxel_engines():
    e = LinearEngine()
    e.sim_type = abi.SIM_MCSUB
    with pytest.raises(ValueError):
        autograd.transport(*_props(), e, n=10)


def test_fluence_normalisation():
    ab = torch.tensor([[1.0, 2.0], [3.0, 0.0]])
    mua = torch.tensor([[2.0, 0.0], [1.0, 1.0]])
    f = autograd.fluence(ab, mua, voxel_volume=0.5)
    np.testing.assert_allclose(f.numpy(), [[1.0, 0.0], [6.0, 0.0]])
