"""Pins the surrogate MLP's NumPy oracle (oracle/mlp_oracle.py) on the CPU.

The GPU tests of csrc/swgpu_mlp.cu compare against this oracle, so the oracle
itself is checked here against independent arithmetic: its BF16 rounding
against torch's float32 -> bfloat16 conversion (round to nearest, ties to
even), its backward pass against central finite differences of the loss (with
the BF16 rounding points made exact, so that the loss is smooth), and its
feature assembly against a hand-computed row.
"""
import numpy as np
import pytest
import torch

from oracle import mlp_oracle as MO


def _problem(seed, nscen=3, ntri=7, nrows=11):
    rng = np.random.default_rng(seed)
    scen = rng.uniform(-1.0, 1.0, (nscen, MO.NP)).astype(np.float32)
    tri = rng.uniform(-2.0, 2.0, (ntri, 4)).astype(np.float32)
    rows = rng.choice(nscen * ntri, nrows, replace=False)
    targets = rng.normal(size=(nscen * ntri, MO.NT))
    mu = rng.normal(size=MO.F).astype(np.float32) * 0.1
    isd = rng.uniform(0.5, 2.0, MO.F).astype(np.float32)
    params = rng.normal(size=MO.NUM_PARAMS) * 0.1
    return params, scen, tri, rows, targets, mu, isd


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(1)
    vals = np.concatenate([
        rng.normal(size=20000).astype(np.float32) * np.float32(1e3),
        rng.normal(size=2000).astype(np.float32) * np.float32(1e-30),
        # exact ties: the low 16 bits 0x8000 on odd and even BF16 mantissas
        np.array([0x3F808000, 0x3F818000, 0xBF808000, 0xBF818000, 0x00008000,
                  0x7F7F8000, 0x7F7FFFFF, 0x00000000, 0x80000000, 0x7F800000],
                 np.uint32).view(np.float32)])
    want = torch.from_numpy(vals.copy()).to(torch.bfloat16).to(torch.float64).numpy()
    got = MO.bf16(vals)
    assert np.array_equal(np.signbit(got), np.signbit(want))
    assert np.array_equal(got, want)


def test_backward_matches_finite_differences(monkeypatch):
    # exact arithmetic at every rounding point: the loss is then a smooth
    # function of the parameters and its central differences are accurate
    monkeypatch.setattr(MO, "bf16", lambda a: np.asarray(a, np.float64))
    params, scen, tri, rows, targets, mu, isd = _problem(7)
    # the biases are read as float32: keep them exactly representable
    P = MO.unflatten(params)
    for b in ("b1", "b2", "b3", "b4"):
        P[b][...] = P[b].astype(np.float32)
    params = MO.flatten(P)
    y0, loss, grad = MO.forward_backward(params, scen, tri, rows, targets, mu, isd, 1.0, 0.5,
                                         0.7)
    # the error term's target |y0 - t0| is a constant of the gradient: hold it
    t0 = np.asarray(targets).reshape(-1, MO.NT)[rows, 0]
    frozen = np.abs(y0[:, 0] - t0)
    rng = np.random.default_rng(3)
    # every block of the flat vector: weights and biases of each layer
    o, picks = 0, []
    for _, shape in MO.SHAPES:
        n = int(np.prod(shape))
        picks += list(o + rng.choice(n, min(n, 6), replace=False))
        o += n
    assert o == params.size
    for j in picks:
        # a power-of-two step: b +- h stays float32-exact for the (float32)
        # biases drawn here, so the forward pass's float32 read of them is exact
        h = 2.0 ** -14
        up, dn = params.copy(), params.copy()
        up[j] += h
        dn[j] -= h
        lu = MO.forward_backward(up, scen, tri, rows, targets, mu, isd, 1.0, 0.5, 0.7,
                                 frozen_error=frozen)[1]
        ld = MO.forward_backward(dn, scen, tri, rows, targets, mu, isd, 1.0, 0.5, 0.7,
                                 frozen_error=frozen)[1]
        fd = (lu - ld) / (2.0 * h)
        assert fd == pytest.approx(grad[j], rel=1e-5, abs=1e-9 * max(1.0, loss)), j


def test_features_hand_computed_row():
    scen = np.zeros((2, MO.NP), np.float32)
    scen[1] = [300.0, 900.0, 2000.0, 0.03, 0.1, 0.2, -0.3, 0.05, 0.0]
    tri = np.array([[0.0, 0.0, -1.0, 10.0], [6.0, 8.0, 2.5, 5.0]], np.float32)
    mu = np.zeros(MO.F, np.float32)
    isd = np.ones(MO.F, np.float32)
    mu[12], isd[12] = 1.0, 0.5
    f = MO.features(scen, tri, [1 * 2 + 1], mu, isd)     # scenario 1, triangle 1
    assert f.dtype == np.float32 and f.shape == (1, MO.F)
    assert np.array_equal(f[0, :MO.NP], scen[1])
    assert (f[0, 9], f[0, 10], f[0, 11]) == (2.5, 6.0, 8.0)
    assert f[0, 12] == np.float32((5.0 - 1.0) * 0.5)          # distance to the inflow is 5
    assert np.all(f[0, 13:] == 0.0)
