"""The BF16 MLP surrogate: forward outputs and loss gradients against the
NumPy FP64 restatement (relative error within BF16 epsilon x sqrt(fan-in)),
inference equal to the training forward, training that lowers the loss,
and the solver-trained surrogate end to end on a small mesh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2.0 ** -8 * np.sqrt(128)      # BF16 epsilon x sqrt(fan-in)
BLOCKS = (("W1", 0, 16 * 128), ("b1", 2048, 128), ("W2", 2176, 128 * 128),
          ("b2", 18560, 128), ("W3", 18688, 256), ("b3", 18944, 2))


@pytest.fixture(scope="module")
def small_family():
    from anuga_cuda.surrogate import FamilyMesh
    return FamilyMesh(cells=12)


def test_gradients_match_oracle(small_family, swgpu_built):
    from anuga_cuda.surrogate import Surrogate, sample_params
    from oracle import mlp_oracle as MO
    fm = small_family
    sg = Surrogate(fm, seed=3)
    th = sample_params(4, seed=7)
    rng = np.random.default_rng(5)
    targets = rng.uniform(0.0, 1.0, (4, fm.N, 2)).astype(np.float32)
    sg.set_data(th, targets)
    rows = rng.choice(4 * fm.N, 777, replace=False)
    y, loss, g = sg.gradients(rows, 1.0, 0.5)
    yo, losso, go = MO.forward_backward(sg.params(), th, fm.tri, rows, targets, sg.mu, sg.isd,
                                        1.0, 0.5)
    assert np.max(np.abs(y - yo)) <= TOL * np.max(np.abs(yo))
    assert abs(loss - losso) <= TOL * losso
    for name, o, n in BLOCKS:
        ref = go[o:o + n]
        assert np.max(np.abs(g[o:o + n] - ref)) <= TOL * np.max(np.abs(ref)), name


def test_predict_equals_training_forward(small_family, swgpu_built):
    from anuga_cuda.surrogate import DEPTH_SCALE, Surrogate, initial_depth, sample_params
    fm = small_family
    sg = Surrogate(fm, seed=4)
    sg.set_tensor_path("mma.sync")   # the training forward's own kernel code
    th = sample_params(3, seed=8)
    targets = np.zeros((3, fm.N, 2), np.float32)
    sg.set_data(th, targets)
    rows = np.arange(3 * fm.N)
    y, _, _ = sg.gradients(rows)
    depth, _, _ = sg.predict(th)
    exp = np.maximum(initial_depth(fm, th).ravel() + y[:, 0] * DEPTH_SCALE, 0)
    assert np.array_equal(depth.ravel(), exp)


def test_training_lowers_loss(small_family, swgpu_built):
    from anuga_cuda.surrogate import Surrogate, sample_params
    fm = small_family
    sg = Surrogate(fm, seed=0)
    th = sample_params(16, seed=9)
    # a smooth synthetic target of the features
    r = np.hypot(fm.tri[None, :, 0] - th[:, 1:2], fm.tri[None, :, 1] - th[:, 2:3])
    targets = np.stack([th[:, :1] / 3.0 * np.exp(-r / 2000.0),
                        np.clip(r / 5000.0, 0, 1)], axis=2).astype(np.float32)
    sg.set_data(th, targets)
    rows = np.arange(16 * fm.N)
    _, loss0, _ = sg.gradients(rows)
    stats = sg.fit(th, targets, steps=400, batch=4096, lr=3e-3)
    _, loss1, _ = sg.gradients(rows)
    assert loss1 < 0.2 * loss0, (loss0, loss1)
    assert stats["samples_per_s"] > 0


def test_solver_trained_surrogate(swgpu_built):
    from anuga_cuda.surrogate import (FamilyMesh, Surrogate, fallback_report, sample_params,
                                      solve, targets_from)
    fm = FamilyMesh(cells=16)
    T = 150.0
    th_train, th_test = sample_params(48, seed=5000), sample_params(8, seed=9000)
    hm, ta, ms_train = solve(fm, th_train, finaltime=T, batch=16)
    assert (ta >= 0).any() and (ta < 0).any() and hm.max() > 0.3
    hmt, tat, ms_test = solve(fm, th_test, finaltime=T, batch=8)
    sg = Surrogate(fm, seed=1)
    sg.fit(th_train, targets_from(fm, th_train, hm, ta, T), steps=1500, batch=8192, lr=3e-3)
    depth, arr, infer_ms = sg.predict(th_test)
    baseline = np.abs(hmt - hm.mean(axis=0)[None]).mean()
    rep = fallback_report(depth, hmt, ms_test / len(th_test), infer_ms)
    assert rep["mean_abs_error_m"] < baseline, (rep, baseline)
    assert 0.0 <= rep["blocks_over_tol_pct"] <= 100.0


def test_tcgen05_inference_matches(small_family, swgpu_built):
    """The tcgen05/TMEM inference kernel against the mma.sync one and the
    NumPy FP64 restatement (BF16 rounding points alike; accumulation order
    differs, so within the BF16 tolerance)."""
    from anuga_cuda.surrogate import DEPTH_SCALE, Surrogate, initial_depth, sample_params
    from oracle import mlp_oracle as MO
    fm = small_family
    sg = Surrogate(fm, seed=11)
    th = sample_params(5, seed=12)
    sg.set_tensor_path("mma.sync")
    d_sync, a_sync, _ = sg.predict(th)
    sg.set_tensor_path("tcgen05")
    d_tc, a_tc, _ = sg.predict(th)
    assert np.isfinite(d_tc).all()
    scale = np.max(np.abs(d_sync)) + 1e-6
    assert np.max(np.abs(d_tc - d_sync)) <= TOL * scale
    rows = np.arange(5 * fm.N)
    yo, _, _ = MO.forward_backward(sg.params(), th, fm.tri, rows,
                                   np.zeros((5, fm.N, 2), np.float32), sg.mu, sg.isd)
    ref = np.maximum(initial_depth(fm, th).ravel() + yo[:, 0] * DEPTH_SCALE, 0)
    assert np.max(np.abs(d_tc.ravel() - ref)) <= TOL * scale
