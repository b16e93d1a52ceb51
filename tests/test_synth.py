"""Synthetic inputs: shapes and value ranges of the benchmark configurations."""
import numpy as np

from aeroapps_gb300 import synth


def test_columns_shapes_and_ranges():
    c = synth.make_columns(16, [470.0, 550.0], seed=20261203)
    km, n = c["km"], 16
    assert km == 72 and c["pe"].shape == (73, n) and c["qm"].shape == (72, 20, n) and c["ROT"].shape == (72, n, 2)
    assert np.all(np.diff(c["pe"], axis=0) > 0) and np.allclose(c["pe"][0], synth.PTOP)
    assert np.all(np.diff(c["he"], axis=0) < 0) and np.all(c["he"][-1] == 0)
    assert np.all((c["rh"] >= 0) & (c["rh"] < 0.99))
    assert np.all((c["sza"] >= 0) & (c["sza"] <= 75)) and np.all((c["vza"] >= 0) & (c["vza"] <= 60))
    tau_r = c["ROT"][:, :, 1].sum(axis=0)
    assert np.allclose(tau_r, 0.0976 * (1 - 1.0 / c["pe"][-1]), rtol=1e-6)
    assert 0.02 < synth.coef_depol(0.55) < 0.04


def test_ragged_layers_merge_top():
    L = np.array([20, 72, 45])
    c = synth.make_columns(3, [550.0], seed=1, nlayers=L)
    for j, l in enumerate(L):
        assert np.all(np.diff(c["pe"][: l + 1, j]) > 0)
        assert c["he"][l, j] == 0.0 and np.all(c["he"][:l, j] > 0)
    assert c["pe"][20, 0] == c["pe"][72, 1] * 0 + c["pe"][20, 0]


def test_seeded_reproducible():
    a = synth.make_columns(4, [550.0], seed=7)
    b = synth.make_columns(4, [550.0], seed=7)
    assert all(np.array_equal(a[k], b[k]) for k in ("qm", "rh", "pe", "sza"))
