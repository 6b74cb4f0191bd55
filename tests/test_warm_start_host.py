"""Host side of the learned warm start (no GPU): normalisation, model files,
initial parameters and the committed model's shape."""
import os

import numpy as np


def test_normalisation_and_model_roundtrip(eb, tmp_path):
    from endobeams_gb300 import warm_start as W
    rng = np.random.default_rng(0)
    sc = np.logspace(-6, 3, W.NRAW)  # raw features span many magnitudes (m, m/s, m/s^2, ...)
    F = (rng.standard_normal((500, W.NRAW)) + 2.0) * sc
    T = rng.standard_normal((500, W.NOUT)) * 1e4
    shift, scale, oscale = W.normalisation(F, T)
    X, Tn = W.normalise(F, T, shift, scale, oscale)
    assert X.shape == (500, W.NIN) and np.all(X[:, W.NRAW:] == 0)
    assert np.allclose(X[:, :W.NRAW].mean(0), 0, atol=1e-5) and np.allclose(X[:, :W.NRAW].std(0), 1, atol=1e-4)
    assert np.allclose(Tn.std(0), 1, atol=1e-4)
    m = W.WarmStartModel(W.init_params(3), shift, scale, oscale, {"note": "test"})
    path = str(tmp_path / "m.npz")
    m.save(path)
    m2 = W.WarmStartModel.load(path)
    for a in ("params", "in_shift", "in_scale", "out_scale"):
        assert np.array_equal(getattr(m, a), getattr(m2, a))


def test_init_params_layout_matches_oracle(eb):
    import mlp_oracle as M
    from endobeams_gb300 import warm_start as W
    p = W.init_params(0, out_gain=0.5)
    assert p.shape == (M.NPARAMS,) and W.NPARAMS == M.NPARAMS
    # biases start at zero, weights do not
    assert np.all(p[M.OFF_B1:M.OFF_W2] == 0) and np.all(p[M.OFF_B2:M.OFF_W3] == 0) and np.all(p[M.OFF_B3:] == 0)
    assert np.std(p[M.OFF_W1:M.OFF_B1]) > 0.1 and np.std(p[M.OFF_W3:M.OFF_B3]) > 0


def test_committed_model_is_well_formed(eb):
    from endobeams_gb300 import warm_start as W
    path = os.path.join(os.path.dirname(eb.__file__), "models", "warm_start_stents.npz")
    m = W.WarmStartModel.load(path)
    assert m.params.shape == (W.NPARAMS,) and np.isfinite(m.params).all()
    assert np.all(m.in_scale != 0) and np.all(m.out_scale > 0)
