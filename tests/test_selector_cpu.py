"""Host-side pieces of the learned parameter selector (no GPU).

* the network oracle's gradient against central finite differences (pins the
  oracle the CUDA kernels are checked against);
* the features on layouts with known answers;
* the mapping between parameter sets and network targets;
* the committed model file's layout.
"""
import os

import numpy as np
import pytest

from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mlp_ref.init(1) + 0.05 * rng.standard_normal(mlp_ref.NPARAMS)
    X = rng.standard_normal((17, 8))
    T = rng.standard_normal((17, 4))
    w = rng.random(17) + 0.5
    loss, g = mlp_ref.loss_grad(p, X, T, w)
    idx = rng.choice(mlp_ref.NPARAMS, 60, replace=False)
    # every block of the packed vector is probed
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in mlp_ref.SHAPES])
    idx = np.concatenate([idx, offs[:-1], offs[1:] - 1])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (mlp_ref.loss_grad(p + e, X, T, w)[0] - mlp_ref.loss_grad(p - e, X, T, w)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_oracle_adam_first_step_is_sign_descent():
    p = np.zeros(5)
    g = np.array([1.0, -2.0, 0.5, 0.0, 3.0])
    q, m, v = mlp_ref.adam(p, g, np.zeros(5), np.zeros(5), 1, lr=0.1, eps=0.0 + 1e-30)
    assert np.allclose(q[g != 0], -0.1 * np.sign(g[g != 0]))


def _nn_periodic(x, y, Lx, Ly):
    """Nearest-neighbour distance of every point (minimum image), brute force."""
    dx = x[:, None] - x[None, :]
    dy = y[:, None] - y[None, :]
    dx -= Lx * np.round(dx / Lx)
    dy -= Ly * np.round(dy / Ly)
    d = np.hypot(dx, dy)
    np.fill_diagonal(d, np.inf)
    return d.min(1)


def test_features_on_known_layouts():
    ft = pytest.importorskip("fasttools2d_gb300")
    from fasttools2d_gb300 import selector

    # a square lattice: every nearest neighbour at the mean spacing
    k = 40
    g = (np.arange(k) + 0.5) / k - 0.5
    X, Y = np.meshgrid(g, g)
    d = _nn_periodic(X.ravel(), Y.ravel(), 1.0, 1.0)
    f = selector.features_from_nn(d, k * k, 1234, 1.0, 1.0, 1e-8)
    assert f.shape == (8,)
    assert f[0] == pytest.approx(np.log10(k * k)) and f[1] == pytest.approx(np.log10(1234))
    assert f[2] == pytest.approx(1.0) and f[3] == 0.0
    assert np.allclose(f[4:7], 0.0, atol=1e-9) and f[7] == pytest.approx(-8.0)
    # all points in one tight cluster: small neighbour distances
    rng = np.random.default_rng(1)
    x, y = 0.001 * rng.standard_normal(2000), 0.001 * rng.standard_normal(2000)
    f2 = selector.features_from_nn(_nn_periodic(x, y, 2.0, 1.0), 2000, 2000, 2.0, 1.0, 1e-6)
    assert f2[2] == pytest.approx(2.0) and f2[3] > 0.9 and f2[5] < -1.0
    del ft


def test_targets_and_params_round_trip():
    """Network outputs map to the candidate set of the labels: zero
    corrections give the tuned cells and support back; others snap to the
    nearest candidate cell scale and support change (xi and the grid follow
    from the chooser)."""
    ft = pytest.importorskip("fasttools2d_gb300")
    from fasttools2d_gb300 import selector

    rng = np.random.default_rng(2)
    n = 20000
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    for Lx, Ly in ((1.0, 1.0), (2.75, 1.0), (1.0, 3.25)):
        T = ft.choose_params(0, f1, f2, n, Lx, Ly, tol=1e-8, form=ft.FORM_MIXED)
        assert selector._rational(T)
        opts = selector.params_from(np.zeros(4), T)
        assert opts == dict(P=T.P, nside_x=T.nside_x, nside_y=T.nside_y)
        o = selector.params_from(np.array([0.3, -0.1, 0.15, 0.8]), T)  # scale 1.4, P + 2
        a = max(1, round(T.nside_x / T.A * 1.4))
        assert o == dict(P=min(T.P + 2, 24), nside_x=T.A * a, nside_y=T.B * a)
        o = selector.params_from(np.array([-0.9, 0.0, 0.0, -3.0]), T)  # scale 0.7, P - 4
        assert o["P"] == max(T.P - 4, 4) and o["nside_x"] == T.A * max(1, round(T.nside_x / T.A * 0.7))


def test_params_round_trip_on_irrational_box():
    """Boxes with a step per axis: zero corrections give the tuned choice
    back, and a cell scale applies to each axis's count on its own."""
    ft = pytest.importorskip("fasttools2d_gb300")
    from fasttools2d_gb300 import selector

    rng = np.random.default_rng(4)
    n = 20000
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    T = ft.choose_params(1, f1, f2, n, 1.0, np.sqrt(2.0), tol=1e-8, form=ft.FORM_MIXED)
    assert not selector._rational(T)
    assert selector.params_from(np.zeros(4), T) == dict(P=T.P, nside_x=T.nside_x, nside_y=T.nside_y)
    o = selector.params_from(np.array([0.3, 0.0, 0.2, -1.0]), T)
    assert o == dict(P=T.P - 2, nside_x=round(T.nside_x * 1.4), nside_y=round(T.nside_y * 1.4))


def test_committed_model_layout():
    ft = pytest.importorskip("fasttools2d_gb300")
    from fasttools2d_gb300 import selector

    if not os.path.exists(selector.MODEL_PATH):
        pytest.skip("no trained selector model in this checkout")
    z = np.load(selector.MODEL_PATH)
    for name in ("slp", "dlp"):
        assert z[f"{name}_params"].shape == (mlp_ref.NPARAMS,)
        assert z[f"{name}_params"].dtype == np.float32
        assert z[f"{name}_xmean"].shape == (8,) and z[f"{name}_xstd"].shape == (8,)
        assert z[f"{name}_yscale"].shape == (4,)
        assert np.all(np.isfinite(z[f"{name}_params"]))
    del ft


def test_records_round_trip_and_labels(tmp_path):
    ft = pytest.importorskip("fasttools2d_gb300")
    from fasttools2d_gb300 import selector

    rng = np.random.default_rng(3)
    n = 5000
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    rec = {"kind": 1, "tol": 1e-8, "n": n, "ntar": n, "Lx": 2.0, "Ly": 1.0, "qsum": float(np.sum(f1 ** 2 + f2 ** 2)),
           "feats": np.arange(8.0)}
    T = ft.choose_params(1, f1, f2, n, 2.0, 1.0, tol=1e-8, form=ft.FORM_MIXED)
    T2 = selector.tuned_of(rec)
    assert (T2.nside_x, T2.Mx, T2.P) == (T.nside_x, T.Mx, T.P) and T2.xi == pytest.approx(T.xi)
    # rows: the tuned choice, a faster candidate that misses the tolerance,
    # and a faster one that meets it
    rows = [[T.P, T.nside_x, T.nside_y, T.Mx, T.My, T.xi, 0, 5.0, 2e-9],
            [T.P - 2, 2 * T.nside_x, 2 * T.nside_y, T.Mx, T.My, T.xi, 0, 2.0, 3e-8],
            [T.P - 2, 2 * T.nside_x, 2 * T.nside_y, 2 * T.Mx, 2 * T.My, 1.5 * T.xi, 0, 3.0, 4e-9]]
    rec["cands"] = np.array(rows, dtype=np.float64)
    y, tb, tT = selector.label_targets(rec)
    assert tb == 3.0 and tT == 5.0
    assert np.allclose(y, [np.log(2.0), np.log(1.5), np.log(2.0), -1.0])
    # a candidate saving less than LABEL_GAIN leaves the label at the tuned choice
    rec3 = dict(rec, cands=rec["cands"].copy())
    rec3["cands"][2, 7] = 4.9
    y3, tb3, _ = selector.label_targets(rec3)
    assert tb3 == 5.0 and np.allclose(y3, [0.0, 0.0, 0.0, 0.0])
    rec2 = dict(rec, cands=rec["cands"][:2])
    rec2["cands"][0, 8] = 1e-7
    assert selector.label_targets(rec2) is None
    path = str(tmp_path / "recs.npz")
    selector.save_records(path, [rec, rec])
    back = selector.load_records(path)
    assert len(back) == 2 and np.array_equal(back[1]["cands"], rec["cands"])
    assert back[0]["qsum"] == rec["qsum"] and back[0]["kind"] == 1
