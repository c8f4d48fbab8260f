"""The radiance-cache oracle checked on its own (CPU): bf16 rounding known answers, the hash-grid
geometry, its gradient against finite differences, and the float32 Adam step."""
import numpy as np
import pytest

from oracle import nrc


def test_bf16_rounding_known_answers():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -7, -2.5, 0.0, 3.0e38], np.float32)
    got = nrc.bf16(x)
    # Halfway cases round to the even neighbour; 1 + 2^-7 is representable.
    assert list(got[:6]) == [1.0, 1.0, 1.0 + 2.0 ** -6, 1.0 + 2.0 ** -7, -2.5, 0.0]
    assert np.isfinite(got[6])


def grid_small(levels=4, log2=10):
    return nrc.Grid.from_config(levels, log2, 4, 64, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))


def test_grid_geometry():
    g = nrc.Grid.from_config(16, 19, 16, 2048, (0, 0, 0), (2, 1, 1))
    assert g.res[0] == 16 and g.res[-1] == 2048
    assert all(a <= b for a, b in zip(g.res, g.res[1:]))
    assert g.dense[0] and not g.dense[-1]  # 17^3 fits in 2^19 entries, 2049^3 does not
    rng = np.random.default_rng(1)
    pos = rng.uniform(-0.5, 2.5, (500, 3)).astype(np.float32)
    for l in range(16):
        idx, w = g.corners(pos, l)
        assert idx.min() >= 0 and idx.max() < g.entries
        assert np.allclose(w.sum(axis=1), 1.0, atol=1e-5)


def test_grid_gradient_matches_feature_perturbation():
    g = grid_small()
    rng = np.random.default_rng(2)
    table = rng.uniform(-1, 1, (g.levels, g.entries, 2)).astype(np.float16)
    rec = np.zeros((64, nrc.REC), np.float32)
    rec[:, :3] = rng.uniform(-1, 1, (64, 3))
    gx = np.zeros((64, 64))
    gx[:, :2 * g.levels] = rng.normal(size=(64, 2 * g.levels))
    grad = nrc.grid_gradient(g, rec, gx)
    # sum(gx * features) is linear in the table: its derivative at an entry is the scatter.
    base = np.sum(gx * nrc.inputs(g, table, rec).astype(np.float64))
    for (l, e, f) in [tuple(x) for x in np.argwhere(np.abs(grad) > 1e-3)[:6]]:
        t2 = table.astype(np.float32).copy()
        t2[l, e, f] += 1.0
        moved = np.sum(gx * nrc.inputs(g, t2, rec).astype(np.float64)) - base
        assert moved == pytest.approx(grad[l, e, f], rel=1e-3, abs=1e-4)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    mlp = (rng.normal(size=nrc.MLP_PARAMS) * 0.2).astype(np.float32)
    mlp[16384 + 3 * 64:] = 0.0
    ws = nrc.layers(mlp, rounded=False)
    x = rng.uniform(0, 1, (32, 64))
    y = rng.uniform(0, 2, (32, 3))
    _, _, out = nrc.forward(ws, x, rounded=False)
    den = out[:, :3] ** 2 + 0.01
    loss, dws, gx = nrc.backward(ws, x, y, rounded=False)
    assert loss == pytest.approx(nrc.loss_fixed_den(ws, x, y, den), rel=1e-12)
    h = 1e-6
    for l, (o, i) in [(0, (3, 7)), (1, (10, 20)), (2, (0, 63)), (3, (40, 1)), (4, (2, 33))]:
        wp = [w.copy() for w in ws]
        wm = [w.copy() for w in ws]
        wp[l][o, i] += h
        wm[l][o, i] -= h
        fd = (nrc.loss_fixed_den(wp, x, y, den) - nrc.loss_fixed_den(wm, x, y, den)) / (2 * h)
        assert dws[l][o, i] == pytest.approx(fd, rel=1e-5, abs=1e-7)
    for r, c in [(0, 0), (5, 33), (31, 44)]:
        xp, xm = x.copy(), x.copy()
        xp[r, c] += h
        xm[r, c] -= h
        fd = (nrc.loss_fixed_den(ws, xp, y, den) - nrc.loss_fixed_den(ws, xm, y, den)) / (2 * h)
        assert gx[r, c] == pytest.approx(fd, rel=1e-5, abs=1e-7)


def test_adam_first_step_moves_by_the_learning_rate():
    p = np.array([1.0, -2.0, 0.5, 0.0], np.float32)
    g = np.array([3.0, -6.0, 0.0, 1e-3], np.float32)
    p1, m, v = nrc.adam_f32(p, g, np.zeros(4), np.zeros(4), used=1, step=1, lr=0.01)
    # Bias-corrected first step: m_hat / sqrt(v_hat) = sign(g) when |g| >> eps.
    assert p1[0] == pytest.approx(0.99, abs=1e-6)
    assert p1[1] == pytest.approx(-1.99, abs=1e-6)
    assert p1[2] == 0.5
    assert p1[3] == pytest.approx(-0.01, abs=1e-5)
