"""Path-guiding network without a GPU: the host build of the forward pass
against the FP64 oracle, and the oracle's analytic gradients against finite
differences of its own loss."""
import numpy as np

from libyafaray_gb300 import gbrt
from oracle import guide_oracle as go

BOUND = [-1.0, 0.0, -1.0, 1.0, 2.0, 1.0]


def _params(rng, log2_table=12):
    mlp = np.zeros(go.N_MLP, np.float64)
    for off, rows, cols in [(go.OFF_W1, 64, 32), (go.OFF_W2, 64, 64), (go.OFF_W3, 40, 64)]:
        mlp[off:off + rows * cols] = rng.uniform(-np.sqrt(6 / cols), np.sqrt(6 / cols), rows * cols)
    mlp[go.OFF_B1:go.OFF_W2] = rng.uniform(-0.1, 0.3, 64)
    mlp[go.OFF_B2:go.OFF_W3] = rng.uniform(-0.1, 0.3, 64)
    mlp[go.OFF_B3:] = rng.normal(0, 0.5, 40)
    tab = rng.uniform(-0.5, 0.5, (16, 1 << log2_table, 2))
    return mlp, tab


def _records(rng, n):
    r = np.zeros((n, 8))
    r[:, 0] = rng.uniform(-1, 1, n); r[:, 1] = rng.uniform(0, 2, n); r[:, 2] = rng.uniform(-1, 1, n)
    d = rng.normal(size=(n, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3:6] = d
    r[:, 6] = rng.exponential(1.0, n)
    return r


def test_host_forward_matches_fp64_oracle(gbrt_lib):
    rng = np.random.default_rng(11)
    mlp, tab = _params(rng)
    rec = _records(rng, 64)
    got = gbrt.guide_forward_host(BOUND, mlp.astype(np.float32), tab.astype(np.float32), rec[:, :3], log2_table=12)
    grid = go.Grid(BOUND, log2_table=12)
    m32, t32 = mlp.astype(np.float32).astype(np.float64), tab.astype(np.float32).astype(np.float64)
    for i in range(len(rec)):
        e, _ = grid.encode(t32, rec[i, :3].astype(np.float32))
        _, _, o = go.mlp_forward(m32, e)
        assert np.allclose(got[i], go.lobes(o), rtol=1e-3, atol=1e-4), i


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(12)
    mlp, tab = _params(rng, log2_table=10)
    rec = _records(rng, 6)
    grid = go.Grid(BOUND, log2_table=10)
    _, dm, dt = go.loss_and_grads(grid, mlp, tab, rec)
    h = 1e-6
    for idx in [0, 100, go.OFF_B1 + 3, go.OFF_W2 + 77, go.OFF_B2 + 5, go.OFF_W3 + 200, go.OFF_B3 + 4, go.OFF_B3 + 3]:
        mp, mm = mlp.copy(), mlp.copy()
        mp[idx] += h; mm[idx] -= h
        num = (go.loss_and_grads(grid, mp, tab, rec)[0] - go.loss_and_grads(grid, mm, tab, rec)[0]) / (2 * h)
        assert abs(num - dm[idx]) <= 1e-5 + 1e-4 * abs(num), (idx, num, dm[idx])
    nz = np.argwhere(np.abs(dt) > 1e-4)[:6]
    for (l, i, f) in nz:
        tp, tm = tab.copy(), tab.copy()
        tp[l, i, f] += h; tm[l, i, f] -= h
        num = (go.loss_and_grads(grid, mlp, tp, rec)[0] - go.loss_and_grads(grid, mlp, tm, rec)[0]) / (2 * h)
        assert abs(num - dt[l, i, f]) <= 1e-5 + 1e-4 * abs(num), ((l, i, f), num, dt[l, i, f])
