"""Oracle of the neural cache (hash-grid encoding + 2x64 MLP): the analytic gradients agree
with FP64 central finite differences, the encoding blends the right corners, and dense and
hashed levels index the table as defined."""
import numpy as np
import pytest


def _model(oracle, dim=3, levels=16, log2T=10, seed=0):
    rng = np.random.default_rng(seed)
    base, top = 4.0, 256.0
    b = np.exp((np.log(top) - np.log(base)) / (levels - 1))
    res = np.floor(base * b ** np.arange(levels)).astype(np.float32)
    T = 1 << log2T
    table = rng.uniform(-0.5, 0.5, (levels, T, 2)).astype(np.float32)
    I = 2 * levels
    W1 = rng.normal(0, np.sqrt(2 / I), (64, I)).astype(np.float32)
    W2 = rng.normal(0, np.sqrt(2 / 64), (64, 64)).astype(np.float32)
    w3 = rng.normal(0, np.sqrt(1 / 64), 64).astype(np.float32)
    b1 = rng.normal(0, 0.1, 64).astype(np.float32)
    b2 = rng.normal(0, 0.1, 64).astype(np.float32)
    lo = np.full(dim, -1.5, np.float32)
    inv = np.full(dim, 1 / 3.0, np.float32)
    return oracle.CacheModel(dim, res, lo, inv, table, W1, b1, W2, b2, w3, 0.3)


def _loss(oracle, m, x, t):
    return m.loss_and_grads(x, t)[0]


@pytest.mark.parametrize("dim", [2, 3])
def test_cache_gradients_match_finite_differences(oracle, dim):
    m = _model(oracle, dim=dim)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1.2, 1.2, (24, dim)).astype(np.float32)
    t = rng.uniform(-1, 1, 24).astype(np.float32)
    loss, g = m.loss_and_grads(x, t)
    assert loss > 0
    checked = 0
    for name in ("W1", "b1", "W2", "b2", "w3", "table"):
        arr = getattr(m, name)
        flat = arr.reshape(-1)
        gflat = g[name].reshape(-1)
        if name == "table":
            cand = np.nonzero(np.abs(gflat) > 1e-6)[0]      # entries the batch touches
        else:
            cand = np.arange(flat.size)
        for k in rng.choice(cand, size=min(12, cand.size), replace=False):
            old = flat[k]
            ok = False
            for h in (1e-3, 2.5e-4):
                up, dn = np.float32(old + h), np.float32(old - h)
                flat[k] = up
                lu = _loss(oracle, m, x, t)
                flat[k] = dn
                ld = _loss(oracle, m, x, t)
                flat[k] = old
                fd = (lu - ld) / (float(up) - float(dn))
                # a ReLU kink inside [old - h, old + h] spoils one step size, not both
                ok = ok or abs(fd - gflat[k]) <= 1e-3 * max(abs(fd), abs(gflat[k])) + 1e-7
            assert ok, (name, k, fd, gflat[k])
            checked += 1
    # b3: d loss / d b3 = mean 2 (y - t)
    y = m.forward(x)
    assert g["b3"][0] == pytest.approx(np.mean(2 * (y - t)), rel=1e-12)
    assert checked >= 60


def test_cache_encoding_is_a_partition_of_unity_blend(oracle):
    m = _model(oracle, dim=3)
    rng = np.random.default_rng(2)
    x = rng.uniform(-1.4, 1.4, (200, 3)).astype(np.float32)
    idx, w = m.corners(x)
    assert np.allclose(w.sum(axis=2), 1.0, atol=1e-12)
    assert np.all(w >= 0)
    # the encoding is the corner blend of the table
    _, enc = m.forward(x, with_encoding=True)
    T = m.table.shape[1]
    for lvl in (0, 7, 15):
        f = (w[:, lvl, :, None] * m.table[lvl][idx[:, lvl, :]].astype(np.float64)).sum(axis=1)
        assert np.allclose(enc[:, 2 * lvl:2 * lvl + 2], f, atol=1e-12)
        assert idx[:, lvl].max() < T


def test_cache_dense_and_hashed_indexing(oracle):
    m = _model(oracle, dim=3, log2T=10)
    # level 0 (res 4): (4+1)^3 = 125 <= 1024 entries -> dense; corner (0,0,0) of cell 0 is 0
    x = np.array([[-1.5, -1.5, -1.5]], np.float32)
    idx, w = m.corners(x)
    assert idx[0, 0, 0] == 0 and w[0, 0, 0] == pytest.approx(1.0)
    # dense: corner bits (1,0,0) -> +1, (0,1,0) -> +(res+1), (0,0,1) -> +(res+1)^2
    r = int(m.res[0])
    assert list(idx[0, 0, [1, 2, 4]]) == [1, r + 1, (r + 1) ** 2]
    # the finest level hashes: (c0 * 1) ^ (c1 * 2654435761) ^ (c2 * 805459861) mod T
    lvl = m.levels - 1
    res = float(m.res[lvl])
    p = np.float32(0.37)
    xx = np.array([[p, -0.2, 0.9]], np.float32)
    idx, _ = m.corners(xx)
    cell = []
    for i in range(3):
        xn = np.float32((xx[0, i] - m.lo[i]) * m.inv[i])
        c = np.floor(np.float32(xn * np.float32(res)))
        cell.append(int(min(c, res - 1)))
    h = (cell[0] * 1) ^ ((cell[1] * 2654435761) & 0xFFFFFFFF) ^ ((cell[2] * 805459861) & 0xFFFFFFFF)
    assert idx[0, lvl, 0] == (h & 0xFFFFFFFF) % m.table.shape[1]
