"""Neural cache on the GPU against its FP64 oracle: hash-grid corner indexing (exact),
encoding, forward pass and gradients of the BF16 tensor-core network, training, and the
cached solve (identical to the plain walk when no walk qualifies for early termination,
unbiased with an exact cache)."""
import numpy as np
import pytest

from zombie_gb300 import _abi as A
from zombie_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _cache(dim, log2T=12, seed=0, max_resolution=512.0, **kw):
    from zombie_gb300 import api
    lo, hi = np.full(dim, -1.5), np.full(dim, 1.5)
    return api.NeuralCache(dim, lo, hi, n_levels=16, log2_table_size=log2T, base_resolution=4.0,
                           max_resolution=max_resolution, seed=seed, padding=0.0, **kw)


def _random_params(c, rng, table_scale=0.5):
    p = c.get_parameters()
    v = c.split(p)
    v["table"][:] = rng.uniform(-table_scale, table_scale, v["table"].shape)
    v["W1"][:] = rng.normal(0, np.sqrt(2 / 32), v["W1"].shape)
    v["W2"][:] = rng.normal(0, np.sqrt(2 / 64), v["W2"].shape)
    v["b1"][:] = rng.normal(0, 0.1, 64)
    v["b2"][:] = rng.normal(0, 0.1, 64)
    v["w3"][:] = rng.normal(0, np.sqrt(1 / 64), 64)
    v["b3"][:] = 0.2
    c.set_parameters(p)
    return p


def _oracle_model(oracle, c, p):
    """The oracle model with the parameters the GPU computes with: the FP16 table, and the FP32
    weights (the GPU splits them into BF16 hi + lo)."""
    v = c.split(p)
    cfg = c.config
    lo = np.array(cfg.domain_min[:c.dim], np.float32)
    inv = (1.0 / (np.array(cfg.domain_max[:c.dim], np.float32) - lo)).astype(np.float32)
    return oracle.CacheModel(c.dim, c.resolutions, lo, inv, v["table"].astype(np.float16).astype(np.float32),
                             v["W1"], v["b1"], v["W2"], v["b2"], v["w3"], float(v["b3"][0]))


@pytest.mark.parametrize("dim", [2, 3])
def test_cache_encoding_matches_oracle(zgpu, oracle, dim):
    c = _cache(dim)
    p = _random_params(c, np.random.default_rng(1))
    m = _oracle_model(oracle, c, p)
    x = np.random.default_rng(2).uniform(-1.5, 1.5, (4000, dim)).astype(np.float32)
    enc = c.encode(x)
    _, oenc = m.forward(x, with_encoding=True)
    # the same corners and weights: FP32 blend vs FP64 blend of the same FP16 entries
    assert np.max(np.abs(enc - oenc)) <= 2e-6


@pytest.mark.parametrize("dim", [2, 3])
def test_cache_forward_and_gradients_match_oracle(zgpu, oracle, dim):
    c = _cache(dim)
    rng = np.random.default_rng(3)
    p = _random_params(c, rng)
    m = _oracle_model(oracle, c, p)
    n = 1000                                       # not a multiple of the 64-point block
    x = rng.uniform(-1.5, 1.5, (n, dim)).astype(np.float32)
    t = rng.uniform(-1, 1, n).astype(np.float32)
    y = c.evaluate(x)
    oy = m.forward(x)
    scale = np.sqrt(np.mean(oy ** 2))
    # activations and weights enter the tensor cores as BF16 hi + lo pairs (~16 mantissa bits,
    # hi*hi + lo*hi + hi*lo): FP32-class agreement with the FP64 oracle
    assert np.max(np.abs(y - oy)) <= 2e-4 * scale
    assert np.sqrt(np.mean((y - oy) ** 2)) <= 5e-5 * scale
    loss, g = c.gradients(x, t)
    oloss, og = m.loss_and_grads(x, t)
    assert loss == pytest.approx(oloss, rel=2e-2)
    gv = c.split(g)
    for name in ("table", "W1", "b1", "W2", "b2", "w3", "b3"):
        a = gv[name].astype(np.float64).ravel()
        b = og[name].ravel()
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel <= 4e-2, (name, rel)
        assert cos >= 0.999, (name, cos)


def test_cache_training_fits_a_smooth_field(zgpu):
    # a smooth field wants a coarse grid: at resolution 64 every cell holds many samples, and a
    # 2^19 table indexes every level densely (no hash collisions)
    c = _cache(3, log2T=19, max_resolution=64.0, learning_rate_grid=1e-2, learning_rate_mlp=5e-3)
    rng = np.random.default_rng(4)
    n = 1 << 17
    x = rng.uniform(-1.2, 1.2, (n, 3)).astype(np.float32)
    f = lambda q: np.exp(0.5 * q[:, 0]) * np.cos(q[:, 1]) + q[:, 2] ** 2
    t = f(x).astype(np.float32)
    first = c.train(x, t, steps=20, batch_size=1 << 14)
    c.train(x, t, steps=500, batch_size=1 << 14)
    # Adam at a fixed step keeps jittering around the minimum: decay it to converge
    for scale in (0.3, 0.1, 0.03):
        c.set_learning_rates(1e-2 * scale, 5e-3 * scale)
        last = c.train(x, t, steps=150, batch_size=1 << 14)
    assert last < 1e-4 * first
    xt = rng.uniform(-1.0, 1.0, (20000, 3)).astype(np.float32)
    err = c.evaluate(xt) - f(xt)
    assert np.sqrt(np.mean(err ** 2)) < 1e-2


def _solve(gp, cache=None, min_distance=0.05):
    d = gp.device_arrays()
    rep = gp.solve(d, cache=cache, cache_min_distance=min_distance)
    return d, rep


def test_cached_solve_without_qualifying_walks_equals_plain_solve(zgpu):
    from zombie_gb300.runner import GpuProblem
    gp = GpuProblem(P.laplace_wos_2d(n_segments=512, grid=24, spp=32))
    c = _cache(2)
    a, ra = _solve(gp)
    b, rb = _solve(gp, cache=c, min_distance=1e9)
    assert rb.cache_terminated == 0
    for k in ("n_solution_estimates", "total_walk_length", "solution_mean", "solution_m2"):
        assert np.array_equal(a[k].cpu().numpy(), b[k].cpu().numpy()), k
    assert ra.total_steps == rb.total_steps


def test_cached_solve_with_an_exact_cache_is_unbiased_and_shorter(zgpu):
    """Train the cache on the exact solution (noise-free), then end walks through it: the
    estimates stay within their standard errors of the exact solution while walks shorten."""
    from zombie_gb300.runner import GpuProblem
    pr = P.laplace_wos_2d(n_segments=1024, grid=48, spp=256)
    gp = GpuProblem(pr)
    c = _cache(2, log2T=16, max_resolution=128.0, learning_rate_grid=1e-2, learning_rate_mlp=5e-3)
    rng = np.random.default_rng(5)
    lo, hi = pr.domain_min[:2], pr.domain_max[:2]
    xt = rng.uniform(lo, hi, (1 << 17, 2)).astype(np.float32)
    c.train(xt, pr.exact(xt).astype(np.float32), steps=800, batch_size=1 << 14)
    xs = pr.points
    cache_err = np.sqrt(np.mean((c.evaluate(xs) - pr.exact(xs)) ** 2))
    plain, rp = _solve(gp)
    cached, rc = _solve(gp, cache=c, min_distance=0.05)
    assert rc.cache_terminated > 0.5 * rc.total_walks
    assert rc.total_steps < 0.5 * rp.total_steps
    ex = pr.exact()
    n = cached["n_solution_estimates"].cpu().numpy().astype(np.float64)
    assert np.array_equal(n, plain["n_solution_estimates"].cpu().numpy())
    mean = cached["solution_mean"].cpu().numpy()
    var = cached["solution_m2"].cpu().numpy() / np.maximum(n - 1, 1)
    se = np.sqrt(var / n)
    err = mean - ex
    # bias bounded by the cache error; the mean error is within a few standard errors of it
    assert abs(np.mean(err)) <= cache_err + 4 * np.sqrt(np.mean(se ** 2) / len(err))
    assert np.sqrt(np.mean(err ** 2)) <= np.sqrt(np.mean(se ** 2)) + 2 * cache_err
