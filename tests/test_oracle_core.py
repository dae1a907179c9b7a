"""Pins the CPU oracle: RNG known answers, Bessel tables, Green's-function identities."""
import json
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def test_pcg32_known_answer(oracle):
    u, f = oracle.pcg32(42, 54, 6)
    assert [hex(int(x)) for x in u] == GOLDEN["pcg32_seed42_stream54"]
    # nextFloat: top 23 bits of the same stream in [0, 1)
    assert np.allclose(f, (u >> 9).astype(np.float64) / 2.0 ** 23, rtol=0, atol=0)


@pytest.mark.parametrize("which", ["i0", "i1", "k0", "k1"])
def test_bessel_tables(oracle, which):
    # A&S 9.8 polynomial approximations: relative error well below 1e-6 on these points
    for x, ref in GOLDEN["bessel"][which]:
        assert abs(oracle.bessel(which, x) - ref) <= 2e-7 * abs(ref)


@pytest.mark.parametrize("which", ["i0", "i1", "k0", "k1"])
def test_bessel_against_scipy(oracle, which):
    sp = pytest.importorskip("scipy.special")
    xs = np.concatenate([np.linspace(1e-3, 3.7, 40), np.linspace(3.8, 30.0, 40)])
    for x in xs:
        ref = getattr(sp, which)(x)
        assert abs(oracle.bessel(which, float(x)) - ref) <= 1e-6 * abs(ref)


def _shell_integral(dim, fn, a, b, n):
    # integral of fn over the shell a < |x| < b, by the midpoint rule in r (G is integrable at 0)
    r = a + (np.arange(n) + 0.5) * (b - a) / n
    w = 2 * np.pi * r if dim == 2 else 4 * np.pi * r * r
    return float(np.sum(np.array([fn(x) for x in r]) * w) * (b - a) / n)


@pytest.mark.parametrize("dim,yukawa,lam", [(2, 0, 0.0), (3, 0, 0.0), (2, 1, 1.0), (3, 1, 4.0), (2, 1, 16.0)])
def test_greens_norm_is_integral(oracle, dim, yukawa, lam):
    """GreensFnBall::norm() equals the integral of G over the ball (distributions.h:489-491, :739-742)."""
    R = 0.7
    L = oracle.lib()
    norm = L.orc_greens_norm(dim, yukawa, lam, R)
    integral = _shell_integral(dim, lambda r: L.orc_greens_evaluate(dim, yukawa, lam, R, r), 0.0, R, 4000)
    assert abs(norm - integral) <= 2e-3 * abs(norm)


@pytest.mark.parametrize("dim,yukawa,lam", [(2, 0, 0.0), (3, 0, 0.0), (2, 1, 1.0), (3, 1, 4.0)])
def test_greens_radius_sampling_matches_pdf(oracle, dim, yukawa, lam):
    """sampleVolume draws radii with density G(r) * |sphere(r)| / norm (distributions.h:460-470, :419-440)."""
    R = 0.8
    L = oracle.lib()
    n = 200000
    out = np.zeros(n, np.float32)
    L.orc_greens_sample_radii(dim, yukawa, lam, R, 1234, n, out.ctypes.data)
    edges = np.linspace(0, R, 17)
    hist = np.histogram(out, edges)[0] / n
    norm = L.orc_greens_norm(dim, yukawa, lam, R)
    expect = []
    for a, b in zip(edges[:-1], edges[1:]):
        expect.append(_shell_integral(dim, lambda r: L.orc_greens_evaluate(dim, yukawa, lam, R, r), a, b, 400) / norm)
    expect = np.array(expect)
    sd = np.sqrt(expect * (1 - expect) / n)
    assert np.all(np.abs(hist - expect) <= 5 * sd + 2e-3)
