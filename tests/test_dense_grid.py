"""Dense-grid PDE fields (DenseGrid<float, 1, DIM>, utils/dense_grid.h): the oracle's lookup
against a scalar restatement of the reference's nearest and bi/trilinear lookups (clamped
indices, clamped blend fractions, row-major with the last axis fastest), the host-side
DenseGrid of the Python API, and the get_dense_grid_*_callback overloads."""
import math

import numpy as np
import pytest

import zombie_gb300 as Z
from zombie_gb300 import _abi as A
from zombie_gb300 import api


def _lookup(data, shape, lo, hi, interp, x):
    """DenseGrid::operator() for one point, written the way dense_grid.h:264-355 reads."""
    D = len(shape)
    t = [(x[i] - lo[i]) / (hi[i] - lo[i]) for i in range(D)]
    if not interp:
        flat, stride = 0, 1
        for i in range(D - 1, -1, -1):
            idx = min(max(int(math.floor(t[i] * shape[i])), 0), shape[i] - 1)
            flat += idx * stride
            stride *= shape[i]
        return float(data[flat])
    u = [0.0 if shape[i] == 1 else t[i] * shape[i] - 0.5 for i in range(D)]
    i0 = [min(max(int(math.floor(u[i])), 0), shape[i] - 1) for i in range(D)]
    i1 = [min(max(i0[i] + 1, 0), shape[i] - 1) for i in range(D)]
    f = [min(max(u[i] - i0[i], 0.0), 1.0) for i in range(D)]
    if D == 2:
        def at(a, b):
            return float(data[a * shape[1] + b])
        x_, y_ = f
        return (at(i0[0], i0[1]) * (1 - x_) * (1 - y_) + at(i1[0], i0[1]) * x_ * (1 - y_) +
                at(i0[0], i1[1]) * (1 - x_) * y_ + at(i1[0], i1[1]) * x_ * y_)

    def at(a, b, c):
        return float(data[(a * shape[1] + b) * shape[2] + c])
    x_, y_, z_ = f
    s = 0.0
    for a, wa in ((i0[0], 1 - x_), (i1[0], x_)):
        for b, wb in ((i0[1], 1 - y_), (i1[1], y_)):
            for c, wc in ((i0[2], 1 - z_), (i1[2], z_)):
                s += at(a, b, c) * wa * wb * wc
    return s


CASES = [(2, (17, 9), False), (2, (17, 9), True), (2, (1, 12), True), (3, (7, 5, 6), False), (3, (7, 5, 6), True),
         (3, (4, 1, 3), True)]


def _grid(dim, shape, interp, seed):
    rng = np.random.default_rng(seed)
    lo = rng.uniform(-1.5, -0.5, dim).astype(np.float32)
    hi = (lo + rng.uniform(1.0, 3.0, dim)).astype(np.float32)
    data = rng.normal(size=int(np.prod(shape))).astype(np.float32)
    return api.DenseGrid(data, shape, lo, hi, interp)


@pytest.mark.parametrize("dim,shape,interp", CASES)
def test_oracle_grid_lookup_matches_dense_grid(oracle, dim, shape, interp):
    g = _grid(dim, shape, interp, 1)
    ga = _grid(dim, shape, interp, 2)
    ga.origin, ga.extent = g.origin, g.extent
    pde = api.PDE(dim)
    pde.source = Z.Utils.get_dense_grid_source_callback(g)
    pde.dirichlet = Z.Utils.get_dense_grid_dirichlet_callback(g, ga)
    pde.robin = Z.Utils.get_dense_grid_robin_callback(ga)
    pde.robin_coeff = Z.Utils.get_dense_grid_robin_coefficient_callback(g, ga)
    pde.are_robin_conditions_pure_neumann = False
    c = pde.to_c()
    rng = np.random.default_rng(3)
    # inside, on and outside the grid box (lookups clamp)
    x = rng.uniform(g.origin - 0.3 * g.extent, g.origin + 1.3 * g.extent, (400, dim)).astype(np.float32)
    x[:20] = g.get(rng.integers(0, g.data.size, 20))             # cell centres
    for aligned in (False, True):
        src, dr, rb, kp = oracle.eval_pde(dim, c, x, aligned=aligned, with_robin_coeff=True)
        ref = np.array([_lookup(g.data, shape, g.origin, g.origin + g.extent, interp, p) for p in x])
        ref_a = np.array([_lookup(ga.data, shape, g.origin, g.origin + g.extent, interp, p) for p in x])
        tol = 2e-6 * (1 + np.abs(ref).max())
        assert np.max(np.abs(src - ref)) <= tol                  # source ignores the orientation
        assert np.max(np.abs(dr - (ref_a if aligned else ref))) <= tol
        assert np.max(np.abs(rb - ref_a)) <= tol                 # one grid: both orientations read it
        assert np.max(np.abs(kp - (ref_a if aligned else ref))) <= tol
        # the host-side DenseGrid reads the same values
        assert np.max(np.abs(g(x) - ref)) <= tol
    # nearest lookups at cell centres return the stored samples
    if not interp:
        idx = rng.integers(0, g.data.size, 50)
        assert np.array_equal(oracle.eval_pde(dim, c, g.get(idx))[0], g.data[idx])


def test_dense_grid_from_callback_and_cell_centres():
    g = Z.Utils.DenseGrid([0.0, -1.0], [2.0, 1.0], True, dim=2)
    g.set(lambda p: 3.0 * p[0] - p[1], [8, 4])
    c = g.get(np.arange(32))
    assert np.allclose(c[0], [0.125, -0.75]) and np.allclose(c[31], [1.875, 0.75])
    assert np.allclose(g.data, 3.0 * c[:, 0] - c[:, 1], atol=1e-6)
    # bilinear lookups reproduce a linear field between the outermost cell centres
    x = np.random.default_rng(0).uniform([0.125, -0.75], [1.875, 0.75], (200, 2))
    assert np.allclose(g(x), 3.0 * x[:, 0] - x[:, 1], atol=1e-5)
    assert g.min() == pytest.approx(float(g.data.min())) and g.max() == pytest.approx(float(g.data.max()))


def test_dense_grid_callback_overloads():
    data, shape, lo, hi = np.arange(12.0), [3, 4], [0.0, 0.0], [3.0, 4.0]
    f = Z.Utils.get_dense_grid_dirichlet_callback(data, shape, lo, hi, True)
    assert f.kind == A.ZGPU_FIELD_GRID and f.grid_aligned is None and f.grid.interpolation_enabled
    f = Z.Utils.get_dense_grid_dirichlet_callback(data, 2 * data, shape, lo, hi)
    assert f.grid_aligned is not None and np.array_equal(f.grid_aligned.data, 2 * data.astype(np.float32))
    f = Z.Utils.get_dense_grid_robin_coefficient_callback(grid_data=data, grid_shape=shape, grid_min=lo, grid_max=hi,
                                                          enable_interpolation=False)
    assert not f.grid.interpolation_enabled
    with pytest.raises(TypeError):
        Z.Utils.get_dense_grid_source_callback(f.grid, f.grid)          # sources have no aligned variant
    with pytest.raises(ValueError):
        api.Field.dense_grid(api.DenseGrid(data, shape, lo, hi), api.DenseGrid(np.arange(6.0), [2, 3], lo, hi))
    with pytest.raises(ValueError):
        api.DenseGrid(np.arange(11.0), shape, lo, hi)
    c = f.grid_to_c()
    assert list(c.shape)[:2] == shape and c.enable_interpolation == 0 and c.values
    pde = api.PDE(2)
    pde.are_robin_conditions_pure_neumann = False
    pde.robin_coeff = f
    assert pde.has_non_zero_robin_coeff([0.5, 0.5]) is False          # the grid reads 0 there
    assert pde.has_non_zero_robin_coeff([2.5, 3.5]) is True
    p = pde.to_c()
    assert p.robin_coeff_kind == A.ZGPU_FIELD_GRID and p.memory == A.ZGPU_MEM_HOST
    assert api.PDE.from_c(2, p).robin_coeff.grid_to_c().values == c.values
