"""Boundary meshes (OBJ) and images (PFM) in the reference's formats, and the mesh helpers."""
import numpy as np
import pytest

from zombie_gb300 import io
from zombie_gb300 import problems as P


def test_obj_round_trip_2d_and_3d(tmp_path):
    pos, idx = P.star_polygon(64)
    f = tmp_path / "star.obj"
    io.write_boundary_mesh(f, pos, idx)
    p2, i2 = io.load_boundary_mesh(f, 2)
    assert np.allclose(p2, pos) and np.array_equal(i2, idx)
    pos3, idx3 = P.icosphere(2)
    f3 = tmp_path / "sphere.obj"
    io.write_boundary_mesh(f3, pos3, idx3)
    p3, i3 = io.load_boundary_mesh(f3, 3)
    assert np.allclose(p3, pos3) and np.array_equal(i3, idx3)


def test_obj_polylines_polygons_and_relative_indices(tmp_path):
    f = tmp_path / "mixed.obj"
    f.write_text("# square\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nl 1 2 3 4 1\n"
                 "f 1/1 2/1 3/1 -1/1\n")
    p, i = io.load_boundary_mesh(f, 2)
    assert p.shape == (4, 2) and i.tolist() == [[0, 1], [1, 2], [2, 3], [3, 0]]
    p, i = io.load_boundary_mesh(f, 3)
    assert i.tolist() == [[0, 1, 2], [0, 2, 3]]               # the quad fan-triangulated
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nl 1 5\n")
    with pytest.raises(ValueError):
        io.load_boundary_mesh(bad, 2)


def test_mesh_helpers():
    pos, idx = P.star_polygon(128)
    p = io.normalize(pos.astype(np.float64) * 3 + 5)
    assert np.allclose(p.mean(axis=0), 0, atol=1e-9) and np.max(np.linalg.norm(p, axis=1)) == pytest.approx(1.0)
    q = io.apply_shift([1.0, -2.0], p.copy())
    assert np.allclose(q - p, [1.0, -2.0])
    j = io.flip_orientation(idx.copy())
    assert np.array_equal(j[:, 0], idx[:, 1]) and np.array_equal(j[:, 1], idx[:, 0])
    lo, hi = io.compute_bounding_box(pos, True, 1.0)
    assert np.allclose(hi - lo, (hi - lo)[0]) and np.all(pos >= lo - 1e-6) and np.all(pos <= hi + 1e-6)
    lo2, hi2 = P.bounding_box(pos)
    assert np.allclose(lo, lo2) and np.allclose(hi, hi2)


def test_pfm_round_trip_and_grid(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.normal(size=(5, 7)).astype(np.float32)
    f = tmp_path / "a.pfm"
    io.write_pfm(f, img)
    assert np.array_equal(io.read_pfm(f), img)
    rgb = rng.normal(size=(4, 3, 3)).astype(np.float32)
    io.write_pfm(tmp_path / "b.pfm", rgb)
    assert np.array_equal(io.read_pfm(tmp_path / "b.pfm"), rgb)
    # big-endian files read too (positive scale)
    be = tmp_path / "be.pfm"
    be.write_bytes(b"Pf\n7 5\n1.0\n" + np.ascontiguousarray(img[::-1]).astype(">f4").tobytes())
    assert np.array_equal(io.read_pfm(be), img)
    # as a dense grid: the top-left pixel sits at (min x, max y)
    g = io.image_to_grid(img, [0.0, 0.0], [7.0, 5.0], enable_interpolation=False)
    assert g([0.5, 4.5]) == pytest.approx(img[0, 0])
    assert g([6.5, 0.5]) == pytest.approx(img[4, 6])
