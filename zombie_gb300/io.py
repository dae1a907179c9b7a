"""Boundary meshes and images in the reference's file formats, and its mesh helpers:
loadBoundaryMesh / loadTexturedBoundaryMesh (utils/fcpw_geometric_queries.h:158-252; FCPW's
OBJ soup readers: `v` positions, `vt` texture coordinates, `l` polylines in 2D, `f` polygons
in 3D, fan-triangulated), normalize / applyShift / flipOrientation / computeBoundingBox
(:255-313), buildBoundingBoxMesh / addBoundingBoxToBoundaryMesh (:318-402),
computeSignedVolume (:421-455), partitionBoundaryMesh (:460-510),
getSpatiallySortedPointIndices (utils/nearest_neighbor_finder.h:60-66), and PFM images
(demo/image.h:190-295: `Pf` one channel / `PF` three, negative scale = little endian, rows
stored bottom to top).  Host-side file and mesh handling around the solver; no compute here.

Where the reference fills output lists (`positions`, `indices`, ...), these functions accept
lists in the same positions and fill them (rows as numpy arrays); they also return the
results as arrays."""
import numpy as np


def _fill(out, arr):
    """Replaces the contents of an output list with the rows of arr (no-op for None)."""
    if out is not None:
        out.clear()
        out.extend(np.array(row) for row in np.asarray(arr))
    return arr


def _obj_index(tok, n):
    i = int(tok.split("/")[0])
    return i - 1 if i > 0 else n + i          # OBJ indices are 1-based, negative = relative


def load_boundary_mesh(obj_file, dim):
    """positions [V, dim] float32 and indices [P, dim] int32 of a segment (2D) or triangle (3D)
    soup from an OBJ file."""
    if dim not in (2, 3):
        raise ValueError("dim must be 2 or 3")
    pos, idx = [], []
    with open(obj_file) as f:
        for line in f:
            t = line.split()
            if not t or t[0].startswith("#"):
                continue
            if t[0] == "v":
                pos.append([float(v) for v in t[1:1 + dim]])
            elif dim == 2 and t[0] == "l":
                ids = [_obj_index(v, len(pos)) for v in t[1:]]
                idx.extend([ids[k], ids[k + 1]] for k in range(len(ids) - 1))
            elif dim == 3 and t[0] == "f":
                ids = [_obj_index(v, len(pos)) for v in t[1:]]
                idx.extend([ids[0], ids[k], ids[k + 1]] for k in range(1, len(ids) - 1))
    positions = np.asarray(pos, np.float32).reshape(-1, dim)
    indices = np.asarray(idx, np.int32).reshape(-1, dim)
    if indices.size and (indices.min() < 0 or indices.max() >= positions.shape[0]):
        raise ValueError(f"{obj_file}: face index outside the vertex list")
    return positions, indices


def write_boundary_mesh(obj_file, positions, indices):
    positions = np.asarray(positions)
    indices = np.asarray(indices)
    dim = positions.shape[1]
    with open(obj_file, "w") as f:
        for p in positions:
            f.write("v " + " ".join(f"{v:.9g}" for v in p) + (" 0\n" if dim == 2 else "\n"))
        key = "l" if dim == 2 else "f"
        for e in indices:
            f.write(key + " " + " ".join(str(int(i) + 1) for i in e) + "\n")


def normalize(positions):
    """Centres the positions on their mean and scales them into the unit ball (in place)."""
    positions -= positions.mean(axis=0)
    positions /= np.max(np.linalg.norm(positions, axis=1))
    return positions


def apply_shift(shift, positions):
    positions += np.asarray(shift, positions.dtype)
    return positions


def flip_orientation(indices):
    """Swaps the first two indices of every primitive (reverses its normal), in place."""
    indices[:, [0, 1]] = indices[:, [1, 0]]
    return indices


def compute_bounding_box(positions, make_square=True, scale=1.0):
    """The box of the positions scaled by `scale` about their mean; a square / cube about its
    centre when make_square."""
    p = np.asarray(positions, np.float64)
    cm = p.mean(axis=0)
    q = (p - cm) * scale + cm
    lo, hi = q.min(axis=0), q.max(axis=0)
    if make_square:
        c, h = 0.5 * (lo + hi), 0.5 * (hi - lo).max()
        lo, hi = c - h, c + h
    return lo.astype(np.float32), hi.astype(np.float32)


def read_pfm(filename):
    """A PFM image as float32 [height, width] (Pf) or [height, width, 3] (PF), row 0 at the top."""
    with open(filename, "rb") as f:
        header = f.readline().strip()
        if header not in (b"Pf", b"PF"):
            raise ValueError(f"{filename}: not a PFM file")
        channels = 3 if header == b"PF" else 1
        dims = f.readline().split()
        while len(dims) < 2:
            dims += f.readline().split()
        w, h = int(dims[0]), int(dims[1])
        scale = float(f.readline().strip())
        data = np.frombuffer(f.read(w * h * channels * 4), dtype="<f4" if scale < 0 else ">f4")
    img = data.astype(np.float32).reshape(h, w, channels)[::-1]
    return np.ascontiguousarray(img[:, :, 0] if channels == 1 else img)


def write_pfm(filename, image):
    """Writes a [height, width] or [height, width, 3] float image (row 0 at the top) as PFM,
    little endian."""
    img = np.asarray(image, np.float32)
    channels = 1 if img.ndim == 2 else img.shape[2]
    if channels not in (1, 3):
        raise ValueError("PFM holds 1 or 3 channels")
    h, w = img.shape[:2]
    with open(filename, "wb") as f:
        f.write(b"Pf\n" if channels == 1 else b"PF\n")
        f.write(f"{w} {h}\n-1\n".encode())
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())


def image_to_grid(image, grid_min, grid_max, enable_interpolation=True):
    """A 2D image (row 0 at the top of the box) as the dense grid the demo's model problems
    read PDE data from: x along the columns, y along the rows (bottom row at grid_min)."""
    from .api import DenseGrid
    img = np.asarray(image, np.float32)
    if img.ndim == 3:
        img = img[:, :, 0]
    data = np.ascontiguousarray(img[::-1].T)      # [x][y], y growing upwards
    return DenseGrid(data, data.shape, grid_min, grid_max, enable_interpolation)


def load_textured_boundary_mesh(obj_file, positions=None, texture_coordinates=None, indices=None,
                                texture_indices=None):
    """A triangle soup with texture coordinates (3D only): positions [V, 3], texture
    coordinates [T, 2], position indices [P, 3] and texture-coordinate indices [P, 3]."""
    pos, uv, idx, tidx = [], [], [], []
    with open(obj_file) as f:
        for line in f:
            t = line.split()
            if not t or t[0].startswith("#"):
                continue
            if t[0] == "v":
                pos.append([float(v) for v in t[1:4]])
            elif t[0] == "vt":
                uv.append([float(v) for v in t[1:3]])
            elif t[0] == "f":
                corners = [c.split("/") for c in t[1:]]
                vi = [_obj_index(c[0], len(pos)) for c in corners]
                ti = [_obj_index(c[1], len(uv)) if len(c) > 1 and c[1] else -1 for c in corners]
                for k in range(1, len(vi) - 1):
                    idx.append([vi[0], vi[k], vi[k + 1]])
                    tidx.append([ti[0], ti[k], ti[k + 1]])
    P = np.asarray(pos, np.float32).reshape(-1, 3)
    T = np.asarray(uv, np.float32).reshape(-1, 2)
    I = np.asarray(idx, np.int32).reshape(-1, 3)
    TI = np.asarray(tidx, np.int32).reshape(-1, 3)
    if I.size and (I.min() < 0 or I.max() >= P.shape[0]):
        raise ValueError(f"{obj_file}: face index outside the vertex list")
    if TI.size and TI.max() >= T.shape[0]:
        raise ValueError(f"{obj_file}: texture index outside the texture-coordinate list")
    return (_fill(positions, P), _fill(texture_coordinates, T), _fill(indices, I), _fill(texture_indices, TI))


# corner order and faces of the box mesh (buildBoundingBoxMesh): the same corners, the same
# outward-facing primitives, so meshes built either way match primitive for primitive
_BOX_CORNERS = {2: [(0, 0), (1, 0), (1, 1), (0, 1)],
                3: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]}
_BOX_FACES = {2: [(0, 1), (1, 2), (2, 3), (3, 0)],
              3: [(0, 2, 1), (0, 3, 2), (0, 5, 4), (0, 1, 5), (0, 7, 3), (0, 4, 7),
                  (6, 7, 4), (6, 4, 5), (6, 5, 1), (6, 1, 2), (6, 2, 3), (6, 3, 7)]}


def build_bounding_box_mesh(bounding_box_min, bounding_box_max, positions=None, indices=None):
    """The boundary of the box as a segment (2D) or triangle (3D) mesh."""
    lo = np.asarray(bounding_box_min, np.float32).ravel()
    hi = np.asarray(bounding_box_max, np.float32).ravel()
    dim = lo.size
    if dim not in (2, 3) or hi.size != dim:
        raise ValueError("the box corners must have 2 or 3 entries")
    sel = np.asarray(_BOX_CORNERS[dim], bool)
    P = np.where(sel, hi, lo).astype(np.float32)
    I = np.asarray(_BOX_FACES[dim], np.int32)
    return _fill(positions, P), _fill(indices, I)


def add_bounding_box_to_boundary_mesh(bounding_box_min, bounding_box_max, positions, indices):
    """Appends the box mesh to a boundary mesh (its indices offset past the existing
    vertices).  Lists are extended in place; for arrays the enlarged arrays are returned."""
    bp, bi = build_bounding_box_mesh(bounding_box_min, bounding_box_max)
    V = len(positions)
    if isinstance(positions, list) and isinstance(indices, list):
        positions.extend(np.array(r) for r in bp)
        indices.extend(np.array(r) for r in bi + V)
        return positions, indices
    P = np.concatenate([np.asarray(positions, np.float32).reshape(-1, bp.shape[1]), bp])
    I = np.concatenate([np.asarray(indices, np.int32).reshape(-1, bi.shape[1]), bi + V])
    return P, I


def compute_signed_volume(boundary_positions, boundary_indices):
    """Signed area (2D, sum of p0 x p1 / 2 over segments) or volume (3D, sum of
    p0 . (p1 x p2) / 6 over triangles) enclosed by the mesh: positive for outward
    (counter-clockwise) orientation."""
    p = np.asarray(boundary_positions, np.float64)
    dim = p.shape[1]
    idx = np.asarray(boundary_indices, np.int64).reshape(-1, dim)
    q = p[idx]
    if dim == 2:
        return float(0.5 * np.sum(q[:, 0, 0] * q[:, 1, 1] - q[:, 0, 1] * q[:, 1, 0]))
    return float(np.sum(np.einsum("ij,ij->i", np.cross(q[:, 0], q[:, 1]), q[:, 2])) / 6.0)


def partition_boundary_mesh(on_reflecting_boundary, positions, indices, absorbing_positions=None,
                            absorbing_indices=None, reflecting_positions=None, reflecting_indices=None):
    """Splits a boundary mesh into absorbing and reflecting parts by where each primitive's
    midpoint lies (on_reflecting_boundary takes an [N, dim] array, or one point at a time);
    each part keeps only its own vertices, renumbered in their original order.  Returns
    ((absorbing_positions, absorbing_indices), (reflecting_positions, reflecting_indices))."""
    positions = np.asarray(positions)
    dim = positions.shape[1]
    indices = np.asarray(indices).reshape(-1, dim)
    mids = positions[indices].mean(1)
    try:
        refl = np.asarray(on_reflecting_boundary(mids), bool)
        if refl.shape != (mids.shape[0],):
            raise TypeError
    except Exception:
        refl = np.array([bool(on_reflecting_boundary(m)) for m in mids], bool)
    out = []
    for mask in (~refl, refl):
        sub = indices[mask]
        if sub.size == 0:
            out.append((np.zeros((0, dim), np.float32), np.zeros((0, dim), np.int32)))
            continue
        uniq, inv = np.unique(sub.reshape(-1), return_inverse=True)
        out.append((positions[uniq].astype(np.float32), inv.reshape(sub.shape).astype(np.int32)))
    _fill(absorbing_positions, out[0][0]); _fill(absorbing_indices, out[0][1])
    _fill(reflecting_positions, out[1][0]); _fill(reflecting_indices, out[1][1])
    return out[0], out[1]


def get_spatially_sorted_point_indices(points, out_indices=None):
    """A permutation that orders the points along a Morton (Z-order) curve over their
    bounding box, 21 bits per axis.  The reference returns its k-d tree's leaf order
    (nanoflann); both are spatially coherent orders, not the same permutation."""
    x = np.asarray(points, np.float64)
    if x.size == 0:
        if out_indices is not None:
            out_indices.clear()
        return np.zeros(0, np.uint32)
    n, dim = x.shape
    lo, hi = x.min(0), x.max(0)
    q = np.floor((x - lo) / np.where(hi > lo, hi - lo, 1.0) * ((1 << 21) - 1)).astype(np.uint64)
    code = np.zeros(n, np.uint64)
    for bit in range(21):
        for d in range(dim):
            code |= ((q[:, d] >> np.uint64(bit)) & np.uint64(1)) << np.uint64(bit * dim + d)
    order = np.argsort(code, kind="stable").astype(np.uint32)
    if out_indices is not None:
        out_indices.clear()
        out_indices.extend(int(i) for i in order)
    return order
