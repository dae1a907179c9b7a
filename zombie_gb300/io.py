"""Boundary meshes and images in the reference's file formats, and its mesh helpers:
loadBoundaryMesh (utils/fcpw_geometric_queries.h:158-211; FCPW's OBJ soup readers: `v`
positions, `l` polylines in 2D, `f` polygons in 3D, fan-triangulated), normalize /
applyShift / flipOrientation / computeBoundingBox (:255-313), and PFM images
(demo/image.h:190-295: `Pf` one channel / `PF` three, negative scale = little endian, rows
stored bottom to top).  Host-side file handling around the solver; no compute here."""
import numpy as np


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
