"""Solution output from device buffers: the reference's binary VTK PolyData
file (LBMSolver::output, src/lbm/solver.cpp:322-384, written through
VTK::BINARY::writePoints, src/common/IO.h:413-507).

The reference turns every value into a string and back (`toStringVector`,
then `std::stod` per point) before encoding it; here the moments come from the
GPU as FP64 arrays and go to the file with one NumPy base64 encode per array.
The file has the reference's layout -- one PolyData piece, Float32 point
coordinates, a single poly-vertex over all points (Int64 connectivity, ASCII
offsets), Float64 point data named U, V[, W] and rho for Navier-Stokes or V for
Poisson -- and each binary array is the VTK "binary" encoding with a UInt64
byte-count header, so ParaView and the reference's own post-processing read
both the same way.
"""
from __future__ import annotations

import base64
from typing import List, Optional, Sequence, Tuple

import numpy as np

VEL_NAMES = ("U", "V", "W")


def _b64(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    return base64.b64encode(np.uint64(a.nbytes).tobytes() + a.tobytes()).decode("ascii")


def reference_rounding(v: np.ndarray) -> np.ndarray:
    """The values the reference's file holds: it prints each value with
    std::fixed and 15 digits (toStringVector, include/common/util/
    string_helper.h:93-107) and parses the text back (std::stod), i.e. rounds
    to 15 decimal places.  That is k / 10^15 with k the integer nearest to the
    exact product v 10^15 (Dekker's error-free product decides the rounding)
    while |v| 10^15 < 2^53; larger magnitudes take the text route.""" 
    v = np.asarray(v, dtype=np.float64)
    p, e = _two_product(v, 1e15)  # v 10^15 = p + e exactly
    k = np.rint(p)
    r = p - k  # exact, |r| <= 1/2
    # the exact value k + r + e against the half-way points k +- 1/2: r -+ 1/2
    # is exact wherever it matters and a rounded sum keeps the sign of the
    # exact one (zero only when exact), so these tests are exact
    up = (r - 0.5) + e
    dn = (r + 0.5) + e
    k = np.where(up > 0, k + 1.0, np.where(dn < 0, k - 1.0, k))
    # exact ties round to the even neighbour, as printf does
    k = np.where((up == 0) & (np.fmod(k, 2.0) != 0), k + 1.0, k)
    k = np.where((dn == 0) & (np.fmod(k, 2.0) != 0), k - 1.0, k)
    q = k / 1e15  # correctly rounded: the double std::stod gives for the text
    big = np.abs(v) >= 8.0
    if big.any():
        q[big] = np.char.mod("%.15f", v[big]).astype(np.float64)
    return q


def _split(a):
    t = 134217729.0 * a  # 2^27 + 1 (Veltkamp)
    hi = t - (t - a)
    return hi, a - hi


def _two_product(a, b):
    """Dekker's error-free product: a b = p + e exactly (no overflow)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(np.float64(b))
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def write_vtp(path: str, points: np.ndarray, arrays: Sequence[Tuple[str, np.ndarray]], match_reference: bool = True) -> str:
    """Write `points` ((n, d) coordinates, d <= 3) and the named point arrays
    (each n values, written as Float64) to `path` (".vtp" appended if
    missing).  match_reference rounds the values as the reference's writer
    does (15 decimals), so the file is the reference's byte for byte in its
    arrays; False writes the full FP64 values.  Returns the file name."""
    if not path.endswith(".vtp"):
        path += ".vtp"
    pts = np.asarray(points, dtype=np.float64)
    n = pts.shape[0]
    xyz = np.zeros((n, 3), dtype=np.float32)
    xyz[:, : pts.shape[1]] = pts
    parts: List[str] = [
        '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
        "  <PolyData>\n",
        f'<Piece NumberOfPoints="{n}" NumberOfVerts="1" NumberOfLines="0" NumberOfStrips="0" NumberOfPolys="0" > \n',
        '<Points>\n<DataArray type="Float32" Name="Points" NumberOfComponents="3" format="binary"> \n',
        _b64(xyz.reshape(-1)),
        "\n        </DataArray>\n      </Points>\n",
        '      <Verts>\n        <DataArray type="Int64" Name="connectivity" format="binary"> \n',
        _b64(np.arange(n, dtype=np.int64)),
        "\n        </DataArray> \n",
        '        <DataArray type="Int64" Name="offsets" format="ascii"> \n',
        f"{n}\n        </DataArray> \n        </Verts> \n      <PointData> \n",
    ]
    for name, values in arrays:
        v = np.asarray(values, dtype=np.float64).reshape(-1)
        if match_reference:
            v = reference_rounding(v)
        if v.size != n:
            raise ValueError(f"array {name}: {v.size} values for {n} points")
        parts += [f'<DataArray type="Float64" Name="{name}" format="binary">\n', _b64(v), "\n        </DataArray> \n"]
    parts += ["      </PointData> \n", "    </Piece>\n", "  </PolyData>\n", "</VTKFile> \n"]
    with open(path, "w") as fh:
        fh.write("".join(parts))
    return path


def solution_arrays(ndim: int, rho: Optional[np.ndarray] = None, u: Optional[Sequence[np.ndarray]] = None,
                    phi: Optional[np.ndarray] = None) -> List[Tuple[str, np.ndarray]]:
    """The reference's output columns: the velocity components U, V[, W] then
    rho for Navier-Stokes; the potential V for Poisson."""
    if phi is not None:
        return [("V", phi)]
    return [(VEL_NAMES[d], u[d]) for d in range(ndim)] + [("rho", rho)]


def line_cells(centers: np.ndarray, half_length, a: Sequence[float], b: Sequence[float]) -> np.ndarray:
    """The cells a line probe samples (PostprocessCartesianFunctionLine::init,
    src/postprocess/postprocessing_cartesian.h:17-39): every cell whose centre
    lies within half a cell length of the line through a and b, ordered by
    coordinates.

    In 2D the distance is the reference's own: the absolute distance to the
    hyperplane through a and b (src/common/line.h, Eigen 3.3.91
    ``Hyperplane<double, 2>::Through``: unit normal (-d_y, d_x) / |d|, offset
    -a . n, distance |n . p + offset|), evaluated with the same operations in
    the same order, so cells at exactly half a cell length are decided alike.
    In 3D that construction is a plane, not a line; here the 3D distance is to
    the line itself.

    Order: x, then y, then z.  The reference sorts with a comparator that is a
    strict weak order only when the probe's cells increase in every
    coordinate together (an axis-parallel line through one row or column of
    centres, or a line of positive slope); for those lines the two orders
    agree, for the others the reference's order is unspecified."""
    c = np.asarray(centers, dtype=np.float64)
    ndim = c.shape[1]
    a = np.asarray(a, dtype=np.float64)[:ndim]
    b = np.asarray(b, dtype=np.float64)[:ndim]
    d = b - a
    if ndim == 2:
        n = np.array([-d[1], d[0]])
        z = n[0] * n[0] + n[1] * n[1]
        if z > 0:
            n = n / np.sqrt(z)
        off = -(a[0] * n[0] + a[1] * n[1])
        dist = np.abs((n[0] * c[:, 0] + n[1] * c[:, 1]) + off)
    else:
        t = d / np.linalg.norm(d)
        r = c - a
        dist = np.linalg.norm(r - np.outer(r @ t, t), axis=1)
    cells = np.nonzero(np.asarray(half_length) >= dist)[0]
    keys = tuple(c[cells, k] for k in reversed(range(ndim)))  # lexsort: last key first
    return cells[np.lexsort(keys)]


def box_line_cells(shape, spacing: float, a: Sequence[float], b: Sequence[float]) -> np.ndarray:
    """line_cells for a dense box of (nx, ny[, nz]) cells of edge `spacing`
    with centres at (i + 1/2) spacing, without visiting every cell: along the
    line's dominant axis each layer of cells holds the line's crossing point,
    and only the cells within two cells of it are tested.  Returns flat cell
    indices x + nx (y + ny z) in probe order."""
    nx, ny, nz = (tuple(shape) + (1, 1))[:3]
    dims = (nx, ny, nz)
    ndim = 2 if nz == 1 else 3
    a = np.asarray(a, dtype=np.float64)[:ndim]
    b = np.asarray(b, dtype=np.float64)[:ndim]
    d = b - a
    h = float(spacing)
    if not np.any(d):
        cand = np.arange(nx * ny * nz)
    else:
        k = int(np.argmax(np.abs(d)))
        others = [j for j in range(ndim) if j != k]
        mesh = np.meshgrid(np.arange(dims[k]), *([np.arange(-2, 4)] * len(others)), indexing="ij")
        t = ((mesh[0] + 0.5) * h - a[k]) / d[k]  # the line's parameter in the layer's mid-plane
        idx = [None] * ndim
        idx[k] = mesh[0]
        for n, j in enumerate(others):
            idx[j] = np.floor((a[j] + t * d[j]) / h - 0.5).astype(np.int64) + mesh[1 + n]
        ok = np.ones(mesh[0].shape, dtype=bool)
        for j in range(ndim):
            ok &= (idx[j] >= 0) & (idx[j] < dims[j])
        flat = idx[0] + nx * (idx[1] + (ny * idx[2] if ndim == 3 else 0))
        cand = np.unique(flat[ok])
    x = cand % nx
    y = (cand // nx) % ny
    z = cand // (nx * ny)
    centers = (np.stack([x, y, z][:ndim], axis=1) + 0.5) * h
    return cand[line_cells(centers, 0.5 * h, a, b)]


def _g15(v: float) -> str:
    """A coordinate as the reference's stream prints it (precision 15, default
    float format: printf's %.15g)."""
    return "%.15g" % v


def write_line_csv(path: str, coords: np.ndarray, values: np.ndarray, name: str = "u") -> str:
    """The reference's line probe file (ASCII::writePointsCSV,
    src/common/IO.h:37-88, called from src/postprocess/postprocessing.h:98-115):
    a header of the coordinate names and the value column, then one row per
    probe cell with its centre (precision 15) and the value printed with
    std::fixed and 15 decimals (toStringVector).  `path` gets ".csv" appended
    if missing (the reference always writes "line.csv")."""
    if not path.endswith(".csv"):
        path += ".csv"
    coords = np.asarray(coords, dtype=np.float64)
    ndim = coords.shape[1]
    rows = [",".join(("x", "y", "z")[:ndim]) + "," + name + "\n"]
    for p, v in zip(coords, np.asarray(values, dtype=np.float64)):
        rows.append(",".join(_g15(float(x)) for x in p) + "," + ("%.15f" % float(v)) + "\n")
    with open(path, "w") as fh:
        fh.write("".join(rows))
    return path


def read_vtp(path: str):
    """Parse a file of this layout (or the reference's): (points (n, 3),
    {name: array}).  For tests and post-processing."""
    import re

    text = open(path).read()
    out = {}
    points = None
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)"[^>]*format="(\w+)">\s*(.*?)\s*</DataArray>', text, re.S):
        typ, name, fmt, body = m.groups()
        if fmt != "binary":
            out[name] = np.array([float(x) for x in body.split()])
            continue
        raw = base64.b64decode(body)
        nbytes = int(np.frombuffer(raw[:8], np.uint64)[0])
        dt = {"Float32": np.float32, "Float64": np.float64, "Int64": np.int64, "Int32": np.int32}[typ]
        arr = np.frombuffer(raw[8:8 + nbytes], dt).copy()
        if name == "Points":
            points = arr.reshape(-1, 3)
        else:
            out[name] = arr
    return points, out
