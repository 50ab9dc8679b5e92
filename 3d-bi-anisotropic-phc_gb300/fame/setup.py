"""Host-side problem setup: lattice, Bloch angles, vertex rasterisation of the
inclusions, constitutive tensors and band paths.

These mirror the reference's MATLAB settings scripts (they run once per
geometry on the host there too); the per-k numerical work happens in the
CUDA library.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import check, load

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

# FCC high-symmetry points in reciprocal-lattice coordinates
# (InputData/BS_Gyroid/Physical_settings_woodpile.m:143-148)
FCC_POINTS = {
    "G": (0.0, 0.0, 0.0),
    "K": (3 / 8, 3 / 8, 3 / 4),
    "L": (0.5, 0.5, 0.5),
    "U": (5 / 8, 1 / 4, 5 / 8),
    "W": (0.5, 1 / 4, 3 / 4),
    "X": (0.5, 0.0, 0.5),
}


def fcc_lattice(a: float = 1.0) -> np.ndarray:
    """Primitive FCC vectors as columns, (a/2)(0,1,1), (1,0,1), (1,1,0)
    (Physical_settings_woodpile.m:7)."""
    return 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])


def reciprocal(A: np.ndarray) -> np.ndarray:
    """2*pi*inv(A') (Physical_settings_woodpile.m:9)."""
    return 2.0 * math.pi * np.linalg.inv(A.T)


def fcc_point(name: str, A: np.ndarray | None = None) -> np.ndarray:
    A = fcc_lattice() if A is None else A
    return reciprocal(A) @ np.asarray(FCC_POINTS[name])


def bloch_angles(wave_vec, A: np.ndarray | None = None) -> np.ndarray:
    """theta_d = k . a_d, with a zero wave vector first shifted by 1e-4 per
    component (band_structure_woodpile_Lanczos_n60_gamma0p2.m:50-56)."""
    A = fcc_lattice() if A is None else A
    k = np.asarray(wave_vec, dtype=np.float64)
    if not np.any(k):
        k = k + 1e-4
    return A.T @ k


def band_path(labels=("G", "X", "U", "|", "K", "G", "L", "W", "X"), npts: int = 40,
              A: np.ndarray | None = None) -> np.ndarray:
    """Wave vectors along a high-symmetry path with `npts` samples in total.

    '|' starts a new piece (a jump between equivalent points).  Every piece
    includes both end points; the intervals are shared among the segments in
    proportion to their lengths (largest remainder, at least one each).
    Returns an (npts, 3) array.
    """
    A = fcc_lattice() if A is None else A
    pieces, cur = [], []
    for lab in labels:
        if lab == "|":
            if cur:
                pieces.append(cur)
            cur = []
        else:
            cur.append(lab)
    if cur:
        pieces.append(cur)
    segs = []
    for pc in pieces:
        for a, b in zip(pc[:-1], pc[1:]):
            segs.append((fcc_point(a, A), fcc_point(b, A)))
    n_int = npts - len(pieces)
    if n_int < len(segs):
        raise ValueError("too few points for the path")
    lens = np.array([np.linalg.norm(b - a) for a, b in segs])
    share = lens / lens.sum() * n_int
    alloc = np.maximum(1, np.floor(share).astype(int))
    while alloc.sum() < n_int:
        alloc[np.argmax(share - alloc)] += 1
    while alloc.sum() > n_int:
        cand = np.where(alloc > 1)[0]
        alloc[cand[np.argmin((share - alloc)[cand])]] -= 1
    out, si = [], 0
    for pc in pieces:
        for s in range(len(pc) - 1):
            a, b = segs[si]
            m = alloc[si]
            start = 0 if s == 0 else 1
            for t in range(start, m + 1):
                out.append(a + (b - a) * (t / m))
            si += 1
    return np.array(out)


def reference_path(path_string: str = "XULGXWK", part_num: int = 10, A: np.ndarray | None = None) -> np.ndarray:
    """The reference's own k-path construction: linspace of `part_num` points per
    segment, joints not repeated (Physical_settings_woodpile.m:165-182)."""
    A = fcc_lattice() if A is None else A
    n = len(path_string)
    out = []
    for i in range(n - 1):
        if path_string[i] == "|" or path_string[i + 1] == "|":
            continue
        a, b = fcc_point(path_string[i], A), fcc_point(path_string[i + 1], A)
        sub = [a + (b - a) * t for t in np.linspace(0.0, 1.0, part_num)]
        last = i == n - 2 or path_string[i + 2] == "|"
        out.extend(sub if last else sub[:-1])
    return np.array(out)


def vertex_positions(n: int, A: np.ndarray | None = None) -> np.ndarray:
    """Cartesian positions of the n^3 grid vertices, x fastest: lattice
    coefficients (i-1)/n (Public/Grid_Generate_Mult_Point.m:7-17) times A'."""
    A = fcc_lattice() if A is None else A
    c = np.arange(n) / n
    c3, c2, c1 = np.meshgrid(c, c, c, indexing="ij")
    coef = np.stack([c1.ravel(), c2.ravel(), c3.ravel()], axis=1)
    return coef @ A.T


def woodpile_inside(P: np.ndarray, width: float, a: float = 1.0) -> np.ndarray:
    """Woodpile rod test of Public/woodpile_isofun.m:4-11: four layers of
    height a/4 with rods along the x = +-y diagonals (t1 = y - x, t2 = y + x),
    half-width sqrt(2)/2*width in t, same-orientation layers offset by a/2."""
    z = P[:, 2]
    t1 = P[:, 1] - P[:, 0]
    t2 = P[:, 1] + P[:, 0]
    h = math.sqrt(2.0) / 2.0 * width

    def band(t, c):
        return (t >= c - h) & (t <= c + h)

    l0 = (z >= 0) & (z < a / 4) & ((t1 >= a - h) | (t1 <= -(a - h)) | band(t1, 0.0))
    l1 = (z >= a / 4) & (z < a / 2) & (band(t2, 1.5 * a) | band(t2, 0.5 * a))
    l2 = (z >= a / 2) & (z < 3 * a / 4) & (band(t1, -0.5 * a) | band(t1, 0.5 * a))
    l3 = (z >= 3 * a / 4) & (z <= a) & ((t2 >= 2 * a - h) | (t2 <= h) | band(t2, a))
    return l0 | l1 | l2 | l3


def sphere_inside(P: np.ndarray, radius: float, A: np.ndarray | None = None,
                  center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Sphere of `radius` at `center` with all periodic images of the lattice."""
    A = fcc_lattice() if A is None else A
    best = np.full(P.shape[0], np.inf)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                c = np.asarray(center) + A @ np.array([i, j, k], dtype=np.float64)
                best = np.minimum(best, np.linalg.norm(P - c, axis=1))
    return best < radius


def tetra_inside(P: np.ndarray, edge: float, A: np.ndarray | None = None,
                 center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Regular tetrahedron of edge length `edge` centred at `center` (vertices
    along (1,1,1), (1,-1,-1), (-1,1,-1), (-1,-1,1)), with all periodic images.
    A point is inside when, for each face, it lies on the same side as the
    opposite vertex (the four half-space tests of
    subroutines/Material_Locate_Isofunction.m:38-90; within 1e-8 of a face
    counts as inside)."""
    A = fcc_lattice() if A is None else A
    s = edge / (2.0 * math.sqrt(2.0))
    base = s * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64)
    inside = np.zeros(P.shape[0], dtype=bool)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                verts = base + np.asarray(center) + A @ np.array([i, j, k], dtype=np.float64)
                ok = np.ones(P.shape[0], dtype=bool)
                for f in range(4):
                    a, b, c = [verts[t] for t in range(4) if t != f]
                    nrm = np.cross(b - a, c - a)
                    dp = (a - P) @ nrm
                    dq = float(np.dot(a - verts[f], nrm))
                    ok &= (np.abs(dp) < 1e-8) | (dp * dq > 0)
                inside |= ok
    return inside


def constitutive(eps, mu, xi, zeta) -> np.ndarray:
    """The 6x6 block [eps xi; zeta mu] (complex)."""
    return np.block([[np.asarray(eps), np.asarray(xi)], [np.asarray(zeta), np.asarray(mu)]]).astype(np.complex128)


def bi_isotropic(eps: float, gamma: float, mu: float = 1.0) -> np.ndarray:
    """eps*I3, mu*I3, xi = +i*gamma*I3, zeta = -i*gamma*I3."""
    I3 = np.eye(3)
    return constitutive(eps * I3, mu * I3, 1j * gamma * I3, -1j * gamma * I3)


def covariant_blocks(c6: np.ndarray, A: np.ndarray | None = None) -> np.ndarray:
    """27 complex (N | M | J, row-major 3x3 each) of one phase through the
    library's fame_material_blocks (6x6 inverse, A'XA)."""
    A = fcc_lattice() if A is None else A
    lib = load()
    c6 = np.ascontiguousarray(np.asarray(c6, dtype=np.complex128).reshape(6, 6))
    lat = np.ascontiguousarray(A, dtype=np.float64)
    out = np.zeros(54, dtype=np.float64)
    pd = C.POINTER(C.c_double)
    check(lib.fame_material_blocks(c6.view(np.float64).ctypes.data_as(pd), lat.ctypes.data_as(pd),
                                   out.ctypes.data_as(pd)), None, "fame_material_blocks")
    return out.view(np.complex128).copy()


SHAPES = {"woodpile": 0, "sphere": 1, "tetra": 2, "tetrahedron": 2, "tri": 2}


def rasterize(n: int, shape: str, size: float, A: np.ndarray | None = None, center=(0.0, 0.0, 0.0),
              a: float = 1.0, phase_id: int = 1, phase=None, device: bool = False):
    """Phase id of every vertex of the n^3 grid from the device rasteriser
    (fame_rasterize): `phase_id` inside the shape, 0 outside, or the id
    already in `phase` when it is given (several inclusions).

    shape 'woodpile': rod width `size`, lattice constant `a`
    (Public/woodpile_isofun.m); 'sphere': radius `size` about `center`
    (Physical_settings_sphere.m:18); 'tetra': regular tetrahedron of edge
    `size` about `center` (Material_Locate_Isofunction.m:135-148).  Sphere and
    tetrahedron include their 27 periodic images.  Returns a uint8 numpy array,
    or a CUDA uint8 tensor when `device` (or when `phase` is one)."""
    A = fcc_lattice() if A is None else A
    if shape not in SHAPES:
        raise ValueError(f"unknown shape {shape!r}: one of {sorted(SHAPES)}")
    kind = SHAPES[shape]
    lib = load()
    if kind == 0:
        params = np.array([size, a], dtype=np.float64)
    else:
        params = np.array([size, *np.asarray(center, dtype=np.float64)], dtype=np.float64)
    lat = np.ascontiguousarray(A, dtype=np.float64)
    pd = C.POINTER(C.c_double)
    Nq = n ** 3
    flags = 2 if phase is not None else 0
    on_device = device or (torch is not None and isinstance(phase, torch.Tensor))
    if on_device:
        if phase is None:
            out = torch.empty(Nq, dtype=torch.uint8, device="cuda")
        else:
            out = phase
            if out.dtype != torch.uint8 or not out.is_cuda or not out.is_contiguous() or out.numel() != Nq:
                raise ValueError("phase must be a contiguous CUDA uint8 tensor of n^3 elements")
        ptr = C.c_void_p(out.data_ptr())
    else:
        if phase is None:
            out = np.zeros(Nq, dtype=np.uint8)
        else:
            out = np.ascontiguousarray(phase, dtype=np.uint8).reshape(-1)
            if out.size != Nq:
                raise ValueError("phase must hold n^3 ids")
        flags |= 1
        ptr = C.c_void_p(out.ctypes.data)
    check(lib.fame_rasterize(int(n), lat.ctypes.data_as(pd), kind, params.ctypes.data_as(pd), int(phase_id), ptr,
                             flags), None, "fame_rasterize")
    return out
