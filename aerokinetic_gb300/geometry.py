"""Section geometry: closed polygons, multi-element sections and NACA 4-digit shapes.

Host-side mirror of the reference's case layer (src/aerokinetic/geometry.py):
the same classes, argument meanings, validation errors and floating-point
arithmetic, so that solid flags, cut links and Bouzidi fractions derived from
these polygons agree bit for bit with the reference.  The per-cell and per-link
work on a lattice (point-in-polygon flags, link fractions) runs on the GPU in
``csrc/ak_geometry.cuh``; the numpy methods here serve small host queries.
"""
from dataclasses import dataclass
from fractions import Fraction
from pathlib import Path

import numpy as np


def cross2(a, b):
    """z component of the 2-D cross product, a_x b_y - a_y b_x, rounded twice."""
    return a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]


def _fused(a, b, c):
    """Correctly rounded a*b + c (one rounding), in exact rational arithmetic."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _rotate(points, rotation):
    """points @ rotation.T with the rounding of the reference's recorded runs.

    The reference evaluates ``xy @ rotation.T`` (geometry.py:143-148) through
    x86-64 OpenBLAS, which rounds x*r0 and then fuses y*r1 into it.  Reproducing
    that rounding explicitly keeps the rotated polygon, and therefore every
    flag and link fraction, identical on any host.
    """
    out = np.empty_like(points)
    for i, (x, y) in enumerate(points):
        for j in range(2):
            out[i, j] = _fused(y, rotation[j, 1], x * rotation[j, 0])
    return out


def segments_intersect(a, b, c, d):
    """Closed-segment intersection test with a relative tolerance (geometry.py:112-123)."""
    ab, cd = b - a, d - c
    den = cross2(ab, cd)
    tol = 1e-12 * max(np.linalg.norm(ab) * np.linalg.norm(cd), 1e-30)
    if abs(den) <= tol:
        if abs(cross2(c - a, ab)) > tol:
            return False
        axis = int(np.argmax(abs(ab)))
        lo = max(min(a[axis], b[axis]), min(c[axis], d[axis]))
        hi = min(max(a[axis], b[axis]), max(c[axis], d[axis]))
        return lo <= hi + 1e-12
    t = cross2(c - a, cd) / den
    u = cross2(c - a, ab) / den
    return -1e-12 <= t <= 1 + 1e-12 and -1e-12 <= u <= 1 + 1e-12


def _pairs_intersect(a, b, c, d):
    """segments_intersect for arrays of segment pairs (a, b) x (c, d), (k, 2) each:
    the same tests and tolerances, evaluated with numpy."""
    ab, cd, ca = b - a, d - c, c - a
    den = cross2(ab, cd)
    norm_ab = np.sqrt(np.einsum("ij,ij->i", ab, ab))
    norm_cd = np.sqrt(np.einsum("ij,ij->i", cd, cd))
    tol = 1e-12 * np.maximum(norm_ab * norm_cd, 1e-30)
    parallel = np.abs(den) <= tol
    # parallel pairs: collinear and overlapping along the first edge's main axis
    axis = np.argmax(np.abs(ab), axis=1)
    rows = np.arange(len(a))
    a_ax, b_ax, c_ax, d_ax = a[rows, axis], b[rows, axis], c[rows, axis], d[rows, axis]
    lo = np.maximum(np.minimum(a_ax, b_ax), np.minimum(c_ax, d_ax))
    hi = np.minimum(np.maximum(a_ax, b_ax), np.maximum(c_ax, d_ax))
    collinear = (np.abs(cross2(ca, ab)) <= tol) & (lo <= hi + 1e-12)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = cross2(ca, cd) / den
        u = cross2(ca, ab) / den
    crossing = (-1e-12 <= t) & (t <= 1 + 1e-12) & (-1e-12 <= u) & (u <= 1 + 1e-12)
    return np.where(parallel, collinear, crossing)


def _any_intersection(starts1, ends1, starts2, ends2, i, j, chunk=1 << 16):
    """Whether edge i of the first list meets edge j of the second for any
    listed pair (i, j), in blocks of pairs."""
    for k in range(0, len(i), chunk):
        ii, jj = i[k:k + chunk], j[k:k + chunk]
        if np.any(_pairs_intersect(starts1[ii], ends1[ii], starts2[jj], ends2[jj])):
            return True
    return False


def _any_segments_intersect(p, nxt):
    """segments_intersect over every pair of non-adjacent edges (i, j), j >= i + 2,
    of one closed polygon, except the closing pair (0, n - 1)."""
    n = len(p)
    i, j = np.triu_indices(n, k=2)
    keep = ~((i == 0) & (j == n - 1))
    return _any_intersection(p, nxt, p, nxt, i[keep], j[keep])


@dataclass(frozen=True)
class Contour:
    """Closed polygon in a common frame (geometry.py:10-85); any length scale."""
    xy: np.ndarray
    name: str = "element"

    def __post_init__(self):
        p = np.array(self.xy, dtype=float, copy=True)
        if p.ndim != 2 or p.shape[1] != 2 or len(p) < 3 or not np.isfinite(p).all():
            raise ValueError("A contour requires at least three finite (x,y) points")
        keep = np.ones(len(p), dtype=bool)
        keep[1:] = np.linalg.norm(np.diff(p, axis=0), axis=1) > 1e-14
        p = p[keep]
        if len(p) > 1 and np.allclose(p[0], p[-1], rtol=0, atol=1e-14):
            p = p[:-1]
        if len(p) < 3:
            raise ValueError("Degenerate contour")
        nxt = np.roll(p, -1, axis=0)
        if abs(np.sum(cross2(p, nxt))) / 2 <= 1e-12 * np.ptp(p, axis=0).max() ** 2:
            raise ValueError("Contour has zero enclosed area")
        if _any_segments_intersect(p, nxt):
            raise ValueError(f"Self-intersection in contour {self.name}")
        p.setflags(write=False)
        object.__setattr__(self, "xy", p)

    @classmethod
    def from_aero2d(cls, airfoil):
        return cls(np.column_stack((airfoil.x, airfoil.y)), getattr(airfoil, "name", "element"))

    @classmethod
    def from_dat(cls, path):
        """One Selig-style polygon: every line holding exactly two numbers is a vertex."""
        rows = []
        for line in Path(path).read_text(encoding="utf-8-sig").splitlines():
            parts = line.replace(",", " ").split()
            if len(parts) != 2:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1])))
            except ValueError:
                continue
        return cls(np.asarray(rows), Path(path).stem)

    def edges(self):
        return self.xy, np.roll(self.xy, -1, axis=0)

    def contains(self, x, y):
        """Even-odd crossing test of points against every non-horizontal edge."""
        x, y = np.broadcast_arrays(x, y)
        inside = np.zeros(x.shape, dtype=bool)
        for a, b in zip(*self.edges()):
            if b[1] == a[1]:
                continue
            straddles = (a[1] > y) != (b[1] > y)
            crossing = (b[0] - a[0]) * (y - a[1]) / (b[1] - a[1]) + a[0]
            inside ^= straddles & (x < crossing)
        return inside

    def link_fraction(self, points, offsets):
        """Smallest q in [0, 1] with points + q*offsets on the polygon, clipped to [1e-10, 1]."""
        points = np.asarray(points)
        offsets = np.asarray(offsets)
        q = np.full(len(points), np.inf)
        for a, b in zip(*self.edges()):
            edge = b - a
            den = cross2(offsets, edge)
            valid = abs(den) > 1e-14
            rel = a - points
            t = np.divide(cross2(rel, edge), den, out=np.full_like(q, np.inf), where=valid)
            v = np.divide(cross2(rel, offsets), den, out=np.full_like(q, np.inf), where=valid)
            hit = valid & (t >= -1e-10) & (t <= 1 + 1e-10) & (v >= -1e-10) & (v <= 1 + 1e-10)
            q = np.minimum(q, np.where(hit, t, np.inf))
        if not np.isfinite(q).all():
            raise ValueError("A fluid-to-solid link has no geometric intersection")
        return np.clip(q, 1e-10, 1.0)


@dataclass(frozen=True)
class Section:
    """Elements, reference chord and moment reference (geometry.py:126-148)."""
    elements: tuple
    chord: float | None = None
    moment_reference: tuple | None = None

    def __post_init__(self):
        elements = tuple(self.elements)
        if not elements:
            raise ValueError("At least one contour is required")
        if not all(isinstance(e, Contour) for e in elements):
            raise TypeError("Use Contour.from_aero2d for existing Airfoil objects")
        object.__setattr__(self, "elements", elements)
        allp = np.concatenate([e.xy for e in elements])
        le = allp[np.argmin(allp[:, 0])]
        te = allp[np.isclose(allp[:, 0], allp[:, 0].max(), rtol=0, atol=1e-12)].mean(axis=0)
        chord = float(np.linalg.norm(te - le)) if self.chord is None else float(self.chord)
        if not np.isfinite(chord) or chord <= 0:
            raise ValueError("Reference chord must be positive")
        if self.moment_reference is None:
            ref = le + 0.25 * (te - le)
        else:
            ref = np.asarray(self.moment_reference, dtype=float)
        if np.shape(ref) != (2,) or not np.isfinite(ref).all():
            raise ValueError("Moment reference requires two finite coordinates")
        object.__setattr__(self, "chord", chord)
        object.__setattr__(self, "moment_reference", tuple(ref))
        for i, e in enumerate(elements):
            for f in elements[i + 1:]:
                touching = bool(e.contains(*f.xy[0]) or f.contains(*e.xy[0]))
                if not touching:
                    (a, b), (c, d) = e.edges(), f.edges()
                    i, j = np.meshgrid(np.arange(len(a)), np.arange(len(c)), indexing="ij")
                    touching = _any_intersection(a, b, c, d, i.ravel(), j.ravel())
                if touching:
                    raise ValueError(f"Elements touch or overlap: {e.name}, {f.name}")

    @classmethod
    def from_aero2d(cls, airfoils, **kwargs):
        if hasattr(airfoils, "x"):
            airfoils = [airfoils]
        return cls(tuple(Contour.from_aero2d(a) for a in airfoils), **kwargs)

    def rotation(self, alpha_deg):
        angle = -np.deg2rad(alpha_deg)
        return np.array([[np.cos(angle), -np.sin(angle)], [np.sin(angle), np.cos(angle)]])

    def normalized(self, alpha_deg):
        """Chord-scaled contours about the moment reference; positive alpha raises the nose.
        The result for an angle is computed once per section (the exact rotation
        and the contours' own checks dominate a case's host-side set-up) and
        shared by later calls; its contours are not to be modified."""
        cache = self.__dict__.setdefault("_normalized", {})
        key = float(alpha_deg)
        if key not in cache:
            rotation = self.rotation(alpha_deg)
            contours = tuple(Contour(_rotate((e.xy - self.moment_reference) / self.chord, rotation), e.name)
                             for e in self.elements)
            for c in contours:
                c.xy.flags.writeable = False
            cache[key] = contours
        return cache[key]


def naca0012(n_side=161, closed_te=False):
    return naca4("0012", n_side, closed_te)


def naca4(code="0012", n_side=161, closed_te=False):
    """NACA 4-digit section of unit chord with cosine spacing (geometry.py:155-185)."""
    code = str(code).strip()
    if len(code) != 4 or not code.isascii() or not code.isdigit():
        raise ValueError("NACA code must contain four digits, e.g. 0012 or 2412")
    m, p, thickness = int(code[0]) / 100, int(code[1]) / 10, int(code[2:]) / 100
    return naca4_parametric(m, p, thickness, n_side, closed_te, f"NACA{code}")


def naca4_parametric(m, p, thickness, n_side=161, closed_te=False, name=None):
    """The 4-digit formula for real-valued camber m, camber position p and thickness."""
    if thickness <= 0 or (m > 0 and p == 0):
        raise ValueError("NACA thickness must be positive; cambered profiles require a nonzero second digit")
    if not isinstance(n_side, int):
        raise ValueError("n_side must be an integer")
    if n_side < 12:
        raise ValueError("Use at least 12 points per side")
    x = (1 - np.cos(np.linspace(0, np.pi, n_side))) / 2
    last = -0.1036 if closed_te else -0.1015
    y = 5 * thickness * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x**2 + 0.2843 * x**3 + last * x**4)
    camber, slope = np.zeros_like(x), np.zeros_like(x)
    if m > 0:
        fore = x < p
        aft = ~fore
        camber[fore] = m / p**2 * (2 * p * x[fore] - x[fore]**2)
        slope[fore] = 2 * m / p**2 * (p - x[fore])
        camber[aft] = m / (1 - p)**2 * (1 - 2 * p + 2 * p * x[aft] - x[aft]**2)
        slope[aft] = 2 * m / (1 - p)**2 * (p - x[aft])
    angle = np.arctan(slope)
    upper = np.column_stack((x - y * np.sin(angle), camber + y * np.cos(angle)))
    lower = np.column_stack((x + y * np.sin(angle), camber - y * np.cos(angle)))
    return Contour(np.concatenate((upper[::-1], lower[1:])), name or f"NACA{m:g}-{p:g}-{thickness:g}")
