"""CPU oracle for the uniform D3Q27 cumulant step: numpy set-up around ak_oracle.c.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the product.  It restates, in the
reference's own structure (padded arrays with one ghost layer, boundary
objects applied in installation order, then "stream_collide" into a second
array and a swap), the uniform solver of the reference:

  * solid flags and boundary masks   solver.py:93-98, 124-155; farfield.py:209-224
  * cut links and Bouzidi fractions  solver.py:100-122; geometry.py:58-85
  * characteristic farfield set-up    farfield.py:56-114
  * initial state                     solver.py:157-202
  * one step and its loads            solver.py:204-279
  * validity diagnostics              solver.py:281-297

The reference's own lattice code (lbmpy 1.4) is not available; ak_oracle.c
restates its published algorithms.  Parity of this oracle is pinned against
the reference's recorded outputs: the acoustic probe records of
docs/verification_stage1_20261106/acoustics/ (UBB, ExtrapolationOutflow), the
272-step known answer of tools/profile_stage1.py, and the Cl/Cd/Cm histories
of docs/verification_*/ (tests/test_oracle_golden.py).
"""
import ctypes
import itertools
import math
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "_build" / "libak_oracle.so"
SOURCE = HERE / "ak_oracle.c"

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
_D = ctypes.c_double
_SIGNATURES = {
    "ako_stencil": [_P, _P, _P],
    "ako_collide_cells": [_P, _L, _D, _D],
    "ako_collide_cells_sgs": [_P, _L, _D, _D, _D],
    "ako_stream_collide": [_P, _P, _I, _I, _I, _D, _D, _I],
    "ako_stream_collide_sgs": [_P, _P, _I, _I, _I, _D, _D, _D, _I],
    "ako_collide": [_P, _I, _I, _I, _D, _D, _I],
    "ako_stream": [_P, _P, _I, _I, _I],
    "ako_sync_periodic": [_P, _I, _I, _I, _I, _I, _I],
    "ako_equilibrium": [_P, _P, _P, _L],
    "ako_macros": [_P, _P, _P, _L],
    "ako_bouzidi": [_P, _I, _I, _I, _L, _P, _P],
    "ako_ubb": [_P, _I, _I, _I, _L, _P, _P],
    "ako_outflow": [_P, _I, _I, _I, _L, _P, _P, _P],
    "ako_farfield": [_P, _I, _I, _I, _L, _P, _P, _P, _D, _I, _P, _P, _P, _P, _P, _P, _P],
    "ako_loads": [_P, _I, _I, _I, _L, _P, _D, _D, _P],
}


def build(force=False):
    """Compile ak_oracle.c with the host C compiler (OpenMP, IEEE doubles)."""
    if LIBRARY.exists() and not force and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIBRARY
    LIBRARY.parent.mkdir(exist_ok=True)
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    cmd = f"gcc -O2 -fopenmp -fPIC -shared -o {tmp} {SOURCE} -lm"
    if os.system(cmd) != 0:
        raise RuntimeError(f"oracle build failed: {cmd}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


_lib = None


def lib():
    global _lib
    if _lib is None:
        handle = ctypes.CDLL(str(build()))
        for name, argtypes in _SIGNATURES.items():
            getattr(handle, name).argtypes = argtypes
            getattr(handle, name).restype = None
        _lib = handle
    return _lib


def _p(a):
    return a.ctypes.data_as(_P)


def stencil():
    c = np.zeros((27, 3), np.int32)
    w = np.zeros(27)
    inv = np.zeros(27, np.int32)
    lib().ako_stencil(_p(c), _p(w), _p(inv))
    return c.astype(np.int64), w, inv.astype(np.int64)


C, WEIGHTS, INVERSE = None, None, None


def _tables():
    global C, WEIGHTS, INVERSE
    if C is None:
        C, WEIGHTS, INVERSE = stencil()
    return C, WEIGHTS, INVERSE


def equilibrium(rho, u):
    """Zero-centred tensor-product equilibrium for arrays rho (...) and u (..., 3)."""
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    g = np.empty(rho.shape + (27,))
    lib().ako_equilibrium(_p(g), _p(rho), _p(u), rho.size)
    return g


def macros(g):
    g = np.ascontiguousarray(g, dtype=np.float64)
    rho = np.empty(g.shape[:-1])
    u = np.empty(g.shape[:-1] + (3,))
    lib().ako_macros(_p(g), _p(rho), _p(u), rho.size)
    return rho, u


def collide(g, omega_s, omega_b=1.0, smagorinsky=0.0):
    """Cumulant collision of independent cells (...,27), returning a new array;
    smagorinsky > 0 (the constant C) uses each cell's Smagorinsky shear rate."""
    out = np.array(g, dtype=np.float64, order="C", copy=True)
    if smagorinsky > 0:
        lib().ako_collide_cells_sgs(_p(out), out.size // 27, omega_s, omega_b, sgs_c18(smagorinsky))
    else:
        lib().ako_collide_cells(_p(out), out.size // 27, omega_s, omega_b)
    return out


def sgs_c18(constant):
    """18 C^2 of the Smagorinsky rate, 0 for molecular viscosity."""
    return 18.0 * float(constant) ** 2 if constant else 0.0


# ---------------------------------------------------------------- geometry
def contains(xy, x, y):
    """Even-odd ray test of a polygon (geometry.py:58-68), same arithmetic."""
    x, y = np.broadcast_arrays(x, y)
    inside = np.zeros(x.shape, dtype=bool)
    nxt = np.roll(xy, -1, axis=0)
    for a, b in zip(xy, nxt):
        if b[1] == a[1]:
            continue
        inside ^= ((a[1] > y) != (b[1] > y)) & (x < (b[0] - a[0]) * (y - a[1]) / (b[1] - a[1]) + a[0])
    return inside


def _cross(a, b):
    return a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]


def link_fraction(xy, points, offsets):
    """First polygon crossing p + q e (geometry.py:70-85), same arithmetic."""
    q = np.full(len(points), np.inf)
    for a, b in zip(xy, np.roll(xy, -1, axis=0)):
        edge = b - a
        den = _cross(offsets, edge)
        ok = abs(den) > 1e-14
        t = np.divide(_cross(a - points, edge), den, out=np.full_like(q, np.inf), where=ok)
        v = np.divide(_cross(a - points, offsets), den, out=np.full_like(q, np.inf), where=ok)
        hit = ok & (t >= -1e-10) & (t <= 1 + 1e-10) & (v >= -1e-10) & (v <= 1 + 1e-10)
        q = np.minimum(q, np.where(hit, t, np.inf))
    if not np.isfinite(q).all():
        raise ValueError("A fluid-to-solid link has no geometric intersection")
    return np.clip(q, 1e-10, 1.0)


# ---------------------------------------------------------------- lattice
class Boundary:
    """One boundary object: its links (x, y, z, d) in padded coordinates."""

    def __init__(self, kind, flag, **params):
        self.kind = kind
        self.flag = flag
        self.params = params
        self.links = np.zeros((0, 4), np.int32)
        self.ready = False


class Lattice:
    """Uniform lattice with one ghost layer, applied the reference's way."""

    def __init__(self, shape, periodic, omega_s, omega_b=1.0, threads=0):
        self.shape = tuple(int(v) for v in shape)
        nx, ny, nz = self.shape
        self.periodic = tuple(bool(p) for p in periodic)
        self.omega_s, self.omega_b = float(omega_s), float(omega_b)
        self.threads = int(threads)
        self.pdf = np.zeros((nx + 2, ny + 2, nz + 2, 27))
        self.tmp = np.zeros_like(self.pdf)
        self.flags = np.zeros((nx + 2, ny + 2, nz + 2), np.int16)
        self.boundaries = []
        self.steps = 0
        self.smagorinsky = 0.0  # Smagorinsky constant C of the bulk collision (0: molecular viscosity)

    def midpoints(self):
        nx, ny, nz = self.shape
        return np.meshgrid(np.arange(-1, nx + 1) + 0.5, np.arange(-1, ny + 1) + 0.5,
                           np.arange(-1, nz + 1) + 0.5, indexing="ij")

    def set_boundary(self, boundary, mask):
        """Flag every (ghost-inclusive) cell of mask; later boundaries replace earlier ones."""
        boundary.flag = len(self.boundaries) + 1
        self.flags[mask] = boundary.flag
        self.boundaries.append(boundary)
        return boundary

    def build_links(self):
        """Fluid interior cells linked to a boundary neighbour, per boundary."""
        c, _, _ = _tables()
        nx, ny, nz = self.shape
        inner = self.flags[1:-1, 1:-1, 1:-1]
        fluid = inner == 0
        for b in self.boundaries:
            rows = []
            for d in range(1, 27):
                e = c[d]
                nb = self.flags[1 + e[0]:nx + 1 + e[0], 1 + e[1]:ny + 1 + e[1], 1 + e[2]:nz + 1 + e[2]]
                hit = np.argwhere(fluid & (nb == b.flag))
                if len(hit):
                    rows.append(np.column_stack((hit + 1, np.full(len(hit), d))))
            b.links = (np.concatenate(rows) if rows else np.zeros((0, 4), np.int64)).astype(np.int32)
            b.links = np.ascontiguousarray(b.links)

    @property
    def fluid(self):
        return self.flags[1:-1, 1:-1, 1:-1] == 0

    def apply_boundaries(self):
        nx, ny, nz = self.shape
        L = lib()
        for b in self.boundaries:
            n = len(b.links)
            if n == 0:
                continue
            if not b.ready:
                _initialise_boundary(self, b)
                b.ready = True
            if b.kind == "bouzidi":
                L.ako_bouzidi(_p(self.pdf), nx, ny, nz, n, _p(b.links), _p(b.q))
            elif b.kind == "ubb":
                L.ako_ubb(_p(self.pdf), nx, ny, nz, n, _p(b.links), _p(b.velocity))
            elif b.kind == "outflow":
                L.ako_outflow(_p(self.pdf), nx, ny, nz, n, _p(b.links), _p(b.normal), _p(b.state))
            elif b.kind == "farfield":
                L.ako_farfield(_p(self.pdf), nx, ny, nz, n, _p(b.links), _p(b.normal), _p(b.velocity),
                               b.density, b.mode, _p(b.incoming), _p(b.derivative), _p(b.clock),
                               _p(b.edge), _p(b.wrap), _p(b.initial), _p(b.periodic_arr))
            else:
                raise ValueError(b.kind)

    def sync(self):
        nx, ny, nz = self.shape
        lib().ako_sync_periodic(_p(self.pdf), nx, ny, nz, *map(int, self.periodic))

    def stream_collide(self):
        nx, ny, nz = self.shape
        lib().ako_stream_collide_sgs(_p(self.pdf), _p(self.tmp), nx, ny, nz, self.omega_s, self.omega_b,
                                     sgs_c18(self.smagorinsky), self.threads)
        self.pdf, self.tmp = self.tmp, self.pdf

    def step(self, before_stream=None):
        self.sync()
        self.apply_boundaries()
        result = before_stream() if before_stream is not None else None
        self.stream_collide()
        self.steps += 1
        return result

    def interior(self):
        return self.pdf[1:-1, 1:-1, 1:-1]

    def set_equilibrium(self, rho, u):
        self.pdf[1:-1, 1:-1, 1:-1] = equilibrium(rho, u)

    def macros(self):
        return macros(self.interior())


def _initialise_boundary(lattice, b):
    """The reference's per-boundary init callbacks, run at the first application.

    Each boundary is initialised just before its own first application, after
    the boundaries installed before it have been applied in that step.  For
    the legacy farfield this lets the outflow's corner links read the ghost
    values the UBB just wrote; that order reproduces the reference's legacy
    history (legacy_down6) to 2e-13 over 960 steps, while initialising every
    boundary before the first application departs from it by 2e-3.
    """
    c, w, inv = _tables()
    if b.kind == "ubb":
        b.velocity = np.asarray(b.params["velocity"], dtype=np.float64)
    elif b.kind == "bouzidi":
        b.q = np.ascontiguousarray(b.params["fractions"](b.links), dtype=np.float64)
    elif b.kind == "outflow":
        # previous neighbour value: the population on x_b - n at the first
        # application; previous boundary value: the zero-centred equilibrium of
        # the boundary's initial density and velocity
        b.normal = np.asarray(b.params["normal"], dtype=np.int32)
        d = b.links[:, 3]
        cell = b.links[:, :3] + c[d] - b.normal
        neighbour = lattice.pdf[cell[:, 0], cell[:, 1], cell[:, 2], inv[d]]
        feq = equilibrium(np.array([b.params["density"]]), np.asarray([b.params["velocity"]]))[0]
        b.state = np.ascontiguousarray(np.column_stack((neighbour, feq[inv[d]])))
    elif b.kind == "farfield":
        _initialise_farfield(lattice, b)


def _initialise_farfield(lattice, b):
    """farfield.py:41-114: edge/wrap flags and the initial characteristic state."""
    c, _, _ = _tables()
    shape = np.array(lattice.shape)
    periodic = lattice.periodic
    normal = np.array(b.params["normal"], dtype=np.int64)
    velocity = np.array(b.params["velocity"], dtype=np.float64)
    density = float(b.params["density"])
    n = len(b.links)
    points = b.links[:, :3].astype(np.int64) - 1
    offsets = c[b.links[:, 3]]
    foot = points + offsets - normal
    edge = np.zeros((n, 3), np.int32)
    wrap = np.zeros((n, 3), np.int32)
    for a in range(3):
        if not periodic[a]:
            assert np.all((foot[:, a] >= 0) & (foot[:, a] < shape[a]))
            edge[foot[:, a] == 0, a] = -1
            edge[foot[:, a] == shape[a] - 1, a] = 1
        else:
            wrap[foot[:, a] < 0, a] = shape[a]
            wrap[foot[:, a] >= shape[a], a] = -shape[a]
            foot[:, a] %= shape[a]
    evolve = float(normal @ velocity) >= 0 and bool(np.any(velocity != 0))
    glancing = evolve and float(normal @ velocity) == 0
    b.mode = 2 if glancing else (1 if evolve else 0)
    b.normal = normal.astype(np.int32)
    b.velocity = velocity
    b.density = density
    b.edge = np.ascontiguousarray(edge)
    b.wrap = np.ascontiguousarray(wrap)
    b.periodic_arr = np.array(periodic, dtype=np.int32)
    b.incoming = np.zeros(n)
    b.derivative = np.zeros(n)
    b.clock = np.zeros(n, np.int64)
    b.initial = np.zeros(1)
    nh = normal.astype(float) / np.linalg.norm(normal.astype(float))
    un_inf = float(nh @ velocity)
    g = lattice.interior()
    cs = math.sqrt(1 / 3)
    if glancing:
        r = 1 + g.sum(axis=-1)
        u = (g @ c.astype(float)) / r[..., None]
        b.initial = np.ascontiguousarray(u @ nh - cs * np.log(r / density) - un_inf)
        return
    if not evolve:
        b.incoming[:] = un_inf
        return

    def macro(coords):
        coords = coords.copy()
        for a, p in enumerate(periodic):
            if p:
                coords[:, a] %= shape[a]
        cells = g[coords[:, 0], coords[:, 1], coords[:, 2]]
        rho = 1 + cells.sum(axis=-1)
        return rho, (cells @ c.astype(float)) / rho[:, None]

    rho, u = macro(foot)
    rm = u @ nh - cs * np.log(rho / density)
    projection = np.eye(3) - nh[:, None] * nh[None, :]
    ut_inf = velocity - un_inf * nh
    F = np.zeros(n)
    for a in range(3):
        if ut_inf[a] == 0 and not np.any(projection[a]):
            continue
        e = edge[:, a]
        off1 = np.where(e == -1, 1, -1)
        off2 = np.where(e == 0, 1, -2 * e)
        c0 = 1.5 * e
        c1 = np.where(e == 0, -.5, -2 * e)
        c2 = np.where(e == 0, .5, .5 * e)
        one, two = foot.copy(), foot.copy()
        one[:, a] += off1
        two[:, a] += off2
        r1, u1 = macro(one)
        r2, u2 = macro(two)
        du = c0[:, None] * u + c1[:, None] * u1 + c2[:, None] * u2
        rm1 = u1 @ nh - cs * np.log(r1 / density)
        rm2 = u2 @ nh - cs * np.log(r2 / density)
        F += un_inf * (du @ projection[a]) - ut_inf[a] * (c0 * rm + c1 * rm1 + c2 * rm2)
    b.incoming = np.ascontiguousarray(rm - F)
    b.derivative = np.ascontiguousarray(F)


# ---------------------------------------------------------------- airfoil case
class AirfoilCase:
    """The reference's uniform Solver on the CPU (solver.py:33-279).

    contours: normalized polygons (chord units, moment reference at 0);
    origin/dx/shape/omega: the plan; leading: the rotated leading edge used to
    place the perturbation envelope (solver.py:172-177).
    """

    def __init__(self, contours, shape, origin, dx, span, omega, speed, chord_cells, farfield="legacy",
                 perturbation=1e-4, seed=31, leading=(0.0, 0.0), threads=0, smagorinsky=0.0):
        self.contours = [np.asarray(cn, dtype=np.float64) for cn in contours]
        self.shape = tuple(shape)
        self.origin = tuple(origin)
        self.dx = float(dx)
        self.span = float(span)
        self.speed = float(speed)
        self.chord_cells = int(chord_cells)
        self.farfield = farfield
        self.lattice = Lattice(shape, (False, False, True), omega, 1.0, threads)
        self.lattice.smagorinsky = float(smagorinsky)
        self.wall_fallback_links = 0
        self._install(farfield)
        self._initialise(perturbation, seed, leading)
        self.lattice.build_links()
        self.last_loads = None

    # solver.py:124-155
    def _install(self, farfield):
        lat = self.lattice
        nx, ny, nz = self.shape
        x, y, z = lat.midpoints()
        freestream = (self.speed, 0.0, 0.0)
        if farfield == "legacy":
            lat.set_boundary(Boundary("ubb", 0, velocity=freestream), (x < 0) | (y < 0) | (y > ny))
            lat.set_boundary(Boundary("outflow", 0, normal=(1, 0, 0), density=1.0, velocity=freestream), x > nx)
        elif farfield == "characteristic_transport_v1":
            for normal in itertools.product((-1, 0, 1), (-1, 0, 1), (0,)):
                if not any(normal):
                    continue
                outside = np.ones(x.shape, dtype=bool)
                for value, n_a, size in zip((x, y), normal[:2], (nx, ny)):
                    if n_a < 0:
                        outside &= value < 0
                    elif n_a > 0:
                        outside &= value > size
                    else:
                        outside &= (value >= 0) & (value <= size)
                lat.set_boundary(Boundary("farfield", 0, normal=normal, velocity=freestream, density=1.0), outside)
        else:
            raise ValueError(f"unsupported farfield {farfield}")
        self._install_walls()

    def _install_walls(self):
        lat = self.lattice
        nx, ny, nz = self.shape
        x, y, z = lat.midpoints()
        self.walls = []
        xx = x[:, :, 0] * self.dx + self.origin[0]
        yy = y[:, :, 0] * self.dx + self.origin[1]
        for contour in self.contours:
            inside = contains(contour, xx, yy)
            wall = Boundary("bouzidi", 0, fractions=self._fractions(contour))
            lat.set_boundary(wall, np.broadcast_to(inside[:, :, None], x.shape))
            self.walls.append(wall)
        cx = (np.arange(nx) + 0.5) * self.dx + self.origin[0]
        cy = (np.arange(ny) + 0.5) * self.dx + self.origin[1]
        solid = np.zeros((nx, ny), dtype=bool)
        for contour in self.contours:
            mask = contains(contour, cx[:, None], cy[None, :])
            if not mask.any():
                raise ValueError("Element has no solid cells; increase resolution")
            solid |= mask
        self.solid_xy = solid

    def _fractions(self, contour):
        def compute(links):
            c, _, _ = _tables()
            xy = np.column_stack([links[:, k].astype(np.int64) - 1 + 0.5 for k in range(2)])
            directions = c[links[:, 3]][:, :2]
            keys, inv = np.unique(np.column_stack((xy, directions)), axis=0, return_inverse=True)
            inv = inv.reshape(-1)
            points = keys[:, :2] * self.dx + np.asarray(self.origin)
            offsets = keys[:, 2:] * self.dx
            q = link_fraction(contour, points, offsets)
            other = points - offsets
            blocked = np.zeros(len(points), dtype=bool)
            for element in self.contours:
                blocked |= contains(element, other[:, 0], other[:, 1])
            fallback = (q < 0.5) & blocked
            q[fallback] = -1.0
            self.wall_fallback_links += int(np.sum(fallback[inv]))
            return q[inv]
        return compute

    # solver.py:157-202
    def _initialise(self, perturbation, seed, leading):
        lat = self.lattice
        nx, ny, nz = self.shape
        rng = np.random.default_rng(seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        x, y, z = np.meshgrid(np.arange(nx) + 0.5, np.arange(ny) + 0.5, np.arange(nz) + 0.5, indexing="ij")
        u = np.zeros(self.shape + (3,))
        u[..., 0] = self.speed
        yy = y * self.dx + self.origin[1]
        xx = x * self.dx + self.origin[0]
        rel_x, rel_y = xx - leading[0], yy - leading[1]
        zz = z * self.dx
        ky = 2 * np.pi / (ny * self.dx)
        kz = 2 * np.pi / self.span
        amp = perturbation * self.speed
        envelope = np.exp(-((rel_x - 0.5) / 0.75) ** 2)
        u[..., 1] = amp * np.sin(ky * rel_y + phase_y) * np.cos(kz * zz + phase_z) * envelope
        u[..., 2] = -amp * ky / kz * np.cos(ky * rel_y + phase_y) * np.sin(kz * zz + phase_z) * envelope
        u[np.broadcast_to(self.solid_xy[:, :, None], self.shape)] = 0.0
        self.initial_velocity = u
        lat.set_equilibrium(np.ones(self.shape), u)

    # solver.py:204-250
    def loads(self):
        nx, ny, nz = self.shape
        per = np.zeros((len(self.walls), 5))
        ox, oy = self.origin[0] / self.dx, self.origin[1] / self.dx
        for i, wall in enumerate(self.walls):
            if len(wall.links):
                lib().ako_loads(_p(self.lattice.pdf), nx, ny, nz, len(wall.links), _p(wall.links), ox, oy,
                                _p(per[i]))
        total = per.sum(axis=0)
        q_area = 0.5 * self.speed ** 2 * self.chord_cells * nz
        return {"cl": float(total[1] / q_area), "cd": float(total[0] / q_area),
                "cm": float(-total[3] / (q_area * self.chord_cells)),
                "element_lattice_loads": per[:, :4].copy(), "wall_mass_exchange_lattice": float(total[4])}

    def step(self, sample=False):
        result = self.lattice.step(self.loads if sample else None)
        if result is not None:
            result["step"] = self.lattice.steps
            self.last_loads = result
        return result

    @property
    def steps(self):
        return self.lattice.steps

    # solver.py:281-297
    def diagnostics(self):
        rho, u = self.lattice.macros()
        fluid = self.lattice.fluid
        r, v = rho[fluid], u[fluid]
        if not np.isfinite(r).all() or not np.isfinite(v).all():
            raise FloatingPointError("Non-finite fluid state")
        return {"local_mach_max": float(np.sqrt(3) * np.sqrt(np.sum(v * v, axis=-1)).max()),
                "density_mean": float(r.mean()), "density_error_max": float(np.max(abs(r - 1.0)))}

    def wall_links(self):
        """All wall links as rows (x, y, z, cx, cy, cz, q) in interior coordinates."""
        c, _, _ = _tables()
        rows = []
        for wall in self.walls:
            if not len(wall.links):
                continue
            if not wall.ready:
                _initialise_boundary(self.lattice, wall)
                wall.ready = True
            e = c[wall.links[:, 3]]
            rows.append(np.column_stack((wall.links[:, :3] - 1, e, wall.q)))
        return np.concatenate(rows) if rows else np.zeros((0, 7))


def leading_edge(elements_xy, moment_reference, chord, alpha_deg):
    """Rotated leading edge in chord units about the moment reference (solver.py:172-177)."""
    original = np.concatenate([np.asarray(e) for e in elements_xy])
    leading = original[np.argmin(original[:, 0])]
    angle = -np.deg2rad(alpha_deg)
    rotation = np.array([[np.cos(angle), -np.sin(angle)], [np.sin(angle), np.cos(angle)]])
    return rotation @ ((leading - np.asarray(moment_reference)) / chord)
