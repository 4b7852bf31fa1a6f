"""CPU oracle for the exterior_regularized_fd_v1 uniform case.

TEST INFRASTRUCTURE ONLY: imported by tests/ and never by the product.  It
restates the reference's exterior mode, src/aerokinetic/exterior.py:18-200 with
its wiring in solver.py:36-41, 81-89, 179-201, 204-271:

  * the lattice is the physical core padded by one auxiliary cell in x and y
    (the "ring"), stepped in collide-stream order with pre-collision storage;
    a UBB at the freestream sits in the ghost layer outside the ring
    (exterior.py:19-35)
  * each step: the macroscopic state (log rho, u) of the stored populations;
    an SSP-RK3 predictor of the ring state driven by one-sided characteristic
    right-hand sides (exterior.py:81-151); collide, boundaries and the wall
    loads (with the incoming-minus-outgoing wall mass); stream; then every
    ring cell is rebuilt from the predicted state as a regularised population
    set (exterior.py:153-171, 186-200), and the change it makes is the
    "exterior source" reported with the loads.

The lattice operations are ak_oracle.c's (the same ones that are pinned for
the uniform solver); only the ring arithmetic below is new.  It is pinned
against the reference's recorded airfoil run of this mode
(docs/verification_exterior_library_20261108/raw/matched_airfoils/
airfoil_down3/history.csv, written by the exterior.py whose SHA-256 the
run's SOURCE_IDENTITY.json records).
"""
import numpy as np

from . import oracle as O

CS = np.sqrt(1.0 / 3.0)


class RingGeometry:
    """Ring cells of an (NX, NY) storage plane with their outward normals."""

    def __init__(self, NX, NY):
        on = np.zeros((NX, NY), dtype=bool)
        on[0, :] = on[-1, :] = on[:, 0] = on[:, -1] = True
        self.x, self.y = np.nonzero(on)
        self.NX, self.NY = NX, NY
        self.nvx = np.where(self.x == 0, -1, np.where(self.x == NX - 1, 1, 0))
        self.nvy = np.where(self.y == 0, -1, np.where(self.y == NY - 1, 1, 0))
        self.ell = np.sqrt(self.nvx ** 2 + self.nvy ** 2.0)
        self.n = np.column_stack((self.nvx / self.ell, self.nvy / self.ell, np.zeros(len(self.x))))


def _derivative_1d(index, edge):
    """d/dx of field (P, nz, 4) along one non-periodic axis at the ring points:
    second-order one-sided at an edge (edge = -1 forward, +1 backward), central
    inside.  index(i) -> field rows at offset i."""
    c0 = 1.5 * edge
    c1 = np.where(edge == 0, -0.5, -2.0 * edge)
    c2 = np.where(edge == 0, 0.5, 0.5 * edge)
    one = np.where(edge == -1, 1, -1)
    two = np.where(edge == 0, 1, -2 * edge)
    return (c0[:, None, None] * index(0) + c1[:, None, None] * index(one)) + c2[:, None, None] * index(two)


class ExteriorState:
    """The ring predictor and reconstruction over a (NX, NY, nz, 4) state."""

    def __init__(self, NX, NY, nz, speed, omega):
        self.g = RingGeometry(NX, NY)
        self.nz = nz
        self.U = np.array([speed, 0.0, 0.0])
        self.omega = float(omega)
        n = self.g.n
        self.uninf = n @ self.U
        self.utinf = self.U[None, :] - self.uninf[:, None] * n
        self.initial = None

    def ring(self, state):
        return state[self.g.x, self.g.y]

    def gradients(self, state):
        """(P, nz, 3 axes, 4 components) at the ring points."""
        g, x, y = self.g, self.g.x, self.g.y
        out = np.empty((len(x), self.nz, 3, 4))
        out[:, :, 0] = _derivative_1d(lambda i: state[x + i, y], g.nvx)
        out[:, :, 1] = _derivative_1d(lambda i: state[x, y + i], g.nvy)
        here = state[x, y]
        out[:, :, 2] = (np.roll(here, -1, axis=1) - np.roll(here, 1, axis=1)) / 2
        return out

    def incoming_trace(self, time):
        """Characteristic u.n - cs log rho of the initial state, traced along the
        freestream to the ring points (trilinear; outside the storage the
        freestream value u_inf.n)."""
        g = self.g
        tx = g.x - self.U[0] * time
        lo = np.floor(tx).astype(np.int64)
        frac = tx - lo
        n = g.n
        answer = np.zeros((len(g.x), self.nz))
        for bit in (0, 1):
            xs = lo + bit
            weight = frac if bit else 1.0 - frac
            valid = (xs >= 0) & (xs < g.NX)
            v = self.initial[np.clip(xs, 0, g.NX - 1), g.y]
            incoming = (v[..., 1] * n[:, None, 0] + v[..., 2] * n[:, None, 1] + v[..., 3] * n[:, None, 2]
                        - CS * v[..., 0])
            answer += weight[:, None] * np.where(valid[:, None], incoming, self.uninf[:, None])
        return answer

    def enforce(self, y, time):
        n = self.g.n[:, None, :]
        y = y.copy()
        u = y[..., 1:]
        un = np.sum(u * n, axis=-1)
        rp = un + CS * y[..., 0]
        inflow = (self.uninf < 0)[:, None] & np.ones(self.nz, dtype=bool)
        glancing = (self.uninf == 0)[:, None] & np.ones(self.nz, dtype=bool)
        chosen = inflow | glancing
        rm = np.where(inflow, self.uninf[:, None], self.incoming_trace(time))
        new_un = (rp + rm) / 2
        tangent = u - un[..., None] * n
        tangent = np.where(inflow[..., None], self.utinf[:, None, :], tangent)
        y[..., 0] = np.where(chosen, (rp - rm) / (2 * CS), y[..., 0])
        y[..., 1:] = np.where(chosen[..., None], new_un[..., None] * n + tangent, u)
        return y

    def rhs(self, y, current):
        g = self.g
        stage = current.copy()
        stage[g.x, g.y] = y
        grad = self.gradients(stage)
        Gv, dq = grad[..., 1:], grad[..., 0]  # Gv[..., a, b] = d u_b / d x_a
        n = g.n[:, None, :]
        u = y[..., 1:]
        un = np.sum(u * n, axis=-1)
        rp = un + CS * y[..., 0]
        inner = stage[g.x - g.nvx, g.y - g.nvy]
        u_in = inner[..., 1:]
        un_in = np.sum(u_in * n, axis=-1)
        rp_in = un_in + CS * inner[..., 0]
        Gn = np.einsum("...ab,...b->...a", Gv, n)  # gradient of the normal velocity
        div = np.trace(Gv, axis1=-2, axis2=-1) - np.sum(n * Gn, axis=-1)
        uninf, utinf, ell = self.uninf[:, None], self.utinf[:, None, :], g.ell[:, None]
        r_minus = uninf * div - np.sum(utinf * (Gn - CS * dq), axis=-1)
        r_plus = -(uninf + CS) * (rp - rp_in) / ell - np.sum(utinf * (Gn + CS * dq), axis=-1) - CS * div
        tangent = u - un[..., None] * n
        tangent_in = u_in - un_in[..., None] * n
        adv = np.einsum("...a,...ab->...b", utinf * np.ones_like(u), Gv)
        adv = adv - np.sum(adv * n, axis=-1)[..., None] * n
        pressure = dq - np.sum(dq * n, axis=-1)[..., None] * n
        d_tangent = -uninf[..., None] * (tangent - tangent_in) / ell[..., None] - adv - CS ** 2 * pressure
        out = np.empty_like(y)
        out[..., 0] = (r_plus - r_minus) / (2 * CS)
        out[..., 1:] = n * ((r_plus + r_minus) / 2)[..., None] + d_tangent
        return out

    def predict(self, current, step):
        """Shu-Osher SSP-RK3 with the boundary conditions enforced at each stage."""
        y0 = self.ring(current)
        y1 = self.enforce(y0 + self.rhs(y0, current), step + 1)
        y2 = self.enforce(0.75 * y0 + 0.25 * (y1 + self.rhs(y1, current)), step + 0.5)
        y3 = self.enforce((y0 + 2 * (y2 + self.rhs(y2, current))) / 3, step + 1)
        if not np.isfinite(y3).all():
            raise FloatingPointError("Non-finite exterior predictor")
        return y3

    def regularized(self, state):
        """Populations (P, nz, 27) of the ring from its (log rho, u) and the
        Navier-Stokes stress of the state's velocity gradients."""
        c, w, _ = O._tables()
        y = self.ring(state)
        rho = np.exp(y[..., 0])
        v = y[..., None, 1:]  # (P, nz, 1, 3)
        Gv = self.gradients(state)[..., 1:]
        div = np.trace(Gv, axis1=-2, axis2=-1)
        om = self.omega
        stress = (-rho[..., None, None] / 3) * ((Gv + np.swapaxes(Gv, -1, -2)) / om
                                                 + np.eye(3) * (2 / 3 * div * (1 - 1 / om))[..., None, None])
        cc = c[None, None, :, :].astype(np.float64)  # (1, 1, 27, 3)
        phi = 2 / 3 - v * v + (1.5 * v * v - 0.5) * cc * cc + cc * v / 2
        first = -2 * v + 3 * v * cc * cc + cc / 2
        second = 1.5 * cc * cc - 1
        g = rho[..., None] * (phi[..., 0] * phi[..., 1] * phi[..., 2]) - w
        others = ((1, 2), (0, 2), (0, 1))
        for a in range(3):
            i, j = others[a]
            g = g + stress[..., a, a, None] * second[..., a] * (phi[..., i] * phi[..., j])
        for a, b in ((0, 1), (0, 2), (1, 2)):
            g = g + stress[..., a, b, None] * first[..., a] * first[..., b] * phi[..., 3 - a - b]
        return g


class ExteriorCase(O.AirfoilCase):
    """The reference's uniform Solver with farfield exterior_regularized_fd_v1.

    shape/origin are the physical plan's; the lattice is padded by the ring
    (solver.py:38-40).  pdf holds pre-collision populations.
    """

    def __init__(self, contours, shape, origin, dx, span, omega, speed, chord_cells, perturbation=1e-4, seed=31,
                 leading=(0.0, 0.0), threads=0):
        self.core_shape = tuple(int(v) for v in shape)
        storage = (self.core_shape[0] + 2, self.core_shape[1] + 2, self.core_shape[2])
        self.omega = float(omega)
        self._core_ny = self.core_shape[1]
        super().__init__(contours, storage, (origin[0] - dx, origin[1] - dx), dx, span, omega, speed, chord_cells,
                         "exterior", perturbation, seed, leading, threads)
        self.exterior = ExteriorState(storage[0], storage[1], storage[2], speed, omega)
        self.source_last = np.zeros(4)
        self.source_total = np.zeros(4)
        self.wall_mass_last = 0.0
        self.wall_mass_total = 0.0

    def _install(self, farfield):
        # exterior.py:33: UBB on every ghost cell outside the storage in x or y
        lat = self.lattice
        nx, ny, _ = self.shape
        x, y, _ = lat.midpoints()
        lat.set_boundary(O.Boundary("ubb", 0, velocity=(self.speed, 0.0, 0.0)), (x < 0) | (x > nx) | (y < 0) | (y > ny))
        self._install_walls()

    def _initialise(self, perturbation, seed, leading):
        # solver.py:157-201 over the storage: perturbed core, freestream ring
        lat = self.lattice
        nx, ny, nz = self.shape
        rng = np.random.default_rng(seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        x, y, z = np.meshgrid(np.arange(nx) + 0.5, np.arange(ny) + 0.5, np.arange(nz) + 0.5, indexing="ij")
        u = np.zeros(self.shape + (3,))
        u[..., 0] = self.speed
        xx, yy = x * self.dx + self.origin[0], y * self.dx + self.origin[1]
        rel_x, rel_y = xx - leading[0], yy - leading[1]
        zz = z * self.dx
        ky = 2 * np.pi / (self._core_ny * self.dx)
        kz = 2 * np.pi / self.span
        amp = perturbation * self.speed
        envelope = np.exp(-((rel_x - 0.5) / 0.75) ** 2)
        u[..., 1] = amp * np.sin(ky * rel_y + phase_y) * np.cos(kz * zz + phase_z) * envelope
        u[..., 2] = -amp * ky / kz * np.cos(ky * rel_y + phase_y) * np.sin(kz * zz + phase_z) * envelope
        u[np.broadcast_to(self.solid_xy[:, :, None], self.shape)] = 0.0
        owned = np.zeros(self.shape, dtype=bool)
        owned[1:-1, 1:-1] = True
        u[~owned] = (self.speed, 0.0, 0.0)
        self.initial_velocity = u
        lat.set_equilibrium(np.ones(self.shape), u)

    @property
    def core_solid_xy(self):
        return self.solid_xy[1:-1, 1:-1]

    def state(self):
        rho, u = self.lattice.macros()
        return np.concatenate((np.log(rho)[..., None], u), axis=-1)

    def step(self, sample=False):
        lat, ext = self.lattice, self.exterior
        nx, ny, nz = self.shape
        current = self.state()
        if ext.initial is None:
            ext.initial = current.copy()
        predicted = ext.predict(current, lat.steps)
        L = O.lib()
        L.ako_collide(O._p(lat.pdf), nx, ny, nz, lat.omega_s, lat.omega_b, lat.threads)
        lat.sync()
        lat.apply_boundaries()
        loads = self.loads()
        L.ako_stream(O._p(lat.pdf), O._p(lat.tmp), nx, ny, nz)
        lat.pdf, lat.tmp = lat.tmp, lat.pdf
        nxt = self.state()
        nxt[ext.g.x, ext.g.y] = predicted
        rebuilt = ext.regularized(nxt)
        inner = lat.interior()
        old = inner[ext.g.x, ext.g.y].copy()
        inner[ext.g.x, ext.g.y] = rebuilt
        dm = rebuilt - old
        c, _, _ = O._tables()
        self.source_last = np.r_[dm.sum(), np.einsum("pzq,qa->a", dm, c.astype(np.float64))]
        self.source_total = self.source_total + self.source_last
        self.wall_mass_last = loads["wall_mass_exchange_lattice"]
        self.wall_mass_total += self.wall_mass_last
        lat.steps += 1
        if not sample:
            return None
        loads.update(step=lat.steps, wall_mass_exchange_accumulated=self.wall_mass_total,
                     exterior_source_mass_lattice=float(self.source_last[0]),
                     exterior_source_mass_accumulated=float(self.source_total[0]))
        self.last_loads = loads
        return loads

    def post_collision(self):
        """The core's populations after the next collision (what a fused
        collide-at-the-end engine stores), (nx, ny, nz, 27)."""
        return O.collide(self.lattice.interior()[1:-1, 1:-1], self.omega, 1.0)

    def diagnostics(self):
        # solver.py:281-297: the guards over every storage fluid cell, the mean
        # density over the physical core
        rho, u = self.lattice.macros()
        fluid = self.lattice.fluid
        r, v = rho[fluid], u[fluid]
        if not np.isfinite(r).all() or not np.isfinite(v).all():
            raise FloatingPointError("Non-finite fluid state")
        core = rho[1:-1, 1:-1][fluid[1:-1, 1:-1]]
        return {"local_mach_max": float(np.sqrt(3) * np.sqrt(np.sum(v * v, axis=-1)).max()),
                "density_mean": float(core.mean()), "density_error_max": float(np.max(abs(r - 1.0)))}
