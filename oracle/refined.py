"""CPU oracle for the two-level (2:1) refined step: numpy around ak_oracle.c.

TEST INFRASTRUCTURE ONLY (see oracle.py).  Restates, in the reference's own
structure, the static two-level solver:

  * levels and stress rescaling          refinement.py:23-65, 205-213
  * moments <-> populations (Hermite)     refinement.py:148-203; parallel.py:14-56
  * 5-point prolongation, restriction     refinement.py:78-114
  * face-flux samplers                    interface.py:44-104
  * one coarse step with two fine steps,
    donors, reflux and restriction        interface.py:257-352
  * airfoil specialisation (virtual core,
    fine walls, outer UBB/outflow, loads)  refined_solver.py:115-345

Both levels store pre-collision populations (collide, boundaries, stream).
"""
from itertools import combinations, product
import math

import numpy as np

from . import oracle as O

CS2 = 1.0 / 3.0
SECOND = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


class Level:
    """dx, dt and relaxation times of one level (refinement.py:23-65)."""

    def __init__(self, dx, dt, tau_shear, tau_bulk):
        self.dx, self.dt, self.tau_shear, self.tau_bulk = float(dx), float(dt), float(tau_shear), float(tau_bulk)

    def refined(self):
        return Level(self.dx / 2, self.dt / 2, 0.5 + 2 * (self.tau_shear - 0.5), 0.5 + 2 * (self.tau_bulk - 0.5))

    @property
    def velocity_unit(self):
        return self.dx / self.dt


class Transfer:
    """Ten-moment regularised remap between populations and (rho, j, Pi_neq)."""

    def __init__(self, coarse):
        self.c, self.w, _ = O.stencil()
        self.coarse, self.fine = coarse, coarse.refined()
        self.second = np.stack([self.c[:, a] * self.c[:, b] for a, b in SECOND], axis=1).astype(float)
        hermite = self.second.copy()
        hermite[:, :3] -= CS2
        hermite[:, 3:] *= 2
        self.recon = self.w[:, None] * hermite / (2 * CS2 ** 2)

    def moments(self, pdf):
        pdf = np.asarray(pdf, dtype=np.float64)
        drho = pdf.sum(axis=-1)
        rho = drho + 1
        if np.any(rho <= 0):
            raise ValueError("Transfer encountered nonpositive density")
        if np.any(pdf + self.w < 0):
            raise ValueError("Donor has negative physical populations")
        j = pdf @ self.c.astype(float)
        self._mach(rho, j)
        pi = pdf @ self.second
        pi[..., :3] -= drho[..., None] * CS2
        for k, (a, b) in enumerate(SECOND):
            pi[..., k] -= j[..., a] * j[..., b] / rho
        return np.concatenate((rho[..., None], j, pi), axis=-1)

    @staticmethod
    def _mach(rho, j):
        if np.any(np.linalg.norm(j, axis=-1) / rho / math.sqrt(CS2) > 0.3):
            raise ValueError("Transfer supports local lattice Mach <= 0.3 only")

    def populations(self, fields):
        fields = np.asarray(fields, dtype=np.float64)
        rho, j = fields[..., 0], fields[..., 1:4]
        if np.any(rho <= 0):
            raise ValueError("Prediction produced nonpositive density")
        self._mach(rho, j)
        u = j / rho[..., None]
        eq = np.ones(rho.shape + (27,))
        for a in range(3):
            v = u[..., a, None]
            d = self.c[:, a]
            eq *= np.where(d == 0, 2 / 3 - v ** 2, (CS2 + v ** 2 + d * v) / 2)
        eq *= rho[..., None]
        pdf = eq + fields[..., 4:] @ self.recon.T
        if not np.isfinite(pdf).all() or np.any(pdf < 0):
            raise ValueError("Prediction produced invalid or negative physical populations")
        return pdf - self.w

    @staticmethod
    def rescale_stress(fields, source, target):
        out = fields.copy()
        pi = out[..., 4:]
        iso = pi[..., :3].mean(axis=-1)
        shear = target.tau_shear * target.dt / (source.tau_shear * source.dt)
        bulk = target.tau_bulk * target.dt / (source.tau_bulk * source.dt)
        pi *= shear
        pi[..., :3] += (bulk - shear) * iso[..., None]
        return out

    def restrict(self, fine_pdf):
        fields = self.moments(fine_pdf)
        return self.populations(self.rescale_stress(restrict_cell_averages(fields), self.fine, self.coarse))


def prolong_cell_averages(values):
    """children = parent -+ [11/64 (a+1 - a-1) - 3/128 (a+2 - a-2)] per axis."""
    for axis in range(3):
        idx = np.arange(2, values.shape[axis] - 2)
        centre = np.take(values, idx, axis=axis)
        offset = (11 / 64 * (np.take(values, idx + 1, axis=axis) - np.take(values, idx - 1, axis=axis))
                  - 3 / 128 * (np.take(values, idx + 2, axis=axis) - np.take(values, idx - 2, axis=axis)))
        values = np.stack((centre - offset, centre + offset), axis=axis + 1)
        shape = list(centre.shape)
        shape[axis] *= 2
        values = values.reshape(shape)
    return values


def restrict_cell_averages(values):
    nx, ny, nz = values.shape[:3]
    return values.reshape(nx // 2, 2, ny // 2, 2, nz // 2, 2, *values.shape[3:]).mean(axis=(1, 3, 5))


class FaceFlux:
    """Moment flux of pull streaming through a face patch (interface.py:44-104)."""

    def __init__(self, shape, axis, index, ranges, periodic):
        c, _, _ = O.stencil()
        self.shape, self.axis = tuple(shape), axis
        others = [a for a in range(3) if a != axis]
        self.out_shape = tuple(hi - lo for lo, hi in ranges)
        self.terms = []
        for d, v in enumerate(c):
            normal = v[axis]
            if normal == 0:
                continue
            moving = [a for a in others if v[a] != 0]
            m = len(moving)
            for count in range(m + 1):
                weight = math.factorial(count) * math.factorial(m - count) / math.factorial(m + 1)
                for subset in combinations(moving, count):
                    coords = [None] * 3
                    coords[axis] = np.array([index + (1 if normal < 0 else 0)])
                    for a, (lo, hi) in zip(others, ranges):
                        coords[a] = np.arange(lo, hi) - (v[a] if a in subset else 0)
                    for a in range(3):
                        if periodic:
                            coords[a] = coords[a] % self.shape[a]
                    coef = weight * normal * np.r_[1.0, v.astype(float)]
                    self.terms.append((d, np.ix_(*coords), coef))

    def __call__(self, pdf):
        out = np.zeros(self.out_shape + (4,))
        for d, idx, coef in self.terms:
            out += pdf[..., d][idx].squeeze(axis=self.axis)[..., None] * coef
        return out


class RefinedCase:
    """RefinedSolver (refined_solver.py:115-345) on the CPU.

    coarse_shape/origin/dx/dt/tau_shear: the uniform plan; box_lower/upper:
    the fine box in coarse cells (z spans the whole span); tau_bulk: the
    coarse bulk relaxation time; contours: normalised polygons.
    """
    pad = 2

    def __init__(self, contours, coarse_shape, origin, dx, dt, tau_shear, tau_bulk, box_lower, box_upper, speed,
                 perturbation, seed, leading, span, threads=0):
        self.contours = [np.asarray(cn, dtype=np.float64) for cn in contours]
        self.shape = tuple(coarse_shape)
        self.origin = tuple(origin)
        self.lower, self.upper = tuple(box_lower), tuple(box_upper)
        self.box_shape = tuple(h - l for l, h in zip(self.lower, self.upper))
        self.box = tuple(slice(l, h) for l, h in zip(self.lower, self.upper))
        self.coarse_level = Level(dx, dt, tau_shear, tau_bulk)
        self.fine_level = self.coarse_level.refined()
        self.speed, self.span = float(speed), float(span)
        self.T = Transfer(self.coarse_level)
        self.fine_shape = tuple(2 * n for n in self.box_shape)
        self.padded = tuple(n + 2 * self.pad for n in self.fine_shape)
        self.fine_slices = tuple(slice(self.pad, self.pad + n) for n in self.fine_shape)
        self.free_fields = np.zeros(10)
        self.free_fields[0] = 1.0
        self.free_fields[1] = self.speed
        self.free_pdf = self.T.populations(self.free_fields)
        core = np.ones(self.box_shape, bool)
        for axis in (0, 1):
            band = np.zeros(self.box_shape[axis], bool)
            band[3:-3] = True
            shape = [1, 1, 1]
            shape[axis] = len(band)
            core &= band.reshape(shape)
        self.virtual_core = core
        self.fine_virtual_core = np.repeat(np.repeat(np.repeat(core, 2, 0), 2, 1), 2, 2)
        self.coarse_owned = np.ones(self.shape, bool)
        self.coarse_owned[self.box] = False
        self._faces()
        self._outer_samplers()
        self.external_in = None
        self.outer_convention = "padded"
        self._lattices(threads)
        self._initialise(perturbation, seed, leading)
        self.steps = 0
        self.fine_steps = 0

    # interface.py:176-195
    def _faces(self):
        self.reflux_support = np.zeros(self.shape, bool)
        self.faces = []
        for axis in range(3):
            if self.lower[axis] == 0 and self.upper[axis] == self.shape[axis]:
                continue
            others = [a for a in range(3) if a != axis]
            cranges = [(self.lower[a], self.upper[a]) for a in others]
            franges = [(self.pad, self.pad + self.fine_shape[a]) for a in others]
            for side in (-1, 1):
                cidx = self.lower[axis] - 1 if side < 0 else self.upper[axis] - 1
                fidx = self.pad - 1 if side < 0 else self.pad + self.fine_shape[axis] - 1
                outside = list(self.box)
                outside[axis] = self.lower[axis] - 1 if side < 0 else self.upper[axis]
                outside = tuple(outside)
                self.reflux_support[outside] = True
                self.faces.append((axis, side, outside, FaceFlux(self.shape, axis, cidx, cranges, True),
                                   FaceFlux(self.padded, axis, fidx, franges, False)))

    # refined_solver.py:215-222: flux samplers on the six outer faces of the
    # padded coarse lattice (the z pair cancels: its ghosts are periodic copies)
    def _outer_samplers(self):
        padded = tuple(n + 2 for n in self.shape)
        self.outer = []
        for axis in range(3):
            ranges = [(1, self.shape[a] + 1) for a in range(3) if a != axis]
            for side, index in ((-1, 0), (1, self.shape[axis])):
                self.outer.append((axis, side, FaceFlux(padded, axis, index, ranges, False)))

    def _wrapped_view(self, pdf):
        """The padded coarse state as a lattice that wraps z by index holds it.

        With z ghost layers (the reference's layout) a ghost-column population
        that streaming pulls across the periodic z seam is written into a z
        ghost layer, while its slot in the interior layer keeps an older value;
        with z wrapped by index it lives in the interior layer.  The outer-face
        samplers read such slots, so the two layouts can give slightly
        different outer fluxes (on the refined start-up case the budgets agree
        to 1e-17 per volume); with outer_convention "wrapped" the samplers read
        this view, the engine's layout."""
        nz = self.shape[2]
        c, _, _ = O.stencil()
        view = pdf.copy()
        ring = np.ones(view.shape[:2], bool)
        ring[1:-1, 1:-1] = False
        for q in np.where(c[:, 2] == 1)[0]:
            view[ring, nz, q] = pdf[ring, 0, q]
        for q in np.where(c[:, 2] == -1)[0]:
            view[ring, 1, q] = pdf[ring, nz + 1, q]
        view[:, :, 0] = view[:, :, nz]
        view[:, :, nz + 1] = view[:, :, 1]
        return view

    def _lattices(self, threads):
        c = self.coarse_level
        f = self.fine_level
        self.coarse = O.Lattice(self.shape, (False, False, True), 1 / c.tau_shear, 1 / c.tau_bulk, threads)
        self.fine = O.Lattice(self.padded, (True, True, True), 1 / f.tau_shear, 1 / f.tau_bulk, threads)
        nx, ny, nz = self.shape
        x, y, z = self.coarse.midpoints()
        freestream = (self.speed, 0.0, 0.0)
        self.coarse.set_boundary(O.Boundary("ubb", 0, velocity=freestream), (x < 0) | (y < 0) | (y > ny))
        self.coarse.set_boundary(O.Boundary("outflow", 0, normal=(1, 0, 0), density=1.0, velocity=freestream),
                                 x > nx)
        # fine walls, in common length units of the padded fine frame
        dxf = f.dx
        self.fine_origin = (self.origin[0] + self.lower[0] * c.dx - self.pad * dxf,
                            self.origin[1] + self.lower[1] * c.dx - self.pad * dxf)
        fx, fy, fz = self.fine.midpoints()
        xx = fx[:, :, 0] * dxf + self.fine_origin[0]
        yy = fy[:, :, 0] * dxf + self.fine_origin[1]
        self.walls = []
        self.fallback_links = 0
        for contour in self.contours:
            inside = O.contains(contour, xx, yy)
            wall = O.Boundary("bouzidi", 0, fractions=self._fractions(contour))
            self.fine.set_boundary(wall, np.broadcast_to(inside[:, :, None], fx.shape))
            self.walls.append(wall)
        self.coarse.build_links()
        self.fine.build_links()

    def _fractions(self, contour):
        def compute(links):
            c, _, _ = O.stencil()
            dxf = self.fine_level.dx
            xy = np.column_stack([links[:, k].astype(np.int64) - 1 + 0.5 for k in range(2)])
            keys, inv = np.unique(np.column_stack((xy, c[links[:, 3]][:, :2])), axis=0, return_inverse=True)
            inv = inv.reshape(-1)
            points = keys[:, :2] * dxf + np.asarray(self.fine_origin)
            offsets = keys[:, 2:] * dxf
            q = O.link_fraction(contour, points, offsets)
            other = points - offsets
            blocked = np.zeros(len(points), bool)
            for element in self.contours:
                blocked |= O.contains(element, other[:, 0], other[:, 1])
            fallback = (q < 0.5) & blocked
            q[fallback] = -1.0
            self.fallback_links += int(np.sum(fallback[inv]))
            return q[inv]
        return compute

    # refined_solver.py:224-269 and interface.py:232-244
    def _initialise(self, perturbation, seed, leading):
        for lat in (self.coarse, self.fine):
            lat.pdf[...] = self.free_pdf
            lat.tmp[...] = self.free_pdf
        rng = np.random.default_rng(seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        c = self.coarse_level
        ky = 2 * np.pi / (self.shape[1] * c.dx)
        kz = 2 * np.pi / self.span
        amp = perturbation * self.speed

        def initial(shape, dx, offset):
            x, y, z = np.meshgrid(*[(np.arange(n) + 0.5) * dx + o for n, o in zip(shape, offset)],
                                  indexing="ij", sparse=True)
            xx, yy = x + self.origin[0], y + self.origin[1]
            rel_x, rel_y = xx - leading[0], yy - leading[1]
            j = np.zeros(tuple(shape) + (3,))
            j[..., 0] = self.speed
            env = np.exp(-((rel_x - 0.5) / 0.75) ** 2)
            j[..., 1] = amp * np.sin(ky * rel_y + phase_y) * np.cos(kz * z + phase_z) * env
            j[..., 2] = -amp * ky / kz * np.cos(ky * rel_y + phase_y) * np.sin(kz * z + phase_z) * env
            solid = np.zeros(shape[:2], bool)
            for contour in self.contours:
                solid |= O.contains(contour, xx[:, :, 0], yy[:, :, 0])
            j[np.broadcast_to(solid[:, :, None], j.shape[:3])] = 0.0
            fields = np.zeros(tuple(shape) + (10,))
            fields[..., 0] = 1.0
            fields[..., 1:4] = j
            return self.T.populations(fields)

        coarse_pdf = initial(self.shape, c.dx, (0.0, 0.0, 0.0))
        offset = tuple(lo * c.dx - self.pad * self.fine_level.dx for lo in self.lower)
        fine_pdf = initial(self.padded, self.fine_level.dx, offset)
        coarse_pdf[self.box] = self.restrict(fine_pdf[self.fine_slices])
        self.coarse.pdf[1:-1, 1:-1, 1:-1] = coarse_pdf
        self.fine.pdf[1:-1, 1:-1, 1:-1] = fine_pdf
        # boundary data is prepared now, from the initial state (refined_solver.py:259-262)
        for lat in (self.coarse, self.fine):
            for b in lat.boundaries:
                if len(b.links) and not b.ready:
                    O._initialise_boundary(lat, b)
                    b.ready = True

    def restrict(self, fine_state):
        safe = fine_state.copy()
        safe[self.fine_virtual_core] = self.free_pdf
        result = self.T.restrict(safe)
        result[self.virtual_core] = self.free_pdf
        return result

    def donor_block(self, coarse_pdf):
        safe = coarse_pdf.copy()
        covered = safe[self.box]
        covered[self.virtual_core] = self.free_pdf
        safe[self.box] = covered
        out = safe
        for axis, (lo, hi) in enumerate(zip(self.lower, self.upper)):
            out = np.take(out, np.arange(lo - 3, hi + 3) % self.shape[axis], axis=axis)
        return out

    def fine_donors(self, before, after, fraction):
        a, b = self.T.moments(before), self.T.moments(after)
        fields = prolong_cell_averages((1 - fraction) * a + fraction * b)
        fields = Transfer.rescale_stress(fields, self.coarse_level, self.fine_level)
        fields[self.fine_slices] = self.free_fields
        return self.T.populations(fields)

    def _wrap_z(self, pdf):
        n, p = self.fine_shape[2], self.pad
        pdf[:, :, 0:p] = pdf[:, :, n:n + p]
        pdf[:, :, n + p:n + 2 * p] = pdf[:, :, p:2 * p]

    def _measure(self):
        """walls.py:68-95 on the fine level, owned links only, common length units."""
        c, _, inv = O.stencil()
        dxf = self.fine_level.dx
        pdf = self.fine.pdf
        force, moment, mass = np.zeros(3), 0.0, 0.0
        lo = [s.start for s in self.fine_slices]
        hi = [s.stop for s in self.fine_slices]
        for wall in self.walls:
            L = wall.links.astype(np.int64)
            owned = np.ones(len(L), bool)
            for a in range(3):
                coord = L[:, a] - 1
                owned &= (coord >= lo[a]) & (coord < hi[a])
            L = L[owned]
            d = L[:, 3]
            e = c[d]
            out = pdf[L[:, 0], L[:, 1], L[:, 2], d]
            inc = pdf[L[:, 0] + e[:, 0], L[:, 1] + e[:, 1], L[:, 2] + e[:, 2], inv[d]]
            lf = (out + inc)[:, None] * e
            force += lf.sum(axis=0)
            rx = (L[:, 0] - 1 + 0.5) * dxf + self.fine_origin[0]
            ry = (L[:, 1] - 1 + 0.5) * dxf + self.fine_origin[1]
            moment += np.sum(rx * lf[:, 1] - ry * lf[:, 0])
            mass += np.sum(inc - out)
        return force, moment, mass

    def _stream(self, lat):
        lat.sync()
        lat.apply_boundaries()
        measured = self._measure() if lat is self.fine else None
        if lat is self.coarse and self.external_in is not None:
            # refined_solver.py:274-278: inflow through the outer faces
            pdf = lat.pdf if self.outer_convention == "padded" else self._wrapped_view(lat.pdf)
            for _, side, sampler in self.outer:
                self.external_in -= side * sampler(pdf).sum(axis=(0, 1)) * self.coarse_level.dx ** 3
        nx, ny, nz = lat.shape
        O.lib().ako_stream(O._p(lat.pdf), O._p(lat.tmp), nx, ny, nz)
        lat.pdf, lat.tmp = lat.tmp, lat.pdf
        return measured

    def _collide(self, lat):
        nx, ny, nz = lat.shape
        O.lib().ako_collide(O._p(lat.pdf), nx, ny, nz, lat.omega_s, lat.omega_b, lat.threads)

    # interface.py:311-352 with the refined_solver.py overrides; loads of refined_solver.py:311-327
    def step(self):
        c, f = self.coarse_level, self.fine_level
        old = self.coarse.interior().copy()
        fine_state = self.fine.interior()[self.fine_slices].copy()
        self._collide(self.coarse)
        post = self.coarse.interior()
        coarse_flux = [s(post) * c.dx ** 3 for _, _, _, s, _ in self.faces]
        self._stream(self.coarse)
        prediction = self.coarse.interior().copy()
        before, after = self.donor_block(old), self.donor_block(prediction)
        fine_flux = [np.zeros_like(x) for x in coarse_flux]
        walls = []
        for sub in range(2):
            padded = self.fine_donors(before, after, sub / 2)
            padded[self.fine_slices] = fine_state
            self._wrap_z(padded)
            self.fine.pdf[1:-1, 1:-1, 1:-1] = padded
            self._collide(self.fine)
            post = self.fine.interior()
            for i, (_, _, _, _, s) in enumerate(self.faces):
                flux = s(post)
                a, b = flux.shape[:2]
                fine_flux[i] += flux.reshape(a // 2, 2, b // 2, 2, 4).sum(axis=(1, 3)) * f.dx ** 3
            walls.append(self._stream(self.fine))
            fine_state = self.fine.interior()[self.fine_slices].copy()
        correction = np.zeros(self.shape + (4,))
        for (axis, side, outside, _, _), fc, ff in zip(self.faces, coarse_flux, fine_flux):
            correction[outside] += side * (ff - fc) / c.dx ** 3
        support = self.reflux_support
        old_m = self.T.moments(prediction[support])
        old_m[..., 4:] = 0
        new_m = old_m.copy()
        new_m[..., :4] += correction[support]
        prediction[support] += self.T.populations(new_m) - self.T.populations(old_m)
        self.T.moments(prediction[support])
        prediction[self.box] = self.restrict(fine_state)
        self.coarse.pdf[1:-1, 1:-1, 1:-1] = prediction
        self.steps += 1
        self.fine_steps += 2
        volume = f.dx ** 3
        unit = f.velocity_unit
        impulse = sum(w[0] for w in walls) * volume * unit
        moment = sum(w[1] for w in walls) * volume * unit
        q_area = 0.5 * self.span
        force = impulse / c.dt
        return {"step": self.steps, "cl": float(force[1] / q_area), "cd": float(force[0] / q_area),
                "cm": float(-(moment / c.dt) / q_area), "wall_mass": float(sum(w[2] for w in walls) * volume),
                "wall_impulse": impulse}

    def fine_fluid(self):
        return np.broadcast_to((self.fine.flags[1:-1, 1:-1, 1:-1] == 0)[self.fine_slices], self.fine_shape)

    # refined_solver.py:291-299
    def conserved_integrals(self):
        mass, impulse = 0.0, np.zeros(3)
        c, _, _ = O.stencil()
        views = (self.coarse.interior(), self.fine.interior()[self.fine_slices])
        for pdf, owned, level in zip(views, (self.coarse_owned, self.fine_fluid()),
                                      (self.coarse_level, self.fine_level)):
            rho = pdf.sum(axis=-1) + 1
            j = pdf @ c.astype(np.float64)
            mass += rho[owned].sum() * level.dx ** 3
            impulse += j[owned].sum(axis=0) * level.dx ** 3 * level.velocity_unit
        return {"mass": float(mass), "momentum": impulse.tolist()}

    # refined_solver.py:311-343: the step plus its mass and momentum budget
    def step_with_budget(self):
        before = self.conserved_integrals()
        self.external_in = np.zeros(4)
        try:
            record = self.step()
        finally:
            external, self.external_in = self.external_in, None
        after = self.conserved_integrals()
        unit = self.fine_level.velocity_unit
        external[1:] *= unit
        impulse = record["wall_impulse"]
        mass_residual = after["mass"] - before["mass"] - external[0] - record["wall_mass"]
        momentum_residual = np.array(after["momentum"]) - before["momentum"] - external[1:] + impulse
        volume = (np.count_nonzero(self.coarse_owned) * self.coarse_level.dx ** 3
                  + np.count_nonzero(self.fine_fluid()) * self.fine_level.dx ** 3)
        record["budget"] = {"mass_residual_per_volume": float(mass_residual / volume),
                            "momentum_residual_per_volume": (momentum_residual / volume).tolist(),
                            "wall_mass_exchange": record["wall_mass"], "external_mass_in": float(external[0]),
                            "wall_impulse": impulse.tolist(), "external_impulse_in": external[1:].tolist()}
        return record

    # refined_solver.py:347-361 (the numeric part): leaf moments over owned
    # coarse cells and fine fluid cells
    def diagnostics(self):
        mach, density_error = 0.0, 0.0
        fine = self.fine.interior()[self.fine_slices].copy()
        fine[~self.fine_fluid()] = self.free_pdf
        for pdf, owned in ((self.coarse.interior(), self.coarse_owned), (fine, self.fine_fluid())):
            m = self.T.moments(pdf)
            rho = m[..., 0][owned]
            u = m[..., 1:4][owned] / rho[:, None]
            mach = max(mach, float(np.linalg.norm(u, axis=-1).max() * math.sqrt(3)))
            density_error = max(density_error, float(np.max(abs(rho - 1))))
        return {"local_mach_max": mach, "density_error_max": density_error}
