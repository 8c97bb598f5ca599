"""FP64 reference of the differentiable FLIP rollout (TEST INFRASTRUCTURE ONLY).

The forward model is the per-substep core that libgfs runs on the GPU, written
in float64 torch so that torch's autograd gives the exact adjoint of it and
central finite differences of it are meaningful.  Only tests/ use it, as the
checker of the CUDA adjoint (gridfluidsim3d_gb300/csrc/adjoint.cu).

One substep, with the discrete structure (fluid cells, splat set masks, fill
contributors, extrapolation layers) taken from the state at the start of the
substep and held fixed, as the adjoint holds it:
  1. fluid cells = non-solid cells holding a particle
     (FluidSimulation::_updateFluidCells, fluidsimulation.cpp:1990-2041);
  2. P2G: per face component, u = sum w v / sum w over particles within dx of
     the face node, w = (1-s)^2 (1-4s/9), s = r^2/dx^2; set where sum w > 1e-9
     (_computeVelocityScalarField, fluidsimulation.cpp:2526-2595);
  3. faces bordering fluid take the splat value if set, else the mean of their
     qualifying 26 neighbours (U: nonzero value, V/W: set); others 0
     (_advectVelocityField, :2597-2736); saved = that field; gravity * dt is
     added on fluid-bordering faces (:2766-2805);
  4. the saved field is extrapolated over 7 layers (macvelocityfield.cpp:560-797);
  5. pressure: b = -div(u)/dx on fluid cells, A the 7-point matrix of
     _calculateMatrixCoefficients (pressuresolver.cpp:222-244) scaled by
     dt/(rho dx^2), p = A^-1 b (solved exactly); u -= dt/(rho dx) grad p on
     fluid-bordering faces, 0 on solid-bordering ones (fluidsimulation.cpp:2895-3061);
  6. the MAC field is extrapolated;
  7. v = 0.05 a + 0.95 (v + a - s), a / s = Catmull-Rom samples of MAC / saved
     at the particle (fluidsimulation.cpp:3104-3129, macvelocityfield.cpp:350-559);
  8. RK4 advection through MAC (particleadvector.cpp:1045-1054).
Collisions and the per-cell cap are not part of the differentiable model (the
scenes used keep particles away from solids and below the cap).

Initial particle velocities are the Catmull-Rom samples of the parameter MAC
field; the loss is sum (rho - target)^2 over cells, rho the cell-centred
particle density with the splat kernel of radius 1.5 dx.
"""
from __future__ import annotations

import numpy as np
import torch

AIR, FLUID, SOLID = 0, 1, 2
DENSITY_RADIUS = 1.5   # in cells


def face_shape(d, ni, nj, nk):
    return (nk + (d == 2), nj + (d == 1), ni + (d == 0))


class Structure:
    """Per-substep discrete structure, from a (detached) particle state."""

    def __init__(self, dims, dx, mat_solid, pos_np, layers=7):
        ni, nj, nk = dims
        self.dims, self.dx = dims, dx
        mat = mat_solid.copy()
        ijk = np.floor(pos_np / dx).astype(np.int64)
        ok = (ijk >= 0).all(1) & (ijk[:, 0] < ni) & (ijk[:, 1] < nj) & (ijk[:, 2] < nk)
        ijk = ijk[ok]
        sel = mat[ijk[:, 2], ijk[:, 1], ijk[:, 0]] != SOLID
        mat[ijk[sel, 2], ijk[sel, 1], ijk[sel, 0]] = FLUID
        self.mat = mat
        # extrapolation layers: BFS over non-solid cells (macvelocityfield.cpp:560-585)
        lay = np.where(mat == FLUID, 0, -1).astype(np.int64)
        for L in range(1, layers + 1):
            pad = np.pad(lay, 1, constant_values=-1)
            nb = np.zeros(lay.shape, bool)
            for ax in range(3):
                for sh in (-1, 1):
                    nb |= np.roll(pad, sh, axis=ax)[1:-1, 1:-1, 1:-1] == L - 1
            grow = (lay == -1) & (mat != SOLID) & nb
            lay[grow] = L
        self.layer = lay
        self.layers = layers

    def cell(self, grid, i, j, k, oob):
        ni, nj, nk = self.dims
        out = np.full(i.shape, oob, grid.dtype)
        m = (i >= 0) & (j >= 0) & (k >= 0) & (i < ni) & (j < nj) & (k < nk)
        out[m] = grid[k[m], j[m], i[m]]
        return out

    def borders(self, grid, d, value, oob):
        """FluidMaterialGrid::isFaceBorderingMaterialU/V/W (fluidmaterialgrid.cpp:119-143)
        over every face of component d: [t == n] lower cell, [0 < t < n] either, [t == 0] upper."""
        ni, nj, nk = self.dims
        sh = face_shape(d, ni, nj, nk)
        k, j, i = np.meshgrid(*[np.arange(n) for n in sh], indexing="ij")
        t = (i, j, k)[d]
        n = (ni, nj, nk)[d]
        lo = self.cell(grid, i - (d == 0), j - (d == 1), k - (d == 2), oob) == value
        hi = self.cell(grid, i, j, k, oob) == value
        return np.where(t == n, lo, np.where(t > 0, lo | hi, hi))


def _flat(sh, i, j, k):
    return i + sh[2] * (j + sh[1] * k)


def catmull_rom(x):
    x2, x3 = x * x, x * x * x
    return torch.stack([0.5 * (-x + 2 * x2 - x3), 0.5 * (2 - 5 * x2 + 3 * x3), 0.5 * (x + 4 * x2 - 3 * x3),
                        0.5 * (x3 - x2)], -1)


class Model:
    """The differentiable rollout on one grid (solid border walls)."""

    def __init__(self, dims, dx, dt, gravity=(0.0, 0.0, 0.0), density=20.0, ratio_pic=0.05, layers=7):
        self.dims, self.dx, self.dt = tuple(dims), float(dx), float(dt)
        self.g = [float(x) for x in gravity]
        self.rho, self.pic, self.layers = float(density), float(ratio_pic), layers
        ni, nj, nk = dims
        m = np.zeros((nk, nj, ni), np.uint8)
        m[0, :, :] = m[-1, :, :] = SOLID
        m[:, 0, :] = m[:, -1, :] = SOLID
        m[:, :, 0] = m[:, :, -1] = SOLID
        self.mat_solid = m

    # ---------------------------------------------------------- sampling
    def sample(self, fields, x):
        """MACVelocityField::evaluateVelocityAtPosition for every row of x (N, 3)."""
        ni, nj, nk = self.dims
        dx = self.dx
        inside = ((x >= 0).all(1) & (x[:, 0] < ni * dx) & (x[:, 1] < nj * dx) & (x[:, 2] < nk * dx))
        X = x / dx
        out = []
        for d in range(3):
            f = torch.nn.functional.pad(fields[d], (2, 2, 2, 2, 2, 2))
            q = X - 0.5 * torch.tensor([d != 0, d != 1, d != 2], dtype=x.dtype)
            base = torch.floor(q.detach())
            w = [catmull_rom(q[:, a] - base[:, a]) for a in range(3)]
            bi = base.long() + 1   # stencil starts at base - 1; +2 for the zero halo
            ii = bi[:, 0, None] + torch.arange(4)
            jj = bi[:, 1, None] + torch.arange(4)
            kk = bi[:, 2, None] + torch.arange(4)
            sh = f.shape
            ii = ii.clamp(0, sh[2] - 1)
            jj = jj.clamp(0, sh[1] - 1)
            kk = kk.clamp(0, sh[0] - 1)
            vals = f[kk[:, :, None, None], jj[:, None, :, None], ii[:, None, None, :]]   # (N, 4c, 4b, 4a)
            s = torch.einsum("nc,nb,na,ncba->n", w[2], w[1], w[0], vals)
            out.append(torch.where(inside, s, torch.zeros_like(s)))
        return torch.stack(out, 1)

    # ---------------------------------------------------------------- P2G
    def p2g(self, st, x, v, frozen_masks=None):
        ni, nj, nk = self.dims
        dx = self.dx
        out, masks = [], []
        for d in range(3):
            sh = face_shape(d, ni, nj, nk)
            off = torch.tensor([0.0 if d == 0 else 0.5, 0.0 if d == 1 else 0.5, 0.0 if d == 2 else 0.5],
                               dtype=x.dtype) * dx
            p = x - off
            c = torch.floor(p.detach() / dx).long()
            r = torch.arange(-1, 3)
            ii = (c[:, 0, None, None, None] + r[None, None, None, :]).expand(-1, 4, 4, 4)
            jj = (c[:, 1, None, None, None] + r[None, None, :, None]).expand(-1, 4, 4, 4)
            kk = (c[:, 2, None, None, None] + r[None, :, None, None]).expand(-1, 4, 4, 4)
            valid = (ii >= 0) & (jj >= 0) & (kk >= 0) & (ii < sh[2]) & (jj < sh[1]) & (kk < sh[0])
            gx = ii.to(x.dtype) * dx - p[:, 0, None, None, None]
            gy = jj.to(x.dtype) * dx - p[:, 1, None, None, None]
            gz = kk.to(x.dtype) * dx - p[:, 2, None, None, None]
            s = (gx * gx + gy * gy + gz * gz) / (dx * dx)
            inr = valid & (s.detach() < 1.0)
            w = torch.where(inr, (1 - s) ** 2 * (1 - 4.0 * s / 9.0), torch.zeros_like(s))
            idx = torch.where(inr, _flat(sh, ii, jj, kk), torch.zeros_like(ii)).reshape(-1)
            n = sh[0] * sh[1] * sh[2]
            S = torch.zeros(n, dtype=x.dtype).index_add(0, idx, (w * v[:, d, None, None, None]).reshape(-1))
            W = torch.zeros(n, dtype=x.dtype).index_add(0, idx, w.reshape(-1))
            m = W.detach() > 1e-9 if frozen_masks is None else torch.from_numpy(frozen_masks[d].reshape(-1))
            u = torch.where(m, S / torch.where(m, W, torch.ones_like(W)), torch.zeros_like(S))
            out.append(u.reshape(sh))
            masks.append(m.reshape(sh).numpy())
        return out, masks

    # --------------------------------------------------------------- fill
    def fill(self, st, u, masks, frozen_qual=None):
        ni, nj, nk = self.dims
        res = []
        for d in range(3):
            sh = face_shape(d, ni, nj, nk)
            bf = st.borders(st.mat, d, FLUID, SOLID)
            un = u[d].detach().numpy()
            qual = ((np.abs(un) > 0) if d == 0 else masks[d]) if frozen_qual is None else frozen_qual[d]
            self._qual.append(qual)
            target = bf & ~masks[d]
            fk, fj, fi = np.nonzero(target)
            srcs, dsts, wts = [], [], []
            for q in range(len(fk)):
                nbr = []
                for kk in (fk[q] - 1, fk[q], fk[q] + 1):
                    for jj in (fj[q] - 1, fj[q], fj[q] + 1):
                        for ii in (fi[q] - 1, fi[q], fi[q] + 1):
                            if (ii, jj, kk) == (fi[q], fj[q], fk[q]):
                                continue
                            if 0 <= ii < sh[2] and 0 <= jj < sh[1] and 0 <= kk < sh[0] and qual[kk, jj, ii]:
                                nbr.append(_flat(sh, ii, jj, kk))
                for nb in nbr:
                    srcs.append(nb)
                    dsts.append(_flat(sh, fi[q], fj[q], fk[q]))
                    wts.append(1.0 / len(nbr))
            flat = u[d].reshape(-1)
            keep = torch.from_numpy((bf & masks[d]).reshape(-1))
            out = torch.where(keep, flat, torch.zeros_like(flat))
            if srcs:
                out = out.index_add(0, torch.tensor(dsts), flat[torch.tensor(srcs)] * torch.tensor(wts, dtype=flat.dtype))
            res.append(out.reshape(sh))
        return res

    # -------------------------------------------------------- extrapolate
    def extrapolate(self, st, fields):
        ni, nj, nk = self.dims
        res = []
        for d in range(3):
            sh = face_shape(d, ni, nj, nk)
            solid = st.borders(st.mat, d, SOLID, SOLID)
            bl = [st.borders(st.layer, d, L, -1) for L in range(st.layers + 1)]
            flat = fields[d].reshape(-1)
            for L in range(1, st.layers + 1):
                tgt = bl[L] & ~bl[L - 1] & ~solid
                fk, fj, fi = np.nonzero(tgt)
                if len(fk) == 0:
                    continue
                srcs, dsts, wts, tgts = [], [], [], []
                for q in range(len(fk)):
                    nbr = []
                    for (a, b, c) in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
                        ii, jj, kk = fi[q] + a, fj[q] + b, fk[q] + c
                        if 0 <= ii < sh[2] and 0 <= jj < sh[1] and 0 <= kk < sh[0] and bl[L - 1][kk, jj, ii]:
                            nbr.append(_flat(sh, ii, jj, kk))
                    f = _flat(sh, fi[q], fj[q], fk[q])
                    tgts.append(f)
                    for nb in nbr:
                        srcs.append(nb)
                        dsts.append(f)
                        wts.append(1.0 / len(nbr))
                t = torch.tensor(tgts)
                keep = torch.ones_like(flat)
                keep[t] = 0.0
                new = flat * keep
                if srcs:
                    new = new.index_add(0, torch.tensor(dsts),
                                        flat[torch.tensor(srcs)] * torch.tensor(wts, dtype=flat.dtype))
                flat = new
            res.append(flat.reshape(sh))
        return res

    # ----------------------------------------------------------- pressure
    def project(self, st, u):
        ni, nj, nk = self.dims
        dx, dt, rho = self.dx, self.dt, self.rho
        mat = st.mat
        fl = np.argwhere(mat == FLUID)   # (k, j, i), lexicographic k -> j -> i
        F = len(fl)
        if F == 0:
            return u
        index = -np.ones(mat.shape, np.int64)
        index[fl[:, 0], fl[:, 1], fl[:, 2]] = np.arange(F)
        kk, jj, ii = fl[:, 0], fl[:, 1], fl[:, 2]
        uu, vv, ww = u
        div = (uu[kk, jj, ii + 1] - uu[kk, jj, ii] + vv[kk, jj + 1, ii] - vv[kk, jj, ii]
               + ww[kk + 1, jj, ii] - ww[kk, jj, ii])
        b = -div / dx
        # solid-neighbour corrections: the solid faces move with velocity 0
        def solid_at(a, b_, c):
            return st.cell(mat, a, b_, c, SOLID) == SOLID
        corr = [(solid_at(ii - 1, jj, kk), -uu[kk, jj, ii]), (solid_at(ii + 1, jj, kk), uu[kk, jj, ii + 1]),
                (solid_at(ii, jj - 1, kk), -vv[kk, jj, ii]), (solid_at(ii, jj + 1, kk), vv[kk, jj + 1, ii]),
                (solid_at(ii, jj, kk - 1), -ww[kk, jj, ii]), (solid_at(ii, jj, kk + 1), ww[kk + 1, jj, ii])]
        for m, val in corr:
            if m.any():
                b = b + torch.where(torch.from_numpy(m), val / dx, torch.zeros_like(val))
        scale = dt / (rho * dx * dx)
        A = np.zeros((F, F))
        for q, (k0, j0, i0) in enumerate(fl):
            diag = 0
            for (a, b_, c) in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
                m = st.cell(mat, np.array([i0 + a]), np.array([j0 + b_]), np.array([k0 + c]), SOLID)[0]
                if m != SOLID:
                    diag += 1
                if m == FLUID:
                    A[q, index[k0 + c, j0 + b_, i0 + a]] = -scale
            A[q, q] = diag * scale
        p = torch.linalg.solve(torch.from_numpy(A), b)
        P = torch.zeros(mat.shape, dtype=p.dtype)
        P = P.index_put((torch.from_numpy(kk), torch.from_numpy(jj), torch.from_numpy(ii)), p)
        out = []
        k_ = dt / (rho * dx)
        for d in range(3):
            sh = face_shape(d, ni, nj, nk)
            bf = torch.from_numpy(st.borders(mat, d, FLUID, SOLID))
            bs = torch.from_numpy(st.borders(mat, d, SOLID, SOLID))
            Pp = torch.nn.functional.pad(P, (1, 1, 1, 1, 1, 1))   # p = 0 outside the fluid set
            K, J, I = np.meshgrid(*[np.arange(n) for n in sh], indexing="ij")
            I1, J1, K1 = I + 1, J + 1, K + 1
            p1 = Pp[K1, J1, I1]
            p0 = Pp[K1 - (d == 2), J1 - (d == 1), I1 - (d == 0)]
            new = u[d] - k_ * (p1 - p0)
            out.append(torch.where(bf, torch.where(bs, torch.zeros_like(new), new), u[d]))
        return out

    # -------------------------------------------------------------- steps
    def substep(self, x, v, frozen=None):
        """One substep.  `frozen` = the (structure, set masks, fill qualifiers) of an
        earlier run of the same substep, to evaluate it with that discrete structure
        (finite differences of the structure-fixed map, the map the adjoint
        differentiates); the structure used is returned."""
        if frozen is None:
            st = Structure(self.dims, self.dx, self.mat_solid, x.detach().numpy(), self.layers)
            u, masks = self.p2g(st, x, v)
            self._qual = []
            filled = self.fill(st, u, masks)
        else:
            st, masks, qual = frozen
            u, _ = self.p2g(st, x, v, frozen_masks=masks)
            self._qual = []
            filled = self.fill(st, u, masks, frozen_qual=qual)
        used = (st, masks, list(self._qual))
        saved = filled
        mac = []
        for d in range(3):
            add = self.g[d] * self.dt
            if abs(self.g[d]) > 0:
                bf = torch.from_numpy(st.borders(st.mat, d, FLUID, SOLID))
                mac.append(torch.where(bf, filled[d] + add, filled[d]))
            else:
                mac.append(filled[d])
        saved = self.extrapolate(st, saved)
        mac = self.project(st, mac)
        mac = self.extrapolate(st, mac)
        a = self.sample(mac, x)
        s = self.sample(saved, x)
        vnew = self.pic * a + (1.0 - self.pic) * (v + a - s)
        dt = self.dt
        k1 = a
        k2 = self.sample(mac, x + 0.5 * dt * k1)
        k3 = self.sample(mac, x + 0.5 * dt * k2)
        k4 = self.sample(mac, x + dt * k3)
        xnew = x + dt / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)
        return xnew, vnew, used

    def density(self, x):
        """Cell-centred particle density, splat kernel of radius DENSITY_RADIUS cells."""
        ni, nj, nk = self.dims
        dx = self.dx
        R = DENSITY_RADIUS * dx
        c = torch.floor(x.detach() / dx - 0.5).long()
        r = torch.arange(-1, 3)
        ii = (c[:, 0, None, None, None] + r[None, None, None, :]).expand(-1, 4, 4, 4)
        jj = (c[:, 1, None, None, None] + r[None, None, :, None]).expand(-1, 4, 4, 4)
        kk = (c[:, 2, None, None, None] + r[None, :, None, None]).expand(-1, 4, 4, 4)
        valid = (ii >= 0) & (jj >= 0) & (kk >= 0) & (ii < ni) & (jj < nj) & (kk < nk)
        gx = (ii.to(x.dtype) + 0.5) * dx - x[:, 0, None, None, None]
        gy = (jj.to(x.dtype) + 0.5) * dx - x[:, 1, None, None, None]
        gz = (kk.to(x.dtype) + 0.5) * dx - x[:, 2, None, None, None]
        s = (gx * gx + gy * gy + gz * gz) / (R * R)
        inr = valid & (s.detach() < 1.0)
        w = torch.where(inr, (1 - s) ** 2 * (1 - 4.0 * s / 9.0), torch.zeros_like(s))
        idx = torch.where(inr, ii + ni * (jj + nj * kk), torch.zeros_like(ii)).reshape(-1)
        rho = torch.zeros(ni * nj * nk, dtype=x.dtype).index_add(0, idx, w.reshape(-1))
        return rho.reshape(nk, nj, ni)

    def run(self, x0, v0, nsteps, frozen=None):
        """Final density and the centroid at the start of every substep and at the end.
        The structures used are left in self.structures (pass them as `frozen`)."""
        x, v = x0, v0
        cents = [x.mean(0)]
        used = []
        for n in range(nsteps):
            x, v, st = self.substep(x, v, None if frozen is None else frozen[n])
            used.append(st)
            cents.append(x.mean(0))
        self.structures = used
        return self.density(x), torch.stack(cents), x, v

    def rollout(self, u0, x0, nsteps, target, frozen=None):
        """loss(u0) for particles starting at x0 with velocities sampled from u0."""
        rho, cents, x, v = self.run(x0, self.sample(u0, x0), nsteps, frozen)
        return ((rho - target) ** 2).sum(), x, v, rho


def gaussian_target(dims, dx, center_cells, sigma_cells, total):
    """Seeded-target helper: a Gaussian blob of cell-centred density summing to `total`."""
    ni, nj, nk = dims
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    c = np.asarray(center_cells, np.float64)
    r2 = (i + 0.5 - c[0]) ** 2 + (j + 0.5 - c[1]) ** 2 + (k + 0.5 - c[2]) ** 2
    g = np.exp(-r2 / (2.0 * sigma_cells ** 2))
    return g * (total / g.sum())
