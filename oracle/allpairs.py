"""FP64 all-pairs reference of the rigid-molecule pair loop, written from the
textbook energies of Lennard-Jones centres, point dipoles and linear point
quadrupoles and differentiated by torch autograd (test infrastructure only:
used by tests/ as a second checker beside the C oracle, independent of both
the C oracle's and the engine's hand-written force expressions).

Conventions it reproduces (each pinned against the C oracle, which is pinned
against the reference itself):

- molecule pairs by minimum image of the centres, all site pairs of a pair
  counted when the centre distance is below rc (LJ centres: below rc_lj),
  the macroscopic rule of VectorizedCellProcessor::_calculatePairs
  (src/particleContainer/adapter/VectorizedCellProcessor.cpp:794-2730);
- site positions r + R(q) d and axes R(q) e with the normalised quaternion
  (FullMolecule::setupSoACache, src/molecules/FullMolecule.cpp:711-767);
- Lorentz-Berthelot mixing eps = xi sqrt(eps_a eps_b), sigma = eta (sigma_a +
  sigma_b) / 2 between components, xi = eta = 1 inside one, and every LJ
  pair of two different components shifted by 4 eps ((sigma/rc_lj)^6 -
  (sigma/rc_lj)^12) whether or not its centres are marked shifted
  (Comp2Param::initialize, src/molecules/Comp2Param.cpp:17-110);
- Upot = sum of the pair energies plus the reaction-field term
  -(2 (eps_RF - 1) / ((2 eps_RF + 1) rc^3)) mu_i mu_j e_i.e_j per dipole pair,
  virial = sum over site pairs of (R_i - R_j).f_site plus three times the
  reaction-field term (VectorizedCellProcessor::endTraversal, :122-155);
- the pair energies (d = r_i - r_j, r = |d|, c_i = e_i.d / r, c_ij = e_i.e_j):
  LJ 4 eps ((sigma/r)^12 - (sigma/r)^6); dipole-dipole mu_i mu_j / r^3
  (c_ij - 3 c_i c_j); dipole(i)-quadrupole(j) 3 mu Q / (2 r^4) (2 c_j c_ij -
  c_i (5 c_j^2 - 1)), the dipole in the field of the quadrupole's potential
  Q (3 c^2 - 1) / (2 r^3); quadrupole-quadrupole 3 Q_i Q_j / (4 r^5) (1 -
  5 c_i^2 - 5 c_j^2 - 15 c_i^2 c_j^2 + 2 (c_ij - 5 c_i c_j)^2).

Charges and shifted LJ centres are not covered (no system this reference
checks carries them).
"""
from __future__ import annotations

import numpy as np


def parameters(ps) -> np.ndarray:
    """Site parameters in the engine's adjoint order: components in order,
    each LJ centre (eps, sigma), each charge q, each dipole |mu|, each
    quadrupole |Q|."""
    vals = []
    for c in ps.components:
        for s in c.lj:
            vals += [s.eps, s.sigma]
        vals += [s.q for s in c.charges] + [s.abs for s in c.dipoles] + [s.abs for s in c.quadrupoles]
    return np.array(vals, dtype=np.float64)


def _group(mol, n):
    """(n, k) table of the site indices of each molecule, -1 where it has fewer."""
    counts = np.bincount(mol, minlength=n)
    k = int(counts.max()) if len(mol) else 0
    out = np.full((n, max(k, 1)), -1, np.int64)
    fill = np.zeros(n, np.int64)
    for s, m in enumerate(mol):
        out[m, fill[m]] = s
        fill[m] += 1
    return out


def _rotate(q, d):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    ww, xx, yy, zz = w * w, x * x, y * y, z * z
    wx, wy, wz, xy, xz, yz = w * x, w * y, w * z, x * y, x * z, y * z
    dx, dy, dz = d[:, 0], d[:, 1], d[:, 2]
    return np.stack([(ww + xx - yy - zz) * dx + 2 * (xy - wz) * dy + 2 * (wy + xz) * dz,
                     2 * (wz + xy) * dx + (ww - xx + yy - zz) * dy + 2 * (yz - wx) * dz,
                     2 * (xz - wy) * dx + 2 * (wx + yz) * dy + (ww - xx - yy + zz) * dz], axis=1)


class AllPairs:
    """All site pairs of one periodic box (minimum image, box edge > 2 rc)."""

    def __init__(self, ps, rc: float, rc_lj: float | None = None):
        import torch
        self.torch = torch
        self.ps = ps
        self.rc = float(rc)
        self.rc_lj = float(rc if rc_lj is None else rc_lj)
        box = np.asarray(ps.box, np.float64)
        if np.any(box <= 2 * self.rc):
            raise ValueError("minimum image needs a box edge above 2 rc")
        for c in ps.components:
            if c.charges or any(s.shifted for s in c.lj):
                raise ValueError("charges and shifted LJ centres are not covered")
        self.box = box
        self.eps_rf_inv_rc3 = 2.0 * (ps.eps_rf - 1.0) / (self.rc ** 3 * (2.0 * ps.eps_rf + 1.0))
        n = ps.n if hasattr(ps, "n") else len(ps.r)
        self.n = n
        r = np.mod(np.asarray(ps.r, np.float64), box)
        self.r0 = r
        q = np.asarray(ps.q, np.float64)
        q = q / np.sqrt((q * q).sum(1, keepdims=True))
        comp = np.asarray(ps.comp, np.int64)

        # parameter slots of every site of every component
        slot = 0
        per_comp = []
        for c in ps.components:
            lj, dip, quad = [], [], []
            for s in c.lj:
                lj.append((np.array(s.r, float), None, slot))
                slot += 2
            for s in c.dipoles:
                dip.append((np.array(s.r, float), np.array(s.e, float), slot))
                slot += 1
            for s in c.quadrupoles:
                quad.append((np.array(s.r, float), np.array(s.e, float), slot))
                slot += 1
            per_comp.append({"lj": lj, "dip": dip, "quad": quad})
        self.nparam = slot

        # lab-frame site tables: molecule, lab offset, lab axis, parameter slot, component
        self.sites = {}
        for kind in ("lj", "dip", "quad"):
            mol, off, ax, sl, cc = [], [], [], [], []
            for ci, pc in enumerate(per_comp):
                idx = np.nonzero(comp == ci)[0]
                for (d, e, s) in pc[kind]:
                    mol.append(idx)
                    off.append(_rotate(q[idx], np.broadcast_to(d, (len(idx), 3))))
                    ax.append(_rotate(q[idx], np.broadcast_to(e, (len(idx), 3))) if e is not None
                              else np.zeros((len(idx), 3)))
                    sl.append(np.full(len(idx), s))
                    cc.append(np.full(len(idx), ci))
            cat = (lambda a, k=0: np.concatenate(a) if a else np.zeros((0,) + ((3,) if k else ()),
                                                                      np.int64 if not k else np.float64))
            self.sites[kind] = dict(mol=cat(mol), off=cat(off, 1), ax=cat(ax, 1), slot=cat(sl), comp=cat(cc))

        # molecule pairs i < j within rc by minimum image: (i, j, image shift of j)
        I, J, S = [], [], []
        for i in range(n - 1):
            d = r[i] - r[i + 1:]
            sh = -box * np.round(d / box)
            dd = d + sh
            m = (dd * dd).sum(1) < self.rc * self.rc
            js = np.nonzero(m)[0] + i + 1
            I.append(np.full(len(js), i))
            J.append(js)
            S.append(sh[m])
        self.pi = np.concatenate(I)
        self.pj = np.concatenate(J)
        self.pshift = np.concatenate(S)   # added to r_i - r_j
        dcent = r[self.pi] - r[self.pj] + self.pshift
        self.plj = (dcent * dcent).sum(1) < self.rc_lj * self.rc_lj

        # LB mixing coefficients per component pair
        nc = len(ps.components)
        self.xi = np.ones((nc, nc))
        self.eta = np.ones((nc, nc))
        k = 0
        for a in range(nc):
            for b in range(a + 1, nc):
                xi, eta = ps.mixing[k]
                self.xi[a, b] = self.xi[b, a] = xi
                self.eta[a, b] = self.eta[b, a] = eta
                k += 1

        # site pairs of every kind over the molecule pairs
        self.sp = {}
        for ka, kb in (("lj", "lj"), ("dip", "dip"), ("dip", "quad"), ("quad", "dip"), ("quad", "quad")):
            A, B = self.sites[ka], self.sites[kb]
            if len(A["mol"]) == 0 or len(B["mol"]) == 0:
                continue
            mask = self.plj if ka == "lj" else np.ones(len(self.pi), bool)
            pidx = np.nonzero(mask)[0]
            ia, ib, pp = [], [], []
            bya = _group(A["mol"], n)
            byb = _group(B["mol"], n)
            for s_a in range(bya.shape[1]):
                sa = bya[self.pi[pidx], s_a]
                for s_b in range(byb.shape[1]):
                    sb = byb[self.pj[pidx], s_b]
                    ok = (sa >= 0) & (sb >= 0)
                    ia.append(sa[ok])
                    ib.append(sb[ok])
                    pp.append(pidx[ok])
            self.sp[(ka, kb)] = (np.concatenate(ia), np.concatenate(ib), np.concatenate(pp))

    def evaluate(self, R, theta, off=None, ax=None):
        """(U, W) as torch FP64 scalars on the graph of the molecule centres
        R (n x 3), the parameters theta and optionally the lab-frame site
        offsets and axes (dicts by kind, for torques)."""
        torch = self.torch
        T = lambda a: torch.as_tensor(a, dtype=torch.float64)
        if off is None:
            off = {k: T(v["off"]) for k, v in self.sites.items()}
        if ax is None:
            ax = {k: T(v["ax"]) for k, v in self.sites.items()}
        D = R[torch.as_tensor(self.pi)] - R[torch.as_tensor(self.pj)] + T(self.pshift)
        xi, eta = T(self.xi), T(self.eta)
        U = torch.zeros((), dtype=torch.float64)
        W = torch.zeros((), dtype=torch.float64)
        for (ka, kb), (ia, ib, pp) in self.sp.items():
            A, B = self.sites[ka], self.sites[kb]
            ia_t, ib_t, pp_t = (torch.as_tensor(x) for x in (ia, ib, pp))
            d = D[pp_t] + off[ka][ia_t] - off[kb][ib_t]
            u, urf = self._pair_energy(ka, kb, d, theta, torch.as_tensor(A["slot"][ia]),
                                       torch.as_tensor(B["slot"][ib]), torch.as_tensor(A["comp"][ia]),
                                       torch.as_tensor(B["comp"][ib]), xi, eta, ax[ka][ia_t], ax[kb][ib_t])
            # site force at fixed orientation; the virial pairs it with the centre difference
            f = -torch.autograd.grad(u.sum(), d, create_graph=True)[0]
            U = U + u.sum() + urf.sum()
            W = W + (D[pp_t] * f).sum() + 3.0 * urf.sum()
        return U, W

    def forces_torques(self):
        """(F, M, U, W) as numpy arrays / floats at the stored state."""
        torch = self.torch
        R = torch.tensor(self.r0, dtype=torch.float64, requires_grad=True)
        theta = torch.tensor(parameters(self.ps), dtype=torch.float64)
        off = {k: torch.tensor(v["off"], dtype=torch.float64, requires_grad=True) for k, v in self.sites.items()}
        ax = {k: torch.tensor(v["ax"], dtype=torch.float64, requires_grad=True) for k, v in self.sites.items()}
        U, W = self.evaluate(R, theta, off, ax)
        kinds = list(self.sites)
        g = torch.autograd.grad(U, [R] + [off[k] for k in kinds] + [ax[k] for k in kinds], allow_unused=True)
        F = -g[0].numpy()
        M = np.zeros((self.n, 3))
        for k, go, ga in zip(kinds, g[1:1 + len(kinds)], g[1 + len(kinds):]):
            tq = np.zeros((len(self.sites[k]["mol"]), 3))
            if go is not None:
                tq -= np.cross(self.sites[k]["off"], go.numpy())
            if ga is not None:
                tq -= np.cross(self.sites[k]["ax"], ga.numpy())
            np.add.at(M, self.sites[k]["mol"], tq)
        return F, M, U.item(), W.item()

    def _pair_energy(self, ka, kb, d, theta, sa, sb, ca, cb, xi, eta, ea, eb):
        """Per site pair energy (without the reaction field) and the
        reaction-field term of dipole pairs."""
        torch = self.torch
        r2 = (d * d).sum(1)
        zero = torch.zeros_like(r2)
        if ka == "lj":
            same = ca == cb
            x = torch.where(same, torch.ones_like(r2), xi[ca, cb])
            y = torch.where(same, torch.ones_like(r2), eta[ca, cb])
            eps = x * torch.sqrt(theta[sa] * theta[sb])
            sig = y * 0.5 * (theta[sa + 1] + theta[sb + 1])
            s6 = (sig * sig / r2) ** 3
            x = (sig * sig / (self.rc_lj * self.rc_lj)) ** 3
            shift = torch.where(same, zero, 4.0 * eps * (x - x * x))
            return 4.0 * eps * (s6 * s6 - s6) + shift, zero
        r = torch.sqrt(r2)
        n = d / r[:, None]
        ci = (ea * n).sum(1)
        cj = (eb * n).sum(1)
        cij = (ea * eb).sum(1)
        pa, pb = theta[sa], theta[sb]
        if ka == "dip" and kb == "dip":
            u = pa * pb / (r2 * r) * (cij - 3.0 * ci * cj)
            return u, -self.eps_rf_inv_rc3 * pa * pb * cij
        if ka == "dip" and kb == "quad":
            return 1.5 * pa * pb / (r2 * r2) * (2.0 * cj * cij - ci * (5.0 * cj * cj - 1.0)), zero
        if ka == "quad" and kb == "dip":
            # the dipole is site b: d points from the dipole to the quadrupole, so c flips sign
            return 1.5 * pa * pb / (r2 * r2) * (2.0 * (-ci) * cij - (-cj) * (5.0 * ci * ci - 1.0)), zero
        t = cij - 5.0 * ci * cj
        return 0.75 * pa * pb / (r2 * r2 * r) * (1.0 - 5.0 * ci * ci - 5.0 * cj * cj - 15.0 * ci * ci * cj * cj
                                                  + 2.0 * t * t), zero

    def gradients(self, gU: float, gW: float, gF=None):
        """(grad_r, grad_params, U, W) of the adjoint's objective: grad_r of
        gU U + gW W + sum gF.F over the molecule centres (orientations held
        fixed), grad_params of gU U + gW W over the site parameters."""
        torch = self.torch
        R = torch.tensor(self.r0, dtype=torch.float64, requires_grad=True)
        theta = torch.tensor(parameters(self.ps), dtype=torch.float64, requires_grad=True)
        U, W = self.evaluate(R, theta)
        Jp = gU * U + gW * W
        Jr = Jp
        if gF is not None:
            F = -torch.autograd.grad(U, R, create_graph=True)[0]
            Jr = Jr + (torch.as_tensor(gF, dtype=torch.float64) * F).sum()
        gp = torch.autograd.grad(Jp, theta, retain_graph=True)[0]
        gr = torch.autograd.grad(Jr, R)[0]
        return gr.numpy(), gp.numpy(), U.item(), W.item()
