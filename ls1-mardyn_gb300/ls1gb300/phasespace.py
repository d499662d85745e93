"""Phase-space model, ASCII ``.inp`` reader/writer and seeded generators.

This mirrors the host-side data the reference keeps for the short-range path:
component definitions (LJ centres, charges, dipoles, quadrupoles, inertia),
Lorentz-Berthelot mixing coefficients, the reaction-field permittivity and the
per-molecule state (id, component, r, v, q, L).

Format followed: ``ASCIIReader::readPhaseSpaceHeader`` / ``readPhaseSpace``
(src/io/ASCIIReader.cpp:60-260, 260-420): ``mardyn trunk <version>`` line,
header tokens (``currentTime``, ``Temperature``, ``Length``,
``NumberOfComponents`` + component blocks + mixing ``xi eta`` pairs + epsilon_RF),
then ``NumberOfMolecules``, ``MoleculeFormat`` (ICRVQD, ICRVQDV, ICRV, IRV) and
one line per molecule.

Mass/inertia rules follow ``Component::updateMassInertia``
(src/molecules/Component.cpp:137-178): only LJ centres and charges carry mass;
the principal moments come from the site offsets; a positive inertia given in
the header overrides the computed one (src/io/ASCIIReader.cpp, ``IDummy``) but
leaves the rotational degrees of freedom as computed from the sites.
The LJ shift of a centre is ``24 eps ((s/rc)^6 - (s/rc)^12)`` with the
centre's own truncation radius when shifting is requested
(src/molecules/Component.cpp:105-123).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np


@dataclass
class LJCenter:
    r: Tuple[float, float, float]
    m: float
    eps: float
    sigma: float
    tcutoff: float = 0.0
    shifted: bool = False

    @property
    def shift6(self) -> float:
        if not self.shifted:
            return 0.0
        sp2 = self.sigma * self.sigma / (self.tcutoff * self.tcutoff)
        sp6 = sp2 * sp2 * sp2
        return 24.0 * self.eps * (sp6 - sp6 * sp6)


@dataclass
class Charge:
    r: Tuple[float, float, float]
    m: float
    q: float


@dataclass
class Dipole:
    r: Tuple[float, float, float]
    e: Tuple[float, float, float]
    abs: float


@dataclass
class Quadrupole:
    r: Tuple[float, float, float]
    e: Tuple[float, float, float]
    abs: float


@dataclass
class Component:
    lj: List[LJCenter] = field(default_factory=list)
    charges: List[Charge] = field(default_factory=list)
    dipoles: List[Dipole] = field(default_factory=list)
    quadrupoles: List[Quadrupole] = field(default_factory=list)
    I_override: Tuple[float, float, float] = (0.0, 0.0, 0.0)

    def mass_inertia(self) -> Tuple[float, np.ndarray, int]:
        """(mass, principal moments, rotational degrees of freedom)."""
        m = 0.0
        I = [0.0, 0.0, 0.0]
        rot_dof = 0
        for s in list(self.lj) + list(self.charges):
            x, y, z = s.r
            m += s.m
            I[0] += s.m * (y * y + z * z)
            I[1] += s.m * (x * x + z * z)
            I[2] += s.m * (x * x + y * y)
            rot_dof = 3 - sum(1 for d in range(3) if I[d] == 0.0)
        for d in range(3):
            if self.I_override[d] > 0.0:
                I[d] = self.I_override[d]
        return m, np.array(I), rot_dof


@dataclass
class PhaseSpace:
    box: np.ndarray                       # (3,) box lengths; the box is [0, L)
    components: List[Component]
    mixing: List[Tuple[float, float]]     # (xi, eta) for i<j pairs in row order
    eps_rf: float
    ids: np.ndarray                       # (N,) uint64
    comp: np.ndarray                      # (N,) int32, 0-based
    r: np.ndarray                         # (N,3) float64
    v: np.ndarray                         # (N,3)
    q: np.ndarray                         # (N,4) w,x,y,z
    L: np.ndarray                         # (N,3) angular momentum
    temperature: float = 1.0
    time: float = 0.0

    @property
    def n(self) -> int:
        return int(self.r.shape[0])

    def copy(self) -> "PhaseSpace":
        return PhaseSpace(self.box.copy(), self.components, list(self.mixing), self.eps_rf,
                          self.ids.copy(), self.comp.copy(), self.r.copy(), self.v.copy(),
                          self.q.copy(), self.L.copy(), self.temperature, self.time)


def _fmt(x: float) -> str:
    return repr(float(x))


def write_inp(ps: PhaseSpace, path: str) -> None:
    """Write ``ps`` in the ICRVQD ASCII format the reference reads."""
    out = ["mardyn trunk 20120726",
           f" currentTime\t{_fmt(ps.time)}",
           f" Length\t{_fmt(ps.box[0])} {_fmt(ps.box[1])} {_fmt(ps.box[2])}",
           f" Temperature\t{_fmt(ps.temperature)}",
           f" NumberOfComponents\t{len(ps.components)}"]
    for c in ps.components:
        out.append(f"{len(c.lj)}\t{len(c.charges)}\t{len(c.dipoles)}\t{len(c.quadrupoles)}\t0")
        for s in c.lj:
            out.append(" ".join(_fmt(x) for x in s.r) + f"\t{_fmt(s.m)}\t{_fmt(s.eps)} {_fmt(s.sigma)} "
                       f"{_fmt(s.tcutoff)} {1 if s.shifted else 0}")
        for s in c.charges:
            out.append(" ".join(_fmt(x) for x in s.r) + f"\t{_fmt(s.m)} {_fmt(s.q)}")
        for s in list(c.dipoles) + list(c.quadrupoles):
            out.append(" ".join(_fmt(x) for x in s.r) + "\t" + " ".join(_fmt(x) for x in s.e) + f" {_fmt(s.abs)}")
        out.append(" ".join(_fmt(x) for x in c.I_override))
    for xi, eta in ps.mixing:
        out.append(f"{_fmt(xi)} {_fmt(eta)}")
    out.append(_fmt(ps.eps_rf))
    out.append(f" NumberOfMolecules\t{ps.n}")
    out.append(" MoleculeFormat\tICRVQD")
    rows = np.concatenate([ps.r, ps.v, ps.q, ps.L], axis=1)
    for k in range(ps.n):
        out.append(f"{int(ps.ids[k])}\t{int(ps.comp[k]) + 1}\t" + " ".join(_fmt(x) for x in rows[k]))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


class _Tokens:
    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.toks: List[str] = []
        for line in self.lines[1:]:
            if line.lstrip().startswith("#"):
                continue
            self.toks.extend(line.split())
        self.pos = 0

    def next(self) -> str:
        t = self.toks[self.pos]
        self.pos += 1
        return t

    def f(self) -> float:
        return float(self.next())

    def i(self) -> int:
        return int(self.next())


def read_inp(path: str) -> PhaseSpace:
    """Read an ASCII phase-space file (header and molecules in one file)."""
    with open(path) as f:
        text = f.read()
    first = text.splitlines()[0].split()
    if len(first) < 3 or first[1] != "trunk":
        raise ValueError(f"{path}: not a mardyn input file")
    t = _Tokens(text)
    box = np.zeros(3)
    temperature, time = 1.0, 0.0
    comps: List[Component] = []
    mixing: List[Tuple[float, float]] = []
    eps_rf = 1.0
    while True:
        tok = t.next()
        if tok in ("currentTime", "t"):
            time = t.f()
        elif tok in ("Temperature", "T"):
            temperature = t.f()
        elif tok in ("Length", "L"):
            box = np.array([t.f(), t.f(), t.f()])
        elif tok in ("NumberOfComponents", "C"):
            nc = t.i()
            for _ in range(nc):
                nlj, nch, ndi, nqu, nte = (t.i() for _ in range(5))
                if nte != 0:
                    raise ValueError("tersoff sites are not supported")
                c = Component()
                for _ in range(nlj):
                    x, y, z, m, eps, sig, tcut, shift = (t.f() for _ in range(8))
                    c.lj.append(LJCenter((x, y, z), m, eps, sig, tcut, shift != 0))
                for _ in range(nch):
                    x, y, z, m, q = (t.f() for _ in range(5))
                    c.charges.append(Charge((x, y, z), m, q))
                for _ in range(ndi):
                    x, y, z, ex, ey, ez, a = (t.f() for _ in range(7))
                    c.dipoles.append(Dipole((x, y, z), (ex, ey, ez), a))
                for _ in range(nqu):
                    x, y, z, ex, ey, ez, a = (t.f() for _ in range(7))
                    c.quadrupoles.append(Quadrupole((x, y, z), (ex, ey, ez), a))
                c.I_override = (t.f(), t.f(), t.f())
                comps.append(c)
            for _ in range(nc * (nc - 1) // 2):
                mixing.append((t.f(), t.f()))
            eps_rf = t.f()
            break
        else:
            raise ValueError(f"{path}: unexpected header token {tok!r}")
    while t.next() not in ("NumberOfMolecules", "N"):
        pass
    n = t.i()
    fmt = "ICRVQD"
    if t.toks[t.pos] in ("MoleculeFormat", "M"):
        t.next()
        fmt = t.next()
    ncol = {"ICRVQDV": 18, "ICRVQD": 15, "ICRV": 8, "IRV": 7}[fmt]
    data = np.array(t.toks[t.pos:t.pos + n * ncol], dtype=np.float64).reshape(n, ncol)
    ids = data[:, 0].astype(np.uint64)
    if fmt == "IRV":
        comp = np.zeros(n, np.int32)
        rest = data[:, 1:]
    else:
        comp = data[:, 1].astype(np.int32) - 1
        rest = data[:, 2:]
    r = rest[:, 0:3].copy()
    v = rest[:, 3:6].copy()
    q = np.zeros((n, 4))
    q[:, 0] = 1.0
    L = np.zeros((n, 3))
    if fmt in ("ICRVQD", "ICRVQDV"):
        q = rest[:, 6:10].copy()
        L = rest[:, 10:13].copy()
    return PhaseSpace(box, comps, mixing, eps_rf, ids, comp, r, v, q, L, temperature, time)


# ---------------------------------------------------------------------------
# Seeded generators for the benchmark workloads (synthetic, no dataset).
# ---------------------------------------------------------------------------

def one_center_lj(eps: float = 1.0, sigma: float = 1.0, m: float = 1.0,
                  shifted: bool = False, rc: float = 0.0) -> Component:
    return Component(lj=[LJCenter((0.0, 0.0, 0.0), m, eps, sigma, rc, shifted)])


def fcc_positions(cells: Sequence[int], a: float, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """fcc lattice with ``cells`` unit cells of edge ``a``; 4 sites per cell,
    offset by a/4 so no site lies on a cell border."""
    nx, ny, nz = cells
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]) + 0.25
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    corners = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    pos = (corners[:, None, :] + base[None, :, :]).reshape(-1, 3) * a
    return pos + np.asarray(origin, dtype=np.float64)


def maxwell_boltzmann(rng: np.random.Generator, n: int, mass: np.ndarray, T: float) -> np.ndarray:
    """Velocities at temperature T with the net momentum removed."""
    v = rng.normal(size=(n, 3)) * np.sqrt(T / mass)[:, None]
    p = (v * mass[:, None]).sum(axis=0) / mass.sum()
    return v - p[None, :]


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random unit quaternions (Shoemake's method), w first."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    return q[:, [3, 0, 1, 2]]


def lj_fcc(cells: int, rho: float, T: float, seed: int, shifted: bool = False, rc: float = 2.5) -> PhaseSpace:
    """Single-centre LJ (eps = sigma = m = 1) fcc crystal at reduced density rho."""
    n = 4 * cells ** 3
    a = (4.0 / rho) ** (1.0 / 3.0)
    box = np.full(3, cells * a)
    rng = np.random.default_rng(seed)
    r = fcc_positions((cells, cells, cells), a)
    v = maxwell_boltzmann(rng, n, np.ones(n), T)
    q = np.zeros((n, 4)); q[:, 0] = 1.0
    return PhaseSpace(box, [one_center_lj(shifted=shifted, rc=rc)], [], 1.0e10,
                      np.arange(1, n + 1, dtype=np.uint64), np.zeros(n, np.int32), r, v, q,
                      np.zeros((n, 3)), T)


def with_vacancies(ps: PhaseSpace, n: int, density: float, seed: int) -> PhaseSpace:
    """Exactly ``n`` molecules of a lattice state at number density
    ``density``: a seeded random choice of n of its molecules (order kept,
    ids renumbered 1..n), box and positions scaled so that n / V = density,
    and the net momentum of the kept molecules removed again."""
    if not 0 < n <= ps.n:
        raise ValueError("n must lie in (0, ps.n]")
    keep = np.sort(np.random.default_rng(seed).choice(ps.n, n, replace=False))
    q = ps.copy()
    s = (n / density / float(np.prod(ps.box))) ** (1.0 / 3.0)
    q.box = np.asarray(ps.box, np.float64) * s
    q.r = ps.r[keep] * s
    q.comp = ps.comp[keep].copy()
    masses = np.array([c.mass_inertia()[0] for c in ps.components])[q.comp]
    v = ps.v[keep]
    q.v = v - ((v * masses[:, None]).sum(axis=0) / masses.sum())[None, :]
    q.q, q.L = ps.q[keep].copy(), ps.L[keep].copy()
    q.ids = np.arange(1, n + 1, dtype=np.uint64)
    return q


def lj_slab(cells_xy: int, rho_liq: float, rho_vap: float, T: float, seed: int,
            elongation: float = 3.0) -> PhaseSpace:
    """Vapour-liquid slab: an fcc liquid at rho_liq filling the middle third of
    a box elongated along z (height = Lx), and vapour at rho_vap in the outer
    thirds on a jittered simple-cubic lattice (so no vapour pair overlaps)."""
    a = (4.0 / rho_liq) ** (1.0 / 3.0)
    lx = cells_xy * a
    lz = elongation * lx
    h = (lz - lx) / 2.0                        # height of each vapour region
    liq = fcc_positions((cells_xy, cells_xy, cells_xy), a, origin=(0.0, 0.0, h))
    rng = np.random.default_rng(seed)
    s = rho_vap ** (-1.0 / 3.0)
    nvx, nvz = max(1, int(round(lx / s))), max(1, int(round(h / s)))
    sx, sz = lx / nvx, h / nvz
    ix, iy, iz = np.meshgrid(np.arange(nvx), np.arange(nvx), np.arange(nvz), indexing="ij")
    lat = np.stack([(ix.ravel() + 0.5) * sx, (iy.ravel() + 0.5) * sx, (iz.ravel() + 0.5) * sz], axis=1)
    lo = lat + rng.uniform(-0.2, 0.2, lat.shape) * np.array([sx, sx, sz])
    hi = lat + rng.uniform(-0.2, 0.2, lat.shape) * np.array([sx, sx, sz])
    hi[:, 2] += h + lx
    r = np.concatenate([liq, lo, hi])
    n = r.shape[0]
    v = maxwell_boltzmann(rng, n, np.ones(n), T)
    q = np.zeros((n, 4)); q[:, 0] = 1.0
    return PhaseSpace(np.array([lx, lx, lz]), [one_center_lj()], [], 1.0e10,
                      np.arange(1, n + 1, dtype=np.uint64), np.zeros(n, np.int32), r, v, q,
                      np.zeros((n, 3)), T)


def lj_on_cell_borders(box: float, rc: float, seed: int) -> PhaseSpace:
    """1CLJ molecules on a simple-cubic lattice of spacing cellLength/2, so
    that half of all coordinates lie exactly on linked-cell borders (as the
    border table computes them) or one ulp beside them; includes coordinates
    0.0 and the last representable value below the box edge."""
    n_cells = int(np.floor(box / rc))
    cl = box / n_cells
    rng = np.random.default_rng(seed)
    coords = []
    for k in range(2 * n_cells):
        if k % 2 == 0:
            x = (k // 2 + 1) * cl + (0.0 - cl)          # reference border expression
        else:
            x = (k / 2.0) * cl
        coords.append(x)
    coords = np.array(coords)
    g = np.stack(np.meshgrid(coords, coords, coords, indexing="ij"), axis=-1).reshape(-1, 3)
    # nudge a few coordinates one ulp to either side of a border
    sel = rng.random(g.shape) < 0.15
    g = np.where(sel & (rng.random(g.shape) < 0.5), np.nextafter(g, np.inf), g)
    g = np.where(sel & (rng.random(g.shape) < 0.5), np.nextafter(g, -np.inf), g)
    g = np.clip(g, 0.0, np.nextafter(box, 0.0))
    n = g.shape[0]
    v = maxwell_boltzmann(rng, n, np.ones(n), 0.5)
    q = np.zeros((n, 4)); q[:, 0] = 1.0
    return PhaseSpace(np.full(3, box), [one_center_lj()], [], 1.0e10,
                      np.arange(1, n + 1, dtype=np.uint64), np.zeros(n, np.int32), g, v, q,
                      np.zeros((n, 3)), 0.5)


# Unit system of the multi-centre mixture: length nm, energy K (k_B = 1),
# mass u, charge-free multipoles with 1/(4 pi eps0) = 1.  One debye is
# sqrt(7.2429 K nm^3); one D*Angstrom is sqrt(0.072429 K nm^5).
DEBYE = math.sqrt(7.242971e0)
DEBYE_ANGSTROM = math.sqrt(7.242971e-2)


def mixture_components(mass_a_site: float = 14.0, mass_b: float = 30.0,
                       inertia_b: Tuple[float, float, float] = (0.04, 0.04, 0.0)) -> List[Component]:
    """2CLJQ (A) + 1CLJD (B) in nm / K / u units.

    A: two LJ centres at +-0.12 nm on the z axis (eps/k = 133 K, sigma =
    0.30 nm, mass ``mass_a_site`` u each) and a point quadrupole of 3.8 D*A
    along z at the centre.  B: one LJ centre (eps/k = 160 K, sigma = 0.34 nm,
    mass ``mass_b`` u) and a point dipole of 1.8 D along z; a single centred
    mass has no inertia, so B is given ``inertia_b`` (u nm^2) to let its
    dipole rotate.
    """
    a = Component(lj=[LJCenter((0.0, 0.0, -0.12), mass_a_site, 133.0, 0.30),
                      LJCenter((0.0, 0.0, 0.12), mass_a_site, 133.0, 0.30)],
                  quadrupoles=[Quadrupole((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 3.8 * DEBYE_ANGSTROM)])
    b = Component(lj=[LJCenter((0.0, 0.0, 0.0), mass_b, 160.0, 0.34)],
                  dipoles=[Dipole((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 1.8 * DEBYE)],
                  I_override=inertia_b)
    return [a, b]


def mixture(n_target: int, density: float, T: float, seed: int, eps_rf: float = 1.0e10) -> PhaseSpace:
    """50/50 A/B mixture on an fcc lattice at number density ``density``
    (nm^-3), uniform random orientations and Maxwell-Boltzmann velocities and
    angular momenta at temperature T (K)."""
    cells = max(2, int(round((n_target / 4) ** (1.0 / 3.0))))
    n = 4 * cells ** 3
    a = (4.0 / density) ** (1.0 / 3.0)
    box = np.full(3, cells * a)
    rng = np.random.default_rng(seed)
    comps = mixture_components()
    comp = np.zeros(n, np.int32)
    comp[rng.permutation(n)[: n // 2]] = 1
    masses = np.array([c.mass_inertia()[0] for c in comps])
    inert = np.array([c.mass_inertia()[1] for c in comps])
    r = fcc_positions((cells, cells, cells), a)
    v = maxwell_boltzmann(rng, n, masses[comp], T)
    q = random_quaternions(rng, n)
    # body-frame angular velocity ~ N(0, T/I), L = R(q) I w (zero along axes with I = 0)
    I = inert[comp]
    w = rng.normal(size=(n, 3)) * np.sqrt(np.where(I > 0, T / np.where(I > 0, I, 1.0), 0.0))
    Lb = I * w
    L = rotate(q, Lb)
    return PhaseSpace(box, comps, [(1.0, 1.0)], eps_rf, np.arange(1, n + 1, dtype=np.uint64),
                      comp, r, v, q, L, T)


def rotate(q: np.ndarray, d: np.ndarray) -> np.ndarray:
    """Rotate body-frame vectors by unit quaternions (Quaternion::rotate,
    src/molecules/Quaternion.cpp:43-64)."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    ww, xx, yy, zz = w * w, x * x, y * y, z * z
    wx, wy, wz, xy, xz, yz = w * x, w * y, w * z, x * y, x * z, y * z
    dx, dy, dz = d[:, 0], d[:, 1], d[:, 2]
    return np.stack([(ww + xx - yy - zz) * dx + 2 * (xy - wz) * dy + 2 * (wy + xz) * dz,
                     2 * (wz + xy) * dx + (ww - xx + yy - zz) * dy + 2 * (yz - wx) * dz,
                     2 * (xz - wy) * dx + 2 * (wx + yz) * dy + (ww - xx - yy + zz) * dz], axis=1)
