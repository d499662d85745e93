"""Seeded test systems beyond the benchmark generators."""
import numpy as np

from ls1gb300 import phasespace as psm


def offcentre_mixture(cells: int = 7, density: float = 16.0, seed: int = 5) -> psm.PhaseSpace:
    """A two-component multipole mixture whose multipoles sit off the
    molecule centres: A = two LJ centres at -+0.1 nm and a dipole (1.5 D) at
    +0.05 nm on the axis; B = one LJ centre and a quadrupole (3.0 D*A, axis x)
    at 0.04 nm on x, with header inertia.  fcc sites jittered by 0.03 nm,
    uniform random orientations, 300 K velocities; eps_RF = 1e10."""
    D, DA = psm.DEBYE, psm.DEBYE_ANGSTROM
    a = psm.Component(lj=[psm.LJCenter((0.0, 0.0, -0.1), 14.0, 120.0, 0.31),
                          psm.LJCenter((0.0, 0.0, 0.1), 14.0, 120.0, 0.31)],
                      dipoles=[psm.Dipole((0.0, 0.0, 0.05), (0.0, 0.0, 1.0), 1.5 * D)])
    b = psm.Component(lj=[psm.LJCenter((0.0, 0.0, 0.0), 30.0, 150.0, 0.33)],
                      quadrupoles=[psm.Quadrupole((0.04, 0.0, 0.0), (1.0, 0.0, 0.0), 3.0 * DA)],
                      I_override=(0.04, 0.04, 0.04))
    n = 4 * cells ** 3
    lat = (4.0 / density) ** (1.0 / 3.0)
    box = np.full(3, cells * lat)
    rng = np.random.default_rng(seed)
    comps = [a, b]
    comp = np.zeros(n, np.int32)
    comp[rng.permutation(n)[: n // 2]] = 1
    r = np.mod(psm.fcc_positions((cells, cells, cells), lat) + rng.uniform(-0.03, 0.03, (n, 3)), box)
    masses = np.array([c.mass_inertia()[0] for c in comps])
    v = psm.maxwell_boltzmann(rng, n, masses[comp], 300.0)
    q = psm.random_quaternions(rng, n)
    return psm.PhaseSpace(box, comps, [(1.0, 1.0)], 1.0e10, np.arange(1, n + 1, dtype=np.uint64), comp, r, v, q,
                          np.zeros((n, 3)), 300.0)
