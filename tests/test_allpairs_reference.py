"""The FP64 all-pairs torch reference (oracle/allpairs.py), written from the
textbook LJ, dipole and quadrupole energies, against the C oracle: forces,
torques, Upot and virial on the 1CLJ box and the 2CLJQ + 1CLJD mixture, its
parameter gradients (eps, sigma, |mu|, |Q|) against central differences of
the oracle's forward and its Hessian-vector product against central
differences of the oracle's forces.  This pins the reference the adjoint's
GPU tests compare with."""
import copy
import os

import numpy as np
import pytest

from ls1gb300 import phasespace as psm

torch = pytest.importorskip("torch")

from oracle.allpairs import AllPairs, parameters  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

THREADS = min(os.cpu_count() or 1, 8)


def systems(name):
    if name == "lj":
        ps = psm.lj_fcc(5, 0.7, 1.1, seed=3)
        ps.r = ps.r + np.random.default_rng(3).uniform(-0.15, 0.15, ps.r.shape)
        return ps, 2.5
    if name == "offcentre":
        from systems import offcentre_mixture
        return offcentre_mixture(), 1.0
    return psm.mixture(2000, 14.0, 300.0, seed=4), 1.0


def set_param(ps, k, value):
    ps = copy.deepcopy(ps)
    slot = 0
    for c in ps.components:
        for s in c.lj:
            if slot == k:
                s.eps = value
            if slot + 1 == k:
                s.sigma = value
            slot += 2
        for group, attr in ((c.charges, "q"), (c.dipoles, "abs"), (c.quadrupoles, "abs")):
            for s in group:
                if slot == k:
                    setattr(s, attr, value)
                slot += 1
    return ps


def oracle_state(ps, rc):
    o = Oracle(ps, rc, threads=THREADS)
    o.rebin()
    fo, _ = o.forces()
    m = o.molecules()
    order = np.argsort(m["ids"])          # ids are 1..n in phase-space order
    return fo.upot, fo.virial, m["F"][order], m["M"][order]


@pytest.mark.parametrize("name", ["lj", "mixture", "offcentre"])
def test_allpairs_matches_the_oracle(name):
    ps, rc = systems(name)
    F, M, U, W = AllPairs(ps, rc).forces_torques()
    Uo, Wo, Fo, Mo = oracle_state(ps, rc)
    assert abs(U - Uo) <= 1e-12 * abs(Uo)
    assert abs(W - Wo) <= 1e-12 * abs(Wo)
    assert np.abs(F - Fo).max() <= 1e-12 * np.abs(Fo).max()
    if name != "lj":
        assert np.abs(M - Mo).max() <= 1e-12 * np.abs(Mo).max()


@pytest.mark.parametrize("name", ["lj", "mixture", "offcentre"])
def test_allpairs_parameter_gradients_vs_oracle_finite_differences(name):
    """Central differences with h = 1e-5 |p|: 5e-8 relative plus the
    differences' own rounding, 1e-9 (|U| + |W|) / |p|."""
    ps, rc = systems(name)
    ap = AllPairs(ps, rc)
    _, gpU, U0, W0 = ap.gradients(1.0, 0.0)
    _, gpW, _, _ = ap.gradients(0.0, 1.0)
    th = parameters(ps)
    for k in range(len(th)):
        h = 1e-5 * abs(th[k])
        Up, Wp, _, _ = oracle_state(set_param(ps, k, th[k] + h), rc)
        Um, Wm, _, _ = oracle_state(set_param(ps, k, th[k] - h), rc)
        fu, fw = (Up - Um) / (2 * h), (Wp - Wm) / (2 * h)
        noise = 1e-9 * (abs(U0) + abs(W0)) / abs(th[k])  # rounding of the differences
        assert abs(gpU[k] - fu) <= 5e-8 * abs(fu) + noise, (k, gpU[k], fu)
        assert abs(gpW[k] - fw) <= 5e-8 * abs(fw) + noise, (k, gpW[k], fw)


def test_allpairs_hessian_vector_product_vs_oracle_finite_differences():
    """d/dr of gU U + gW W + sum gF.F on the mixture against central
    differences of the oracle's Upot, virial and forces."""
    ps, rc = systems("mixture")
    rng = np.random.default_rng(12)
    gF = rng.normal(size=(ps.n, 3))
    gU, gW = 0.3, -0.2
    gr, _, _, _ = AllPairs(ps, rc).gradients(gU, gW, gF)

    def objective(r):
        q = ps.copy()
        q.r = r
        U, W, F, _ = oracle_state(q, rc)
        return gU * U + gW * W + (gF * F).sum()

    for i in rng.choice(ps.n, 3, replace=False):
        for c in range(3):
            h = 1e-6
            rp, rm = ps.r.copy(), ps.r.copy()
            rp[i, c] += h
            rm[i, c] -= h
            fd = (objective(rp) - objective(rm)) / (2 * h)
            assert abs(gr[i, c] - fd) <= 2e-7 * max(abs(fd), 1e-3 * np.abs(gr).max()), (i, c, gr[i, c], fd)
