"""Adjoint of the force field (md_adjoint) against FP64 central finite
differences of the C oracle's forward (the restatement pinned against the
reference) and of the engine's own FP64 forward, against FP64 all-pairs torch
references (1CLJ here; the 2CLJQ + 1CLJD mixture through oracle/allpairs.py,
written from the textbook multipole energies), and through a
torch.autograd.Function used only here (validation harness).  Tolerances:
parameter and position gradients 1e-6 relative to the largest component
(FP64 adjoint) unless stated, 2e-4 (FP32 pair arithmetic, FP64 sums)."""
import copy
import os

import numpy as np
import pytest

from ls1gb300 import phasespace as psm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import importlib, os, sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "ls1-mardyn_gb300"))
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


def lj_box(n_cells=5, rho=0.7, seed=3):
    ps = psm.lj_fcc(n_cells, rho, 1.1, seed=seed)
    ps.r = ps.r + np.random.default_rng(seed).uniform(-0.15, 0.15, ps.r.shape)
    return ps


def forward(E, ps, rc, precision="fp64"):
    e = E.Engine(ps, rc, precision=precision)
    fo = e.forces()
    return e, fo.upot, fo.virial


def set_param(ps, k, value):
    """Set parameter k in md_adjoint's order (components, sites LJ/C/D/Q)."""
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


def get_param(ps, k):
    vals = []
    for c in ps.components:
        for s in c.lj:
            vals += [s.eps, s.sigma]
        vals += [s.q for s in c.charges] + [s.abs for s in c.dipoles] + [s.abs for s in c.quadrupoles]
    return vals[k]


@pytest.mark.parametrize("gU,gW", [(1.0, 0.0), (0.0, 1.0), (0.7, -0.3)])
def test_lj_parameter_gradients_vs_finite_differences(E, gU, gW):
    ps = lj_box()
    e, U, W = forward(E, ps, 2.5)
    _, gp = e.adjoint(gU, gW)
    for k in range(2):
        p0 = get_param(ps, k)
        h = 1e-6 * p0
        _, Up, Wp = forward(E, set_param(ps, k, p0 + h), 2.5)
        _, Um, Wm = forward(E, set_param(ps, k, p0 - h), 2.5)
        fd = gU * (Up - Um) / (2 * h) + gW * (Wp - Wm) / (2 * h)
        assert abs(gp[k] - fd) <= 1e-6 * max(abs(fd), 1.0), (k, gp[k], fd)


def test_lj_position_gradient_and_hvp_vs_finite_differences(E):
    ps = lj_box(4)
    rng = np.random.default_rng(5)
    gF = rng.normal(size=(ps.n, 3))
    gU, gW = 0.4, 0.9
    e, U, W = forward(E, ps, 2.5)
    F = e.molecules()["F"]
    gr, _ = e.adjoint(gU, gW, gF)

    def objective(r):
        q = ps.copy()
        q.r = r
        e2, U2, W2 = forward(E, q, 2.5)
        return gU * U2 + gW * W2 + (gF * e2.molecules()["F"]).sum()

    for i in rng.choice(ps.n, 6, replace=False):
        for c in range(3):
            h = 1e-6
            rp, rm = ps.r.copy(), ps.r.copy()
            rp[i, c] += h
            rm[i, c] -= h
            fd = (objective(rp) - objective(rm)) / (2 * h)
            assert abs(gr[i, c] - fd) <= 1e-5 * max(abs(fd), 1.0), (i, c, gr[i, c], fd)
    # dU/dr = -F
    e2, _, _ = forward(E, ps, 2.5)
    gr_u, _ = e2.adjoint(1.0, 0.0)
    assert np.abs(gr_u + F).max() <= 1e-9 * np.abs(F).max()


def test_mixture_parameter_gradients_vs_finite_differences(E):
    ps = psm.mixture(256, 14.0, 300.0, seed=4)
    e, U, W = forward(E, ps, 1.0)
    gU, gW = 1.0, 0.25
    _, gp = e.adjoint(gU, gW)
    npar = e.param_count()
    assert npar == 2 * 2 + 1 + 2 + 1
    for k in range(npar):
        p0 = get_param(ps, k)
        h = 1e-6 * abs(p0)
        _, Up, Wp = forward(E, set_param(ps, k, p0 + h), 1.0)
        _, Um, Wm = forward(E, set_param(ps, k, p0 - h), 1.0)
        fd = gU * (Up - Um) / (2 * h) + gW * (Wp - Wm) / (2 * h)
        scale = max(abs(fd), 1e-6 * (abs(U) + abs(W)) / abs(p0))
        assert abs(gp[k] - fd) <= 2e-5 * scale, (k, gp[k], fd)


def test_mixed_precision_adjoint_close_to_fp64(E):
    ps = psm.mixture(256, 14.0, 300.0, seed=6)
    out = {}
    for prec in ("fp64", "mixed"):
        e, _, _ = forward(E, ps, 1.0, prec)
        out[prec] = e.adjoint(1.0, 0.5)
    gr64, gp64 = out["fp64"]
    gr32, gp32 = out["mixed"]
    assert np.abs(gp32 - gp64).max() <= 2e-4 * np.abs(gp64).max()
    assert np.sqrt(((gr32 - gr64) ** 2).mean()) <= 2e-4 * np.sqrt((gr64 ** 2).mean())


def _oracle_uw(ps, rc):
    from oracle.oracle import Oracle
    o = Oracle(ps, rc, threads=min(os.cpu_count() or 1, 16))
    o.rebin()
    fo, _ = o.forces()
    return fo.upot, fo.virial


def _system(name):
    if name == "lj":
        return lj_box(), 2.5
    if name == "offcentre":
        from systems import offcentre_mixture
        return offcentre_mixture(), 1.0
    return psm.mixture(2000, 14.0, 300.0, seed=4), 1.0


@pytest.mark.parametrize("name", ["lj", "mixture", "offcentre"])
def test_parameter_gradients_vs_oracle_finite_differences(E, name):
    """dUpot/dp and dvirial/dp for every site parameter (eps and sigma of each
    LJ centre, |Q| of the quadrupole, |mu| of the dipole) against central
    differences of the oracle's FP64 forward with the parameter perturbed by
    h = 1e-5 |p| (the differences agree with the all-pairs reference to about
    1e-9 at this step): 5e-8 relative plus the differences' own rounding,
    1e-9 (|U| + |W|) / |p|, which dominates for parameters whose gradient is
    small beside the energy (the off-centre dipole's |mu|)."""
    ps, rc = _system(name)
    e, U, W = forward(E, ps, rc)
    _, gpU = e.adjoint(1.0, 0.0)
    _, gpW = e.adjoint(0.0, 1.0)
    U0, W0 = _oracle_uw(ps, rc)
    assert abs(U - U0) <= 1e-10 * abs(U0) and abs(W - W0) <= 1e-10 * abs(W0)
    for k in range(e.param_count()):
        p0 = get_param(ps, k)
        h = 1e-5 * abs(p0)
        Up, Wp = _oracle_uw(set_param(ps, k, p0 + h), rc)
        Um, Wm = _oracle_uw(set_param(ps, k, p0 - h), rc)
        fu, fw = (Up - Um) / (2 * h), (Wp - Wm) / (2 * h)
        # plus the rounding of the differences: about 1e-14 of |U| + |W| over the step h = 1e-5 |p|
        noise = 1e-9 * (abs(U0) + abs(W0)) / abs(p0)
        assert abs(gpU[k] - fu) <= 5e-8 * abs(fu) + noise, (k, gpU[k], fu, noise)
        assert abs(gpW[k] - fw) <= 5e-8 * abs(fw) + noise, (k, gpW[k], fw, noise)


@pytest.mark.parametrize("system", ["mixture", "offcentre"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-4)])
def test_mixture_against_fp64_all_pairs_torch_reference(E, precision, tol, system):
    """2,048-molecule 2CLJQ + 1CLJD mixture (multipoles at the molecule
    centres: without gF its multipole Hessian-vector products take the
    homogeneity shortcut) and a 1,372-molecule mixture with off-centre
    dipoles and quadrupoles (tests/systems.py; dual numbers throughout):
    position gradients (with a force cotangent gF, i.e. the pair
    Hessian-vector products of the LJ, dipole and quadrupole bodies) and
    parameter gradients of the adjoint against the FP64 all-pairs torch
    reference, for three (gU, gW, gF) combinations.  FP64: per parameter
    1e-9 relative; mixed: 2e-4 of the largest."""
    pytest.importorskip("torch")
    from oracle.allpairs import AllPairs
    ps, rc = _system(system)
    ap = AllPairs(ps, rc)
    gF = np.random.default_rng(17).normal(size=(ps.n, 3))
    e, U, W = forward(E, ps, rc, precision)
    for gU, gW, g in ((1.0, 0.0, None), (0.0, 1.0, None), (0.3, -0.2, gF)):
        gr, gp = e.adjoint(gU, gW, g)
        gr_t, gp_t, Ut, Wt = ap.gradients(gU, gW, g)
        if precision == "fp64":
            assert abs(U - Ut) <= 1e-10 * abs(Ut) and abs(W - Wt) <= 1e-10 * abs(Wt)
        assert np.abs(gr - gr_t).max() <= tol * np.abs(gr_t).max(), (gU, gW, np.abs(gr - gr_t).max())
        scale = np.abs(gp_t) if precision == "fp64" else np.abs(gp_t).max()
        assert np.all(np.abs(gp - gp_t) <= tol * scale), (gU, gW, gp, gp_t)


@pytest.mark.parametrize("shifted", [False, True])
def test_mixed_single_component_lj_adjoint_close_to_fp64(E, shifted):
    """The FP32 single-component LJ adjoint (with the pair Hessian-vector
    product) against the FP64 adjoint on the same state."""
    ps = psm.lj_fcc(6, 0.7, 1.1, seed=8, shifted=shifted, rc=2.5)
    rng = np.random.default_rng(8)
    ps.r = ps.r + rng.uniform(-0.15, 0.15, ps.r.shape)
    gF = rng.normal(size=(ps.n, 3))
    out = {}
    for prec in ("fp64", "mixed"):
        e = E.Engine(ps, 2.5, precision=prec, skin=0.3)
        e.forces()
        out[prec] = e.adjoint(0.7, -0.3, gF)
        e.close()
    gr64, gp64 = out["fp64"]
    gr32, gp32 = out["mixed"]
    assert np.abs(gp32 - gp64).max() <= 2e-4 * np.abs(gp64).max()
    assert np.sqrt(((gr32 - gr64) ** 2).mean()) <= 2e-4 * np.sqrt((gr64 ** 2).mean())


def test_lj_against_fp64_all_pairs_torch_reference(E):
    """N=2048 subset: FP64 all-pairs minimum-image LJ in torch (autograd)
    gives dU/dr, dU/deps, dU/dsigma and the virial's parameter gradients."""
    torch = pytest.importorskip("torch")
    ps = lj_box(8, rho=0.7, seed=9)
    rc = 2.5
    e, U, W = forward(E, ps, rc)
    gr, gp = e.adjoint(1.0, 0.0)
    _, gpw = e.adjoint(0.0, 1.0)
    r = torch.tensor(ps.r, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    L = torch.tensor(ps.box, dtype=torch.float64)
    d = r[:, None, :] - r[None, :, :]
    d = d - L * torch.round(d / L)
    r2 = (d * d).sum(-1)
    n = ps.n
    mask = (r2 < rc * rc) & ~torch.eye(n, dtype=torch.bool)
    r2s = torch.where(mask, r2, torch.ones_like(r2))
    s6 = (sig * sig / r2s) ** 3
    u = torch.where(mask, 4 * eps * (s6 * s6 - s6), torch.zeros_like(r2))
    Ut = 0.5 * u.sum()
    w = torch.where(mask, 24 * eps * (2 * s6 * s6 - s6), torch.zeros_like(r2))
    Wt = 0.5 * w.sum()
    assert abs(Ut.item() - U) <= 1e-10 * abs(U)
    assert abs(Wt.item() - W) <= 1e-10 * abs(W)
    gr_t, ge, gs = torch.autograd.grad(Ut, (r, eps, sig), retain_graph=True)
    assert np.abs(gr - gr_t.numpy()).max() <= 1e-9 * np.abs(gr_t.numpy()).max()
    assert abs(gp[0] - ge.item()) <= 1e-9 * abs(ge.item())
    assert abs(gp[1] - gs.item()) <= 1e-9 * abs(gs.item())
    we, ws = torch.autograd.grad(Wt, (eps, sig))
    assert abs(gpw[0] - we.item()) <= 1e-9 * abs(we.item())
    assert abs(gpw[1] - ws.item()) <= 1e-9 * abs(ws.item())


def test_autograd_function_loss_gradient(E):
    """torch.autograd.Function over the engine (validation harness only): the
    loss (U - U*)^2 + w (P - P*)^2 of a snapshot, differentiated w.r.t. eps,
    sigma and positions, matches central differences."""
    torch = pytest.importorskip("torch")
    ps = lj_box(4, seed=11)
    rc = 2.5
    V = float(np.prod(ps.box))

    class EnergyVirial(torch.autograd.Function):
        @staticmethod
        def forward(ctx, r, params):
            q = set_param(set_param(ps, 0, float(params[0])), 1, float(params[1]))
            q.r = r.detach().numpy().copy()
            e = E.Engine(q, rc)
            fo = e.forces()
            ctx.e = e
            return torch.tensor([fo.upot, fo.virial], dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            gr, gp = ctx.e.adjoint(float(g[0]), float(g[1]))
            return torch.from_numpy(gr), torch.from_numpy(gp)

    r = torch.tensor(ps.r, dtype=torch.float64, requires_grad=True)
    params = torch.tensor([1.0, 1.0], dtype=torch.float64, requires_grad=True)
    Ut, Pt, w = -2500.0, 0.5, 3.0

    def loss(r, params):
        uw = EnergyVirial.apply(r, params)
        n = ps.n
        P = n / V * 1.1 + uw[1] / (3 * V)
        return (uw[0] - Ut) ** 2 + w * (P - Pt) ** 2

    l0 = loss(r, params)
    l0.backward()
    with torch.no_grad():
        for k in range(2):
            h = 1e-6
            pp, pm = params.clone(), params.clone()
            pp[k] += h
            pm[k] -= h
            fd = (loss(r, pp) - loss(r, pm)).item() / (2 * h)
            assert abs(params.grad[k].item() - fd) <= 1e-5 * abs(fd), (k, params.grad[k].item(), fd)
        i, c = 17, 1
        rp, rm = r.clone(), r.clone()
        rp[i, c] += 1e-6
        rm[i, c] -= 1e-6
        fd = (loss(rp, params) - loss(rm, params)).item() / 2e-6
        assert abs(r.grad[i, c].item() - fd) <= 1e-5 * max(abs(fd), 1.0)
