"""Precision report: the mixed-precision engine against its own FP64 kernel
on one phase-space state.

Both precisions evaluate the forces of the same molecules at the same
positions (``md_compute_forces``); the report gives the relative rms errors
of the per-molecule forces and torques (rms of |X_mixed - X_fp64| over rms of
|X_fp64|, the form of the precision target for this path), the largest
per-molecule force error relative to that rms, the relative errors of Upot,
the virial and the pressure p = (sum m v^2 + virial) / (3V), and whether the
interacting molecule and site pair counts agree exactly.  The comparison of a
float computation with a double one over whole configurations follows the
reference's own Vectorized-vs-Legacy checks
(src/particleContainer/adapter/tests/VectorizedCellProcessorTest.cpp:136-219),
with the error norms above in place of a per-component bound.
"""
from __future__ import annotations

import numpy as np

from . import engine as E
from .phasespace import PhaseSpace


def state_of(mol: dict, ps: PhaseSpace) -> PhaseSpace:
    """The phase space `ps` with the molecules of a download (sorted by id)."""
    order = np.argsort(mol["ids"], kind="stable")
    q = ps.copy()
    q.r, q.v, q.q, q.L = mol["r"][order], mol["v"][order], mol["q"][order], mol["L"][order]
    q.ids, q.comp = mol["ids"][order], mol["comp"][order]
    return q


def _rel_rms(a: np.ndarray, b: np.ndarray) -> float:
    den = np.sqrt((b ** 2).sum(axis=1).mean())
    return float(np.sqrt(((a - b) ** 2).sum(axis=1).mean()) / den) if den > 0 else 0.0


def _rel(a: float, b: float) -> float:
    return abs(a - b) / abs(b) if b != 0 else abs(a - b)


def kinetic_sum(ps: PhaseSpace) -> float:
    """sum m v^2 of the phase space (molecule masses from the components)."""
    m = np.array([c.mass_inertia()[0] for c in ps.components])[ps.comp]
    return float((m * (ps.v ** 2).sum(axis=1)).sum())


def report(ps: PhaseSpace, rc: float, rc_lj: float | None = None, skin: float = 0.0, device: int = 0,
           mixed_forces=None) -> dict:
    """Mixed vs FP64 forces of the state `ps`.  `mixed_forces` = (MdForcesOut,
    molecules()) of an engine already holding `ps` in mixed precision (the
    engine that ran the workload); otherwise a mixed engine is created."""
    def run(prec):
        e = E.Engine(ps, rc, rc_lj, precision=prec, skin=skin, device=device)
        fo = e.forces()
        mol = e.molecules()
        e.close()
        return fo, mol

    fom, mm = mixed_forces if mixed_forces is not None else run("mixed")
    fo6, m6 = run("fp64")
    om, o6 = np.argsort(mm["ids"], kind="stable"), np.argsort(m6["ids"], kind="stable")
    Fm, F6 = mm["F"][om], m6["F"][o6]
    Mm, M6 = mm["M"][om], m6["M"][o6]
    frms = np.sqrt((F6 ** 2).sum(axis=1).mean())
    vol = float(np.prod(ps.box))
    kin = kinetic_sum(ps)
    pm, p6 = (kin + fom.virial) / (3 * vol), (kin + fo6.virial) / (3 * vol)
    out = {
        "molecules": int(ps.n),
        "force_rel_rms": _rel_rms(Fm, F6),
        "force_max_err_over_rms": float(np.sqrt(((Fm - F6) ** 2).sum(axis=1)).max() / frms) if frms > 0 else 0.0,
        "upot_rel": _rel(fom.upot, fo6.upot),
        "virial_rel": _rel(fom.virial, fo6.virial),
        "pressure_rel": _rel(pm, p6),
        "mol_pairs": int(fo6.mol_pairs),
        "pairs_equal": bool(fom.mol_pairs == fo6.mol_pairs and list(fom.site_pairs) == list(fo6.site_pairs)),
        "upot_per_molecule_fp64": fo6.upot / ps.n,
    }
    if np.abs(M6).max() > 0:
        out["torque_rel_rms"] = _rel_rms(Mm, M6)
    return out
