"""bench.py's choice of pair scheme (CPU): `--pair-scheme auto` runs
multi-site molecules (any component that is more than one LJ centre at its
origin) in the Newton-3 form and single-centre LJ on the rows; an explicit
choice is kept."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from ls1gb300 import phasespace as psm  # noqa: E402


def test_auto_scheme_follows_the_molecules():
    lj = psm.lj_fcc(3, 0.8, 1.0, seed=1)
    mix = psm.mixture(108, 18.0, 300.0, seed=1)
    assert not bench.is_multisite(lj)
    assert bench.is_multisite(mix)
    assert bench.scheme_for("auto", lj) == "rows"
    assert bench.scheme_for("auto", mix) == "newton3"
    for explicit in ("rows", "newton3"):
        assert bench.scheme_for(explicit, lj) == explicit
        assert bench.scheme_for(explicit, mix) == explicit


def test_an_off_centre_single_lj_centre_counts_as_multi_site():
    ps = psm.lj_fcc(3, 0.8, 1.0, seed=2)
    c = psm.one_center_lj()
    c.lj[0].r = (0.1, 0.0, 0.0)
    ps.components = [c]
    assert bench.is_multisite(ps)
    assert bench.scheme_for("auto", ps) == "newton3"
    assert np.all(ps.comp == 0)
