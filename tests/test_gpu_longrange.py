"""The engine's homogeneous long-range correction (md_longrange_homogeneous)
against the reference's own values (tests/golden/lrc_*.npz, made by
tests/golden/make_lrc.py): UpotCorr and VirialCorr to 1e-13 relative (host
arithmetic in the reference's order; pow of the C library), and the
per-molecule virial-tensor correction VirialCorr / (3 N)."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


@pytest.mark.parametrize("name", golden_io.names("lrc_"))
def test_longrange_homogeneous_matches_reference(engine_mod, name):
    ps, g = golden_io.load(name)
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    u, w = e.longrange_homogeneous()
    e.close()
    for got, ref in ((u, float(g["upot_corr"])), (w, float(g["virial_corr"]))):
        assert abs(got - ref) <= 1e-13 * max(abs(ref), 1e-300), (got, ref)


def test_longrange_adds_the_virial_correction_per_molecule(engine_mod):
    ps, g = golden_io.load("lrc_lj864")
    e = engine_mod.Engine(ps, g["rc"], g["rc_lj"], precision="fp64")
    e.forces()
    vi0 = e.molecules()["Vi"]
    _, w = e.longrange_homogeneous(add_to_molecule_virial=True)
    vi1 = e.molecules()["Vi"]
    e.close()
    assert np.allclose(vi1 - vi0, w / (3.0 * ps.n), rtol=1e-12, atol=0)
