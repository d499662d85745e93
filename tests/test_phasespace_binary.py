"""ls1's binary phase-space (checkpoint) format: the engine's device-side
writer and reader (md_write_phasespace_binary / md_read_phasespace_binary)
against files the reference itself wrote and read (tests/golden/binary_*.npz,
made by tests/golden/make_binary.py: Domain::writeCheckpoint with the binary
format, then BinaryReader).

All comparisons are bit-exact: the format stores doubles as they are, so
the engine must reproduce the reference's bytes record by record (the
reference writes in container order, the engine in upload order, so
records are matched by molecule id) and read back exactly the values the
reference's reader produced.
"""
import os

import numpy as np
import pytest

import golden_io
from oracle import oracle as O

NAMES = golden_io.names("binary_")


def _golden(name):
    ps, g = golden_io.load(name)
    dat = g["restart_dat"].tobytes()
    return ps, g, dat, str(g["restart_header"])


def _records_by_id(data: bytes) -> dict:
    a = np.frombuffer(data, O.RECORD_DTYPES["ICRVQD"])
    raw = np.frombuffer(data, np.uint8).reshape(-1, 116)
    return {int(i): raw[k].tobytes() for k, i in enumerate(a["id"])}


# ---------------------------------------------------------------- oracle (CPU)
@pytest.mark.parametrize("name", NAMES)
def test_oracle_reader_matches_reference_reader(name):
    _, g, dat, hdr = _golden(name)
    t, box, m = O.read_phasespace_binary(hdr, dat)
    assert t == float(g["binr_time"])
    assert np.array_equal(box, g["binr_length"])
    o = np.argsort(m["id"])
    assert np.array_equal(m["id"][o], g["out_ids"])
    assert np.array_equal(m["comp"][o], g["out_comp"])
    for k, f in (("r", "out_r"), ("v", "out_v"), ("q", "out_q"), ("L", "out_L")):
        assert np.array_equal(m[k][o], g[f]), k


@pytest.mark.parametrize("name", NAMES)
def test_oracle_writer_matches_reference_writer(name):
    ps, g, dat, hdr = _golden(name)
    t, box, m = O.read_phasespace_binary(hdr, dat)
    assert O.phasespace_binary_header(ps.box, ps.n, float(g["time"])) == hdr
    assert O.phasespace_binary_records(m["id"], m["comp"], m["r"], m["v"], m["q"], m["L"]) == dat
    # the reference wrote exactly the input state
    order = np.argsort(ps.ids)
    assert O.phasespace_binary_records(ps.ids[order], ps.comp[order], ps.r[order], ps.v[order], ps.q[order],
                                       ps.L[order]) == O.phasespace_binary_records(
        *(m[k][np.argsort(m["id"])] for k in ("id", "comp", "r", "v", "q", "L")))


# ---------------------------------------------------------------- engine (GPU)
@pytest.fixture(scope="module")
def engine_mod():
    import importlib
    import build as eb
    eb.build()
    return importlib.import_module("ls1gb300.engine")


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_writes_reference_bytes(engine_mod, name, tmp_path):
    ps, g, dat, hdr = _golden(name)
    e = engine_mod.Engine(ps, g["rc"], precision="fp64")
    prefix = str(tmp_path / "ck")
    e.write_phasespace_binary(prefix, float(g["time"]))
    e.close()
    assert open(prefix + ".header.xml").read() == hdr
    ours = open(prefix + ".dat", "rb").read()
    assert len(ours) == len(dat)
    assert _records_by_id(ours) == _records_by_id(dat)
    # upload order
    assert np.array_equal(np.frombuffer(ours, O.RECORD_DTYPES["ICRVQD"])["id"], ps.ids)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_reads_reference_file(engine_mod, name, tmp_path):
    ps, g, dat, hdr = _golden(name)
    (tmp_path / "r.header.xml").write_text(hdr)
    (tmp_path / "r.dat").write_bytes(dat)
    e = engine_mod.Engine(ps, g["rc"], precision="fp64")
    f_up = e.forces()
    F_up = e.molecules()["F"]
    t, n = e.read_phasespace_binary(str(tmp_path / "r.header.xml"), str(tmp_path / "r.dat"))
    assert (t, n) == (float(g["binr_time"]), ps.n)
    m = e.molecules()
    _, _, want = O.read_phasespace_binary(hdr, dat)
    assert np.array_equal(m["ids"], want["id"])
    assert np.array_equal(m["comp"], want["comp"])
    for k in ("r", "v", "q", "L"):
        assert np.array_equal(m[k], want[k]), k
    # the same state as uploaded, so the same forces (file order differs: per id)
    f_rd = e.forces()
    F_rd = e.molecules()["F"]
    e.close()
    assert int(f_rd.site_pairs[0]) == int(f_up.site_pairs[0])
    assert abs(f_rd.upot - f_up.upot) <= 1e-12 * abs(f_up.upot)
    a, b = np.argsort(ps.ids), np.argsort(m["ids"])
    assert np.abs(F_rd[b] - F_up[a]).max() <= 1e-12 * np.abs(F_up).max()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["ICRV", "IRV"])
def test_engine_reads_short_formats(engine_mod, fmt, tmp_path):
    ps, g, dat, hdr = _golden("binary_lj500")
    _, _, m = O.read_phasespace_binary(hdr, dat)
    a = np.zeros(ps.n, O.RECORD_DTYPES[fmt])
    a["id"], a["r"], a["v"] = m["id"], m["r"], m["v"]
    if fmt == "ICRV":
        a["cid"] = m["comp"] + 1
    (tmp_path / "s.header.xml").write_text(hdr.replace('type="ICRVQD"', 'type="%s"' % fmt))
    (tmp_path / "s.dat").write_bytes(a.tobytes())
    e = engine_mod.Engine(ps, g["rc"], precision="fp64")
    e.read_phasespace_binary(str(tmp_path / "s.header.xml"), str(tmp_path / "s.dat"))
    out = e.molecules()
    e.close()
    assert np.array_equal(out["r"], m["r"]) and np.array_equal(out["v"], m["v"])
    assert np.all(out["q"] == [1.0, 0.0, 0.0, 0.0]) and np.all(out["L"] == 0.0)
    assert np.all(out["comp"] == 0)


@pytest.mark.gpu
def test_engine_rejects_bad_files(engine_mod, tmp_path):
    ps, g, dat, hdr = _golden("binary_lj500")
    e = engine_mod.Engine(ps, g["rc"], precision="fp64")
    (tmp_path / "b.header.xml").write_text(hdr.replace("<number>500</number>", "<number>501</number>"))
    (tmp_path / "b.dat").write_bytes(dat)
    with pytest.raises(engine_mod.EngineError):  # truncated data
        e.read_phasespace_binary(str(tmp_path / "b.header.xml"), str(tmp_path / "b.dat"))
    x = "%21.15e" % ps.box[0]
    (tmp_path / "c.header.xml").write_text(hdr.replace("<x>%s</x>" % x, "<x>%21.15e</x>" % (ps.box[0] * 1.01)))
    with pytest.raises(engine_mod.EngineError):  # other box
        e.read_phasespace_binary(str(tmp_path / "c.header.xml"), str(tmp_path / "b.dat"))
    bad = np.frombuffer(dat, O.RECORD_DTYPES["ICRVQD"]).copy()
    bad["cid"][7] = 0
    (tmp_path / "d.dat").write_bytes(bad.tobytes())
    (tmp_path / "d.header.xml").write_text(hdr)
    with pytest.raises(engine_mod.EngineError):  # component id 0
        e.read_phasespace_binary(str(tmp_path / "d.header.xml"), str(tmp_path / "d.dat"))
    e.close()


@pytest.mark.gpu
def test_checkpoint_restart_continues_the_run(engine_mod, tmp_path):
    """A 1CLJ box of 108,000 molecules: 20 steps in one go against 10 steps,
    a binary checkpoint, a new engine restarted from it and 10 more steps
    (the restarted engine sees the molecules in checkpoint order, so its sums
    run in another order: 1e-12 relative)."""
    from ls1gb300 import phasespace as psm
    ps = psm.lj_fcc(30, 0.8, 1.0, seed=5)
    a = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    a.forces()
    rec_a = a.run(0.002, 20)
    b = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    b.forces()
    b.run(0.002, 10)
    name = b.write_checkpoint(str(tmp_path / "run"), 10, 0.02, num_steps=20)
    assert os.path.exists(name + ".dat") and name.endswith("run-10.restart")
    state_b = b.molecules()
    b.close()
    c = engine_mod.Engine(ps, 2.5, precision="fp64", skin=0.3)
    t, n = c.read_phasespace_binary(name + ".header.xml", name + ".dat")
    assert n == ps.n and abs(t - 0.02) <= 1e-15
    state_c = c.molecules()
    for k in ("r", "v", "q", "L"):
        assert np.array_equal(state_c[k], state_b[k]), k
    c.forces()
    rec_c = c.run(0.002, 10)
    a_state, c_state = a.molecules(), c.molecules()
    a.close()
    c.close()
    for col in range(3):
        assert np.abs(rec_c[:, col] - rec_a[10:, col]).max() <= 1e-12 * np.abs(rec_a[10:, col]).max(), col
    assert np.abs(c_state["r"] - a_state["r"]).max() <= 1e-10
