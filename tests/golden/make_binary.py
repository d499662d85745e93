"""Golden files of ls1's binary phase-space (checkpoint) format, written and
read back by the reference itself through oracle/ref/ref_harness.cpp:
`binw` runs Domain::writeCheckpoint with the binary format (header XML +
FullMolecule::writeBinary records in container order), `binr` reads the pair
with BinaryReader.  Writes binary_*.npz in the format of make_golden.py (the
input phase space; out_* = the molecules BinaryReader produced) plus the raw
files and the header's time and box as the reference read them.

    python tests/golden/make_binary.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402


def main():
    tmp = tempfile.mkdtemp()
    cases = [("mix500", mg.psm.mixture(500, 18.0, 300.0, seed=31), 1.0, 0.75),
             ("lj500", mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12), 2.5, 12.5)]
    for name, ps, rc, time in cases:
        inp = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, inp)
        ps = mg.psm.read_inp(inp)
        prefix = os.path.join(tmp, name + ".restart")
        w = mg.subprocess.run([mg.HARNESS, "binw", inp, str(rc), prefix, repr(time)], capture_output=True, text=True)
        if w.returncode != 0:
            raise RuntimeError(w.stderr[-2000:])
        r = mg.subprocess.run([mg.HARNESS, "binr", inp, prefix + ".header.xml", prefix + ".dat", str(rc)],
                              capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        res = mg.parse(r.stdout)
        res["grid"] = np.zeros(3, np.int64)
        res["cell_length"] = np.zeros(3)
        mg.store("binary_" + name, ps, rc, rc, True, res)
        z = dict(np.load(os.path.join(HERE, "binary_" + name + ".npz")))
        lines = r.stdout.splitlines()
        z["binr_time"] = float([l for l in lines if l.startswith("TIME")][0].split()[1])
        z["binr_length"] = np.array([float(x) for x in [l for l in lines if l.startswith("LENGTH")][0].split()[1:]])
        z["time"] = time
        z["restart_dat"] = np.frombuffer(open(prefix + ".dat", "rb").read(), np.uint8)
        z["restart_header"] = open(prefix + ".header.xml").read()
        np.savez_compressed(os.path.join(HERE, "binary_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
