"""Generate the fixtures of the reference's own mixed precision (spdp_*.npz).

Runs the reference's SPDP build (float pair arithmetic, double accumulation;
``oracle/ref/Makefile`` with PREC=SPDP into ``oracle/_ref/``) on the inputs
of the periodic fixtures per_lj500, per_lj4000j, per_lj864_rclj, per_mix500
and per_slab (one force evaluation, set up as make_golden.py does for its
DPDP runs) and stores its F, M, Vi, Upot, virial and pair counts.  Against
the DPDP fixtures of the same inputs this is the reference's own
mixed-precision error, the yardstick of the engine's mixed precision.  Only
this script reads the reference tree.

    python tests/golden/make_spdp.py [--ref <ls1-mardyn tree>]   (default: oracle/refpath.py)
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from ls1gb300 import phasespace as psm  # noqa: E402
import golden_io  # noqa: E402
import make_golden  # noqa: E402

INPUTS = ["per_lj500", "per_lj4000j", "per_lj864_rclj", "per_mix500", "per_slab"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    a = ap.parse_args()
    if a.ref is None:
        from oracle.refpath import reference_tree
        a.ref = reference_tree()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={a.ref}", "PREC=SPDP", "-j8"],
                   check=True)
    make_golden.HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness_SPDP")
    tmp = tempfile.mkdtemp()
    for name in INPUTS:
        ps, g = golden_io.load(name)
        path = os.path.join(tmp, name + ".inp")
        psm.write_inp(ps, path)
        res = make_golden.run(["forces", path, g["rc"], g["rc_lj"], 1])
        mol = np.array(res["mol"])
        out = "spdp_" + name[len("per_"):]
        np.savez_compressed(os.path.join(HERE, out + ".npz"), input=name, upot=res["upot"], virial=res["virial"],
                            counts=res["counts"], out_ids=mol[:, 0].astype(np.uint64), F=mol[:, 16:19],
                            M=mol[:, 19:22], Vi=mol[:, 22:25])
        print(f"{out}: N={mol.shape[0]} upot={res['upot']}")


if __name__ == "__main__":
    main()
