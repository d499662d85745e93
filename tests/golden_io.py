"""Load the golden fixtures written by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

from ls1gb300 import phasespace as psm

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(prefix=""):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def _component(d):
    return psm.Component(lj=[psm.LJCenter(tuple(s["r"]), s["m"], s["eps"], s["sigma"], s["tcutoff"], s["shifted"])
                             for s in d["lj"]],
                         charges=[psm.Charge(tuple(s["r"]), s["m"], s["q"]) for s in d["charges"]],
                         dipoles=[psm.Dipole(tuple(s["r"]), tuple(s["e"]), s["abs"]) for s in d["dipoles"]],
                         quadrupoles=[psm.Quadrupole(tuple(s["r"]), tuple(s["e"]), s["abs"]) for s in d["quadrupoles"]],
                         I_override=tuple(d["I_override"]))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    comps = [_component(c) for c in json.loads(str(z["components"]))]
    ps = psm.PhaseSpace(z["box"].copy(), comps, [tuple(m) for m in z["mixing"]], float(z["eps_rf"]),
                        z["ids"].copy(), z["comp"].copy(), z["r"].copy(), z["v"].copy(), z["q"].copy(),
                        z["L"].copy())
    g = {k: z[k] for k in z.files if k not in ("components",)}
    g["rc"] = float(z["rc"])
    g["rc_lj"] = float(z["rc_lj"])
    g["periodic"] = bool(int(z["periodic"]))
    return ps, g
