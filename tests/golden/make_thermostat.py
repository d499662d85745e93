"""Golden runs of the reference with its global velocity-scaling thermostat
(Simulation::simulateOneTimestep with VELSCALE_THERMOSTAT and one
thermostat: beta_trans = (3 N T / sum m v^2)^0.4, beta_rot =
(rotDOF T / sum I w^2)^0.4, then v *= beta_trans, D *= beta_rot), driven
by oracle/ref/ref_harness.cpp's `nvt` mode.  Writes nvtt_*.npz in the
format of make_golden.py plus the per-step betas.

    python tests/golden/make_thermostat.py
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
    cases = [("lj500", mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12), 2.5, 2.5, 0.002, 20, 1.0),
             ("mix500", mg.psm.mixture(500, 18.0, 300.0, seed=31), 1.0, 1.0, 9.118e-5, 10, 500.0)]
    for name, ps, rc, rclj, dt, n, T in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        ps = mg.psm.read_inp(path)
        p = mg.subprocess.run([mg.HARNESS, "nvt", path, str(rc), str(rclj), str(dt), str(n), str(T)],
                              capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-2000:])
        res = mg.parse(p.stdout)
        betas = np.array([[float(x) for x in l.split()[1:]] for l in p.stdout.splitlines() if l.startswith("BETA")])
        mg.store("nvtt_" + name, ps, rc, rclj, True, res, dt, n, True)
        z = dict(np.load(os.path.join(HERE, "nvtt_" + name + ".npz")))
        z["betas"] = betas
        z["target_temperature"] = T
        np.savez_compressed(os.path.join(HERE, "nvtt_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
