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


def two_component_lj(seed):
    """1CLJ fcc 5^3x4 at rho* = 0.8 with every second molecule of a heavier,
    smaller second component (m = 2, eps = 0.9, sigma = 0.95; LB mixing)."""
    ps = mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=seed), 0.1, seed + 1)
    ps.components = [mg.psm.one_center_lj(), mg.psm.one_center_lj(eps=0.9, sigma=0.95, m=2.0)]
    ps.mixing = [(1.0, 1.0)]
    ps.comp = (np.arange(ps.n) % 2).astype(np.int32)
    return ps


def main_componentwise():
    """nvtc_*.npz: component c on thermostat c + 1 (oracle/ref/ref_harness.cpp `nvtc`); betas per step and
    thermostat in `betas_c` rows (step, thermostat, beta_trans, beta_rot)."""
    tmp = mg.tempfile.mkdtemp()
    cases = [("lj2c", two_component_lj(21), 2.5, 2.5, 0.002, 20, (1.2, 0.8)),
             ("mix500", mg.psm.mixture(500, 18.0, 500.0, seed=31), 1.0, 1.0, 9.118e-5, 10, (520.0, 480.0))]
    for name, ps, rc, rclj, dt, n, T in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        ps = mg.psm.read_inp(path)
        p = mg.subprocess.run([mg.HARNESS, "nvtc", path, str(rc), str(rclj), str(dt), str(n)] + [str(x) for x in T],
                              capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-2000:])
        res = mg.parse(p.stdout)
        res["grid"] = np.zeros(3, np.int64)
        res["cell_length"] = np.zeros(3)
        betas = np.array([[float(x) for x in l.split()[1:]] for l in p.stdout.splitlines() if l.startswith("BETA")])
        mg.store("nvtc_" + name, ps, rc, rclj, True, res, dt, n, True)
        z = dict(np.load(os.path.join(HERE, "nvtc_" + name + ".npz")))
        z["betas_c"] = betas
        z["targets"] = np.array(T)
        np.savez_compressed(os.path.join(HERE, "nvtc_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
    main_componentwise()
