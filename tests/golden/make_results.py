"""Golden ResultWriter files of the reference: oracle/ref/ref_harness.cpp's
`res` mode runs NVE or NVT Leapfrog steps with the reference's own
io/ResultWriter (every step written, a short accumulation window so the
sliding averages wrap) and stores the `.res` lines without the two
time-stamped comments, together with the input state (format of
make_golden.py).

    python tests/golden/make_results.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

FREQ, ACC, PREC = 1, 7, 10


def main():
    tmp = mg.tempfile.mkdtemp()
    cases = [("lj500_nve", mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12), 2.5, 2.5, 0.002, 25, 0.0),
             ("lj500_nvt", mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12), 2.5, 2.5, 0.002, 25, 1.0),
             ("mix500_nvt", mg.psm.mixture(500, 18.0, 300.0, seed=31), 1.0, 1.0, 9.118e-5, 12, 500.0)]
    for name, ps, rc, rclj, dt, n, T in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        ps = mg.psm.read_inp(path)
        prefix = os.path.join(tmp, name)
        p = mg.subprocess.run([mg.HARNESS, "res", path, str(rc), str(rclj), str(dt), str(n), str(T), prefix,
                               str(FREQ), str(ACC), str(PREC)], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-2000:])
        res = mg.parse(p.stdout)
        lines = open(prefix + ".res").read().splitlines()
        body = [l for l in lines if not l.startswith("# ls1")]
        mg.store("res_" + name, ps, rc, rclj, True, res, dt, n, True)
        z = dict(np.load(os.path.join(HERE, "res_" + name + ".npz")))
        z.update(res_lines=np.array("\n".join(body)), target_temperature=T, write_frequency=FREQ,
                 accumulation_steps=ACC, write_precision=PREC)
        np.savez_compressed(os.path.join(HERE, "res_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
