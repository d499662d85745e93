"""Golden runs of the reference's region-wise temperature control
(thermostats/TemperatureControl, velocity scaling per region and slab),
driven by oracle/ref/ref_harness.cpp's `tc` mode: NVE Leapfrog steps with
TemperatureControl::DoLoopsOverMolecules after each step's global values.
Writes tc_*.npz in the format of make_golden.py plus the control settings
(`tc_json`), the reference's XML (`tc_xml`) and the betas of every measuring
step (`tcb` rows: step, region, slab, beta_trans, beta_rot, N).

    python tests/golden/make_tempctl.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

DIRS = {1: "x", 2: "y", 4: "z", 3: "xy", 5: "xz", 6: "yz", 7: "xyz"}


def xml_of(tc, box):
    def corner(v, d):
        return "box" if v is None else repr(float(v))
    regs = []
    for r in tc["regions"]:
        ramp = ""
        if r.get("ramp"):
            p = r["ramp"]
            ramp = ("<ramp><start>%r</start><end>%r</end><update><start>%d</start><stop>%d</stop>"
                    "<freq>%d</freq></update></ramp>" % (p["start"], p["end"], p["update_start"], p["update_stop"],
                                                           p["update_freq"]))
        regs.append(
            "<region><coords><lcx>%r</lcx><lcy>%r</lcy><lcz>%r</lcz><ucx>%s</ucx><ucy>%s</ucy><ucz>%s</ucz></coords>"
            "<target><temperature>%r</temperature><component>%d</component>%s</target>"
            "<settings><numslabs>%d</numslabs><exponent>%r</exponent><directions>%s</directions></settings>"
            "<writefreq>1000</writefreq><fileprefix>betalog</fileprefix></region>"
            % (float(r["lower"][0]), float(r["lower"][1]), float(r["lower"][2]),
               corner(r["upper"][0], 0), corner(r["upper"][1], 1), corner(r["upper"][2], 2),
               float(r["T"]), r["component"], ramp, r["numslabs"], float(r["exponent"]), DIRS[r["directions"]]))
    return ('<?xml version="1.0" encoding="UTF-8"?>\n<temperatureControl><control><start>%d</start>'
            "<frequency>%d</frequency><stop>%d</stop></control><regions>%s</regions></temperatureControl>\n"
            % (tc["start"], tc["frequency"], tc["stop"], "".join(regs)))


def main():
    tmp = mg.tempfile.mkdtemp()
    lj = mg.jitter(mg.psm.lj_fcc(5, 0.8, 1.0, seed=11), 0.15, 12)
    tc_lj = {"start": 0, "frequency": 2, "stop": 17, "regions": [
        {"lower": [0.0, 1.0, 0.0], "upper": [None, 7.5, None], "T": 1.3, "component": 0, "numslabs": 3,
         "exponent": 0.4, "directions": 5},
        {"lower": [1.0, 0.0, 2.0], "upper": [7.0, None, 8.0], "T": 0.8, "component": 0, "numslabs": 2,
         "exponent": 0.5, "directions": 7,
         "ramp": {"start": 0.8, "end": 1.1, "update_start": 2, "update_stop": 12, "update_freq": 4}}]}
    mix = mg.psm.mixture(500, 18.0, 300.0, seed=31)
    tc_mix = {"start": 1, "frequency": 1, "stop": 1000, "regions": [
        {"lower": [0.0, 0.0, 0.0], "upper": [None, None, None], "T": 400.0, "component": 1, "numslabs": 4,
         "exponent": 0.4, "directions": 7,
         "ramp": {"start": 400.0, "end": 450.0, "update_start": 2, "update_stop": 8, "update_freq": 2}},
        {"lower": [0.0, 0.5, 0.0], "upper": [None, 2.5, None], "T": 300.0, "component": 2, "numslabs": 2,
         "exponent": 0.4, "directions": 3}]}
    cases = [("lj500", lj, 2.5, 2.5, 0.002, 20, tc_lj), ("mix500", mix, 1.0, 1.0, 9.118e-5, 10, tc_mix)]
    for name, ps, rc, rclj, dt, n, tc in cases:
        path = os.path.join(tmp, name + ".inp")
        mg.psm.write_inp(ps, path)
        ps = mg.psm.read_inp(path)
        xml = xml_of(tc, ps.box)
        xpath = os.path.join(tmp, name + ".xml")
        open(xpath, "w").write(xml)
        p = mg.subprocess.run([mg.HARNESS, "tc", path, str(rc), str(rclj), str(dt), str(n), xpath],
                              capture_output=True, text=True, cwd=tmp)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-2000:])
        res = mg.parse(p.stdout)
        tcb = np.array([[float(x) for x in l.split()[1:]] for l in p.stdout.splitlines() if l.startswith("TCB")])
        mg.store("tc_" + name, ps, rc, rclj, True, res, dt, n, True)
        z = dict(np.load(os.path.join(HERE, "tc_" + name + ".npz")))
        z.update(tc_json=np.array(json.dumps(tc)), tc_xml=np.array(xml), tcb=tcb)
        np.savez_compressed(os.path.join(HERE, "tc_" + name + ".npz"), **z)


if __name__ == "__main__":
    main()
