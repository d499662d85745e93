"""The ls1-MarDyn drop-in (ls1-mardyn_gb300/ls1/): GpuLinkedCells and
GpuLeapfrog compile against the reference's own headers, the selection patch
applies to the reference's Simulation.cpp, the patched MarDyn links against
the reference's objects and libls1gb300.so -- and it runs: linked against a
stand-in of the engine library built over the oracle (tests/dropin/oracle_abi.c,
no GPU needed), the patched MarDyn with <datastructure type="GpuLinkedCells">
and <integrator type="GpuLeapfrog"> reproduces, step by step, the ResultWriter
output of the same binary with the reference's LinkedCells and Leapfrog.  The
NVT ensemble's velocity-scaling thermostat iterates the container every step
from OpenMP parallel regions, so each step also exercises the host-mirror
sync by the thread team, the edit of the mirror and the re-upload (with the
forces the next pre-force half step needs).  Needs the reference tree
(present where the engine is developed, absent on GPU hosts: skipped there)."""
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle.refpath import reference_tree  # noqa: E402

REF = reference_tree()
LS1 = os.path.join(ROOT, "ls1-mardyn_gb300", "ls1")
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj_DPDP")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference tree not present")

FLAGS = ["-std=c++17", "-O1", "-fopenmp", "-DMARDYN_DPDP", "-DTIMERS", "-w", f"-I{REF}/src", f"-I{REF}/libs/rapidxml",
         f"-I{ROOT}/include", f"-I{LS1}"]


def patched_simulation(tmp):
    a = os.path.join(tmp, "src")
    os.makedirs(a)
    shutil.copy(os.path.join(REF, "src", "Simulation.cpp"), a)
    subprocess.run(["patch", "-s", "-p1", "-i", os.path.join(LS1, "Simulation.patch")], cwd=tmp, check=True)
    return os.path.join(a, "Simulation.cpp")


def test_adapter_and_patch_compile():
    tmp = tempfile.mkdtemp()
    sim = patched_simulation(tmp)
    for src in (os.path.join(LS1, "GpuLinkedCells.cpp"), os.path.join(LS1, "GpuLeapfrog.cpp"), sim):
        subprocess.run(["g++", *FLAGS, "-fsyntax-only", src], check=True)


def test_patched_mardyn_links():
    if not os.path.isdir(OBJ):
        pytest.skip("reference objects not built (make -C oracle/ref)")
    sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
    import build as eb
    lib = eb.build()
    tmp = tempfile.mkdtemp()
    sim = patched_simulation(tmp)
    # a minimal driver in place of MarDyn.cpp (whose version header is generated by cmake)
    main = os.path.join(tmp, "driver.cpp")
    with open(main, "w") as f:
        f.write('#include <memory>\n#include "Simulation.h"\n#include "utils/Logger.h"\n'
                'int main(int argc, char** argv) {\n'
                '  Log::global_log = std::make_unique<Log::Logger>(Log::Info);\n'
                '  Simulation sim;\n'
                '  if (argc > 1) { sim.readConfigFile(argv[1]); sim.prepare_start(); sim.simulate(); }\n'
                '  return 0;\n}\n')
    objs = []
    for src in (os.path.join(LS1, "GpuLinkedCells.cpp"), os.path.join(LS1, "GpuLeapfrog.cpp"), sim, main):
        o = os.path.join(tmp, os.path.basename(src) + ".o")
        subprocess.run(["g++", *FLAGS, "-c", src, "-o", o], check=True)
        objs.append(o)
    ref_objs = []
    for dp, _, fs in os.walk(OBJ):
        for f in fs:
            if f.endswith(".o") and f not in ("Simulation.o", "harness.o"):
                ref_objs.append(os.path.join(dp, f))
    exe = os.path.join(tmp, "MarDyn_gpu")
    subprocess.run(["g++", "-fopenmp", "-o", exe, *objs, *ref_objs, lib, f"-Wl,-rpath,{os.path.dirname(lib)}"],
                   check=True)
    assert os.path.exists(exe)


# ---------------------------------------------------------------- the drop-in at run time (oracle stand-in)
DRIVER = ('#include <memory>\n#include "Simulation.h"\n#include "utils/Logger.h"\n'
          'int main(int argc, char** argv) {\n'
          '  Log::global_log = std::make_unique<Log::Logger>(Log::Info);\n'
          '  Simulation sim;\n'
          '  if (argc > 1) { sim.readConfigFile(argv[1]); sim.prepare_start(); sim.simulate(); }\n'
          '  return 0;\n}\n')


def _mardyn_over_oracle(tmp):
    """The patched MarDyn linked against the reference's objects and the oracle stand-in of the engine library."""
    sim = patched_simulation(tmp)
    main = os.path.join(tmp, "driver.cpp")
    with open(main, "w") as f:
        f.write(DRIVER)
    objs = []
    for src in (os.path.join(LS1, "GpuLinkedCells.cpp"), os.path.join(LS1, "GpuLeapfrog.cpp"), sim, main):
        o = os.path.join(tmp, os.path.basename(src) + ".o")
        subprocess.run(["g++", *FLAGS, "-c", src, "-o", o], check=True)
        objs.append(o)
    for src in (os.path.join(ROOT, "tests", "dropin", "oracle_abi.c"), os.path.join(ROOT, "oracle", "md_oracle.c")):
        o = os.path.join(tmp, os.path.basename(src) + ".o")
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c11", "-c", src, "-o", o], check=True)
        objs.append(o)
    ref_objs = [os.path.join(dp, f) for dp, _, fs in os.walk(OBJ) for f in fs
                if f.endswith(".o") and f not in ("Simulation.o", "harness.o", "harness_tc.o")]
    exe = os.path.join(tmp, "MarDyn_oracle")
    subprocess.run(["g++", "-fopenmp", "-o", exe, *objs, *ref_objs, "-lm"], check=True)
    return exe


def _components_xml(ps):
    """<components> of the phase space in ls1's XML form (sites, moments of inertia, LB mixing)."""
    out = ["<components>"]
    for c, comp in enumerate(ps.components, 1):
        out.append(f'<moleculetype id="{c}" name="C{c}">')
        k = 1
        for s in comp.lj:
            x, y, z = s.r
            out.append(f'<site type="LJ126" id="{k}"><coords><x>{x!r}</x><y>{y!r}</y><z>{z!r}</z></coords>'
                       f'<mass>{s.m!r}</mass><sigma>{s.sigma!r}</sigma><epsilon>{s.eps!r}</epsilon>'
                       f'<shifted>{"true" if s.shifted else "false"}</shifted></site>')
            k += 1
        for s in comp.charges:
            x, y, z = s.r
            out.append(f'<site type="Charge" id="{k}"><coords><x>{x!r}</x><y>{y!r}</y><z>{z!r}</z></coords>'
                       f'<mass>{s.m!r}</mass><charge>{s.q!r}</charge></site>')
            k += 1
        for kind, tag, sites in (("Dipole", "dipolemoment", comp.dipoles),
                                 ("Quadrupole", "quadrupolemoment", comp.quadrupoles)):
            for s in sites:
                x, y, z = s.r
                ex, ey, ez = s.e
                out.append(f'<site type="{kind}" id="{k}"><coords><x>{x!r}</x><y>{y!r}</y><z>{z!r}</z></coords>'
                           f'<{tag}><x>{ex!r}</x><y>{ey!r}</y><z>{ez!r}</z><abs>{s.abs!r}</abs></{tag}></site>')
                k += 1
        I = comp.mass_inertia()[1]
        out.append(f'<momentsofinertia rotaxes="xyz"><Ixx>{float(I[0])!r}</Ixx><Iyy>{float(I[1])!r}</Iyy>'
                   f'<Izz>{float(I[2])!r}</Izz></momentsofinertia></moleculetype>')
    if len(ps.components) > 1:
        out.append("<mixing>")
        k = 0
        for i in range(len(ps.components)):
            for j in range(i + 1, len(ps.components)):
                xi, eta = ps.mixing[k]
                out.append(f'<rule type="LB" cid1="{i + 1}" cid2="{j + 1}"><eta>{eta!r}</eta><xi>{xi!r}</xi></rule>')
                k += 1
        out.append("</mixing>")
    out.append("</components>")
    return "\n".join(out)


def _config(ps, inp, rc, dt, T, steps, gpu, prefix):
    L = [float(x) for x in ps.box]
    if gpu:
        ds = ('<datastructure type="GpuLinkedCells"><cellsInCutoffRadius>1</cellsInCutoffRadius>'
              '<precision>fp64</precision><skin>0.3</skin></datastructure>')
        it = f'<integrator type="GpuLeapfrog"><timestep unit="reduced">{dt!r}</timestep></integrator>'
    else:
        ds = '<datastructure type="LinkedCells"><cellsInCutoffRadius>1</cellsInCutoffRadius></datastructure>'
        it = f'<integrator type="Leapfrog"><timestep unit="reduced">{dt!r}</timestep></integrator>'
    return f"""<?xml version="1.0" encoding="UTF-8"?>
<mardyn version="20100525">
  <simulation type="MD">
    {it}
    <run><currenttime>0</currenttime><production><steps>{steps}</steps></production></run>
    <ensemble type="NVT">
      <temperature unit="reduced">{T!r}</temperature>
      <domain type="box"><lx>{L[0]!r}</lx><ly>{L[1]!r}</ly><lz>{L[2]!r}</lz></domain>
      {_components_xml(ps)}
      <phasespacepoint><file type="ASCII">{inp}</file></phasespacepoint>
    </ensemble>
    <algorithm>
      {ds}
      <cutoffs type="CenterOfMass"><defaultCutoff unit="reduced">{rc!r}</defaultCutoff>
        <radiusLJ unit="reduced">{rc!r}</radiusLJ></cutoffs>
      <electrostatic type="ReactionField"><epsilon>{ps.eps_rf!r}</epsilon></electrostatic>
      <longrange type="none"></longrange>
    </algorithm>
    <output>
      <outputplugin name="ResultWriter"><writefrequency>1</writefrequency><outputprefix>{prefix}</outputprefix>
        <writeprecision>12</writeprecision></outputplugin>
    </output>
  </simulation>
</mardyn>
"""


def _res(path):
    import numpy as np
    return np.array([[float(x) for x in line.split()] for line in open(path)
                     if line.strip() and not line.lstrip().startswith("#")])


@pytest.mark.parametrize("system", ["lj500", "mix500"])
def test_patched_mardyn_runs_like_the_reference(system):
    if not os.path.isdir(OBJ):
        pytest.skip("reference objects not built (make -C oracle/ref)")
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
    from ls1gb300 import phasespace as psm
    tmp = tempfile.mkdtemp()
    exe = _mardyn_over_oracle(tmp)
    if system == "lj500":
        ps = psm.lj_fcc(5, 0.8, 1.0, seed=11)
        ps.r = np.mod(ps.r + np.random.default_rng(12).uniform(-0.15, 0.15, ps.r.shape), ps.box)
        rc, dt, T, steps = 2.5, 0.002, 1.0, 30
    else:
        ps = psm.mixture(500, 18.0, 300.0, seed=31)
        rc, dt, T, steps = 1.0, 9.118e-5, 300.0, 20
    inp = os.path.join(tmp, system + ".inp")
    psm.write_inp(ps, inp)
    out = {}
    for gpu in (False, True):
        prefix = os.path.join(tmp, ("gpu_" if gpu else "ref_") + system)
        cfg = prefix + ".xml"
        with open(cfg, "w") as f:
            f.write(_config(ps, inp, rc, dt, T, steps, gpu, prefix))
        p = subprocess.run([exe, cfg], cwd=tmp, capture_output=True, text=True,
                           env=dict(os.environ, OMP_NUM_THREADS="2"), timeout=600)
        assert p.returncode == 0, (p.stdout + p.stderr)[-3000:]
        out[gpu] = _res(prefix + ".res")
    ref, got = out[False], out[True]
    assert ref.shape == got.shape and ref.shape[0] == steps + 1
    # columns: step, time, U_pot, U_pot_avg, U_kin, U_kin_avg, p, p_avg, beta_trans, beta_rot, c_v, N
    for col in (2, 4, 6, 8, 9):
        assert np.abs(got[:, col] - ref[:, col]).max() <= 1e-9 * np.abs(ref[:, col]).max(), col
    assert np.array_equal(got[:, 11], ref[:, 11])
