"""The ls1-MarDyn drop-in (ls1-mardyn_gb300/ls1/): GpuLinkedCells and
GpuLeapfrog compile against the reference's own headers, the selection patch
applies to the reference's Simulation.cpp, and the patched MarDyn links
against the reference's objects and libls1gb300.so.  Needs the reference tree
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
