"""The C-ABI library: it builds, loads without a GPU, exports every entry
point declared in include/ls1gb300.h, and the ctypes structs match the C
layouts (checked against a C program compiled from the header)."""
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ls1-mardyn_gb300"))
import build as engine_build  # noqa: E402
from ls1gb300 import abi  # noqa: E402

HEADER = os.path.join(ROOT, "include", "ls1gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(md_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    path = engine_build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_struct_layouts_match_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "ls1gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(md_config), sizeof(md_component), sizeof(md_bin_stats),
         sizeof(md_forces_out), sizeof(md_kinetic_out), sizeof(md_step_record));
  printf("%zu %zu %zu\n", offsetof(md_config, skin), offsetof(md_component, inertia), offsetof(md_forces_out, site_pairs));
  return 0;
}
'''
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "t.c"), "w") as f:
        f.write(src)
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), "-o", os.path.join(d, "t"), os.path.join(d, "t.c")],
                   check=True)
    out = subprocess.run([os.path.join(d, "t")], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(x) for x in out]
    assert sizes[:6] == [ctypes.sizeof(t) for t in (abi.MdConfig, abi.MdComponent, abi.MdBinStats,
                                                    abi.MdForcesOut, abi.MdKineticOut, abi.MdStepRecord)]
    assert sizes[6] == abi.MdConfig.skin.offset
    assert sizes[7] == abi.MdComponent.inertia.offset
    assert sizes[8] == abi.MdForcesOut.site_pairs.offset


def test_batch_struct_layouts_match_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "ls1gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(md_batch_config), sizeof(md_box_sums), sizeof(md_batch_tuning),
         sizeof(md_kernel_times), offsetof(md_kernel_times, adjoint_ms));
  printf("%zu %zu %zu %zu %zu %zu\n", offsetof(md_batch_config, box_len), offsetof(md_batch_config, skin),
         offsetof(md_batch_config, device), offsetof(md_batch_tuning, trial_ms_per_step),
         offsetof(md_batch_config, cell_occupancy), offsetof(md_batch_tuning, trial_occupancy));
  return 0;
}
'''
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "t.c"), "w") as f:
        f.write(src)
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), "-o", os.path.join(d, "t"), os.path.join(d, "t.c")],
                   check=True)
    out = [int(x) for x in subprocess.run([os.path.join(d, "t")], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert out[:3] == [ctypes.sizeof(t) for t in (abi.MdBatchConfig, abi.MdBoxSums, abi.MdBatchTuning)]
    assert out[3:5] == [ctypes.sizeof(abi.MdKernelTimes), abi.MdKernelTimes.adjoint_ms.offset]
    assert out[5:] == [abi.MdBatchConfig.box_len.offset, abi.MdBatchConfig.skin.offset,
                       abi.MdBatchConfig.device.offset, abi.MdBatchTuning.trial_ms_per_step.offset,
                       abi.MdBatchConfig.cell_occupancy.offset, abi.MdBatchTuning.trial_occupancy.offset]



def test_control_struct_layouts_match_header():
    """Temperature control, planar long-range and kinetic-output structs."""
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "ls1gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(md_tc_region), sizeof(md_temperature_control),
         offsetof(md_tc_region, ramp_update_freq), offsetof(md_tc_region, method), offsetof(md_tc_region, nu),
         offsetof(md_temperature_control, regions), offsetof(md_temperature_control, timestep),
         offsetof(md_temperature_control, seed));
  printf("%zu %zu %d %d %d %d\n", sizeof(md_planar_config), sizeof(md_kinetic_out), MD_TC_MAX_REGIONS,
         MD_TC_MAX_SLABS, MD_TC_VELOCITY_SCALING, MD_TC_ANDERSEN);
  return 0;
}
'''
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "t.c"), "w") as f:
        f.write(src)
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), "-o", os.path.join(d, "t"), os.path.join(d, "t.c")],
                   check=True)
    out = [int(x) for x in subprocess.run([os.path.join(d, "t")], capture_output=True, text=True,
                                          check=True).stdout.split()]
    R, T = abi.MdTcRegion, abi.MdTemperatureControl
    assert out[:8] == [C_size(R), C_size(T), R.ramp_update_freq.offset, R.method.offset, R.nu.offset,
                       T.regions.offset, T.timestep.offset, T.seed.offset]
    assert out[8:] == [C_size(abi.MdPlanarConfig), C_size(abi.MdKineticOut), abi.MD_TC_MAX_REGIONS,
                       abi.MD_TC_MAX_SLABS, 0, 1]


def C_size(t):
    return ctypes.sizeof(t)

def test_batch_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import numpy as np
    lib.md_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(abi.MdBatchConfig)]
    lib.md_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.md_batch_last_error.argtypes = [ctypes.c_void_p]
    lib.md_batch_last_error.restype = ctypes.c_char_p
    L = np.full(6, 10.0)
    cfg = abi.MdBatchConfig(nbox=2, precision=abi.MD_PREC_MIXED, box_len=L.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            rc=2.5, epsilon=1.0, sigma=1.0, mass=1.0, skin=-1.0)
    h = ctypes.c_void_p()
    assert lib.md_batch_create(ctypes.byref(h), ctypes.byref(cfg)) == abi.MD_ERR_DEVICE
    assert b"device" in lib.md_batch_last_error(h)
    lib.md_batch_destroy(h)
    cfg.rc = 4.0   # 10 < 3 rc: rejected before any device call
    h = ctypes.c_void_p()
    assert lib.md_batch_create(ctypes.byref(h), ctypes.byref(cfg)) == abi.MD_ERR_ARG
    lib.md_batch_destroy(h)


def test_create_without_gpu_fails_cleanly(lib):
    """Without a visible GPU md_create returns MD_ERR_CUDA instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    lib.md_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(abi.MdConfig)]
    h = ctypes.c_void_p()
    cfg = abi.make_config((10.0, 10.0, 10.0), 2.5, 2.5, 1e10)
    assert lib.md_create(ctypes.byref(h), ctypes.byref(cfg)) == abi.MD_ERR_CUDA
    assert not h.value
