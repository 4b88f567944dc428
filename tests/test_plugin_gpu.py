"""The mbsolve-lib plugin (mbsolve_gb300/plugin/solver_gpu_fdtd.cpp) on the
GPU through the C++ solver factory: solver_gpu_loader, then
solver::create_instance(name, dev, scen) -> run() -> get_results(), as
mbsolve-tool calls a solver (mbsolve-tool.cpp:669-686), on two golden
setups (FP64 within 1e-9 and FP32 within 1e-5 of the reference's own time
loop). The check program is built against the reference's mbsolve-lib
where its source tree exists, else against tests/mbsolve_lib_standin
(project-written headers with the same names and meaning for the subset
the plugin uses; the GPU machines do not have the reference tree)."""
import os
import subprocess

import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MBSOLVE_REFERENCE") or os.path.normpath(
    os.path.join(ROOT, "..", "reference"))
TOL = {"fp64": 1e-9, "fp32": 1e-5}


@pytest.fixture(scope="module")
def check_exe(native, tmp_path_factory):
    lib_dir = os.path.join(ROOT, "mbsolve_gb300")
    exe = str(tmp_path_factory.mktemp("plugin") / "plugin_check_gpu")
    srcs = [os.path.join(ROOT, "tests", "plugin_check_gpu.cpp"),
            os.path.join(ROOT, "mbsolve_gb300", "plugin",
                         "solver_gpu_fdtd.cpp")]
    ref_src = os.path.join(REF, "mbsolve-lib", "src")
    if os.path.isdir(ref_src):
        inc = os.path.join(REF, "mbsolve-lib", "include")
        srcs += [os.path.join(ref_src, f) for f in
                 ("device.cpp", "material.cpp", "record.cpp", "result.cpp",
                  "scenario.cpp", "solver.cpp", "writer.cpp")]
        which = "reference mbsolve-lib"
    else:
        inc = os.path.join(ROOT, "tests", "mbsolve_lib_standin")
        which = "stand-in headers"
    cmd = ["g++", "-O1", "-std=c++17", "-w", "-include", "iostream",
           "-I" + inc] + srcs + ["-L" + lib_dir, "-lmbsolve_gb300",
                                 "-Wl,-rpath," + lib_dir, "-o", exe]
    subprocess.check_call(cmd)
    print("plugin check built against the", which)
    return exe


def _run(exe, args, tmp_path):
    out = subprocess.run([exe] + args[:2] + [str(tmp_path)] + args[2:],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    res = []
    for line in out.stdout.splitlines():
        if line.startswith("result "):
            _, k, rows, cols = line.split()
            a = np.fromfile(str(tmp_path / ("result%s.bin" % k)))
            res.append(a.reshape(int(rows), int(cols)))
    return res


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_plugin_sit_matches_golden(check_exe, prec, tmp_path):
    meta, recs = helpers.load_golden("sit_cvr")
    kw = meta["spec"]["kw"]
    dev, sce = setups.sit_2lvl(**kw)
    length = dev.get_regions()[0].get_x_end()
    src = sce.get_sources()[0]
    args = ["sit", "gpu-fdtd-2lvl-cvr-rodr-" + prec, str(kw["num_gridpoints"]),
            repr(sce.get_endtime()), repr(length), repr(src._ampl),
            repr(src._beta)]
    res = _run(check_exe, args, tmp_path)
    assert len(res) == len(recs)
    for a, b in zip(res, recs):
        assert a.shape == b.shape
        assert helpers.rel_err(a, b) <= TOL[prec], helpers.rel_err(a, b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_plugin_ziolkowski_cayley_matches_golden(check_exe, prec, tmp_path):
    meta, recs = helpers.load_golden("zio_cayley")
    assert meta["spec"]["kw"] == dict(num_gridpoints=1024, endtime=60e-15)
    res = _run(check_exe, ["zio", "gpu-fdtd-2lvl-reg-cayley-" + prec],
               tmp_path)
    assert len(res) == len(recs)
    for a, b in zip(res, recs):
        assert a.shape == b.shape
        assert helpers.rel_err(a, b) <= TOL[prec], helpers.rel_err(a, b)
