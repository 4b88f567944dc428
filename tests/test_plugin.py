"""The mbsolve-lib plugin (mbsolve_gb300/plugin) compiled against the
reference's own library sources: factory registration, the reference's
exceptions and, where a GPU is present, a run whose grid equals the one
the reference's init_fdtd_simulation derives. Skipped without the
reference tree (it is not on the GPU machines)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MBSOLVE_REFERENCE") or os.path.normpath(
    os.path.join(ROOT, "..", "reference"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "mbsolve-lib", "src")),
                    reason="reference tree not present")
def test_plugin_against_reference_library(native, tmp_path):
    lib_dir = os.path.join(ROOT, "mbsolve_gb300")
    srcs = [os.path.join(REF, "mbsolve-lib", "src", f) for f in
            ("device.cpp", "material.cpp", "record.cpp", "result.cpp",
             "scenario.cpp", "solver.cpp", "writer.cpp")]
    exe = str(tmp_path / "plugin_check")
    cmd = ["g++", "-O1", "-std=c++17", "-w",
           "-include", "iostream",
           "-I" + os.path.join(REF, "mbsolve-lib", "include"),
           os.path.join(ROOT, "tests", "plugin_check.cpp"),
           os.path.join(ROOT, "mbsolve_gb300", "plugin", "solver_gpu_fdtd.cpp"),
           ] + srcs + ["-L" + lib_dir, "-lmbsolve_gb300",
                       "-Wl,-rpath," + lib_dir, "-o", exe]
    subprocess.check_call(cmd)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    assert "registered 22" in text
    assert "no-regions: invalid_argument: No regions in device!" in text
    assert "levels: invalid_argument: Number of energy levels does not " \
           "match selected solver!" in text
    assert "duplicate: invalid_argument: Solver already registered." in text
    # without a GPU the engine reports the CUDA error as runtime_error;
    # with one, the grid equals the reference's and the run completes
    assert ("create: runtime_error: CUDA:" in text) or \
        ("grid: same" in text and "run: 2 results" in text), text
