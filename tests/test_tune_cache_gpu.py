"""The autotuner's results persist across processes through the file named
by MBG_TUNE_CACHE: a second process reuses the tuning without timing the
candidates again."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = """
import json, sys
sys.path.insert(0, %r)
from mbsolve_gb300 import ensemble, lib as mb, setups
runs, _ = setups.ensemble_2lvl(num_runs=16, num_timesteps=400, seed=3)
e = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp32", runs)
print(json.dumps({"info": e.info()}))
""" % ROOT


def _run(env):
    out = subprocess.run([sys.executable, "-c", PROG], env=env, check=True,
                         capture_output=True, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


def test_tuning_reused_from_file(native, tmp_path):
    env = dict(os.environ, MBG_TUNE_CACHE=str(tmp_path / "tune.txt"))
    first = _run(env)
    lines = open(env["MBG_TUNE_CACHE"]).read().split("\n")
    assert len([l for l in lines if l.strip()]) == 1
    second = _run(env)
    assert second["info"] == first["info"]
    # a process that tuned again would have appended a second line
    lines = open(env["MBG_TUNE_CACHE"]).read().split("\n")
    assert len([l for l in lines if l.strip()]) == 1
