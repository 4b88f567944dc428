"""ORACLE — test infrastructure only: the timed CPU baseline.

Times the reference's two CPU time loops, as restated in mb_oracle.cpp
(solver_cpu_fdtd and the temporally blocked solver_cpu_fdtd_red with its
8-step overlap; the same results bit for bit), built with the reference's
own solver-cpu flags (oracle/build.py build_baseline), on a bounded sample
of the batched 2-level ensemble, on all physical cores of this host with
the OpenMP threads pinned one per core. bench.py runs this module in a
child process so that the OpenMP runtime starts with the pinning set:

    OMP_NUM_THREADS=<cores> OMP_PROC_BIND=close OMP_PLACES=cores \\
        python -m oracle.cpu_baseline --runs 8 --target-s 12

prints one JSON object: cell-updates/s per loop, the better loop, the
sample, threads, compiler flags and the CPU model. With --steps S and
--repeats K (the reference arm of bench.py) every repeat times the same
S-step sample once per loop. --compare-reference (only where the
reference tree is present) also times the reference's own two loops,
compiled from its sources with the same flags (oracle/_ref), on the same
runs truncated to the same step count.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LOOPS = (("plain", 0), ("red", 8))


def cpu_info():
    """CPU model, physical cores and usable logical CPUs of this host."""
    info = {"machine": platform.machine()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True,
                             timeout=10).stdout
        kv = {}
        for line in out.splitlines():
            if ":" in line:
                k, v = line.split(":", 1)
                kv[k.strip()] = v.strip()
        info["model"] = kv.get("Model name") or kv.get("Vendor ID")

        def num(key, default):
            v = kv.get(key, "")
            return int(v) if v.isdigit() else default
        # Arm hosts report cores per cluster and "-" sockets
        per = num("Core(s) per socket", 0) or num("Core(s) per cluster", 0)
        cores = per * (num("Socket(s)", 0) or num("Cluster(s)", 1))
        if cores:
            info["physical_cores"] = cores
        info["threads_per_core"] = num("Thread(s) per core", 1)
    except Exception as e:  # lscpu missing: /proc/cpuinfo
        info["lscpu"] = "unavailable: %s" % e
    try:
        info["usable_cpus"] = len(os.sched_getaffinity(0))
    except AttributeError:
        info["usable_cpus"] = os.cpu_count() or 1
    return info


def default_threads(info=None):
    info = info or cpu_info()
    phys = info.get("physical_cores") or info["usable_cpus"]
    return max(1, min(phys, info["usable_cpus"]))


def _runs(n, seed):
    from mbsolve_gb300 import setups
    runs, _ = setups.ensemble_2lvl(num_runs=n, seed=seed)
    return runs


def time_loops(runs, steps, threads):
    """Seconds per loop for `steps` steps of every run in `runs`."""
    from mbsolve_gb300 import lib as mb
    from oracle import oracle as O
    out = {}
    for name, ol in LOOPS:
        t0 = time.perf_counter()
        for dev, sce in runs:
            o = O.OracleRun("cvr-rodr", 2, mb.to_pod(dev, sce), baseline=True)
            o.run(threads=threads, max_steps=steps, red=ol)
        out[name] = time.perf_counter() - t0
    return out


def time_reference(n, seed, steps, threads):
    """Seconds of the reference's own solver_cpu_fdtd and
    solver_cpu_fdtd_red (reference flags) and of the restatement, on the
    first n runs truncated to `steps` steps; None without the tree."""
    from mbsolve_gb300 import lib as mb
    from mbsolve_gb300 import setups
    from oracle import oracle as O
    if O.ref_lib(baseline=True) is None:
        return None
    os.environ["OMP_NUM_THREADS"] = str(threads)
    out = {}
    for name, solver, ol in (("plain", "cpu-fdtd-2lvl-cvr-rodr", 0),
                             ("red", "cpu-fdtd-red-2lvl-cvr-rodr", 8)):
        for who in ("reference", "restatement"):
            mb.material.clear_library()
            runs, _ = setups.ensemble_2lvl(num_runs=n, num_timesteps=steps,
                                           seed=seed)
            t0 = time.perf_counter()
            for dev, sce in runs:
                b = mb.to_pod(dev, sce)
                if who == "reference":
                    O.ReferenceRun(solver, b, baseline=True).run()
                else:
                    O.OracleRun("cvr-rodr", 2, b, baseline=True).run(
                        threads=threads, red=ol)
            out["%s_%s" % (who, name)] = time.perf_counter() - t0
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=8,
                    help="first runs of the ensemble in the sample")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--target-s", type=float, default=12.0)
    ap.add_argument("--steps", type=int, default=0,
                    help="fixed steps per run (default: calibrated)")
    ap.add_argument("--repeats", type=int, default=1)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--compare-reference", action="store_true")
    a = ap.parse_args(argv)
    from oracle import build as B
    info = cpu_info()
    threads = a.threads or int(os.environ.get("OMP_NUM_THREADS", "0") or 0) \
        or default_threads(info)
    runs = _runs(a.runs, a.seed)
    cells = sum(s.get_num_gridpoints() for _, s in runs)
    steps = a.steps
    if not steps:
        # calibrate on the first run, then size each loop to half the target
        t = time_loops(runs[:1], 100, threads)["plain"]
        rate = runs[0][1].get_num_gridpoints() * 100 / t
        steps = int(max(50, min(50000, 0.5 * a.target_s * rate / cells)))
    secs = {name: [] for name, _ in LOOPS}
    for _ in range(a.repeats):
        for name, s in time_loops(runs, steps, threads).items():
            secs[name].append(s)
    cu = float(cells) * steps
    rates = {n: cu * len(v) / sum(v) for n, v in secs.items()}
    best = max(rates, key=rates.get)
    extra = {}
    if a.compare_reference:
        ref = time_reference(a.runs, a.seed, steps, threads)
        extra["reference_loops"] = (
            {k: cu / v for k, v in ref.items()} if ref else
            "reference tree not present")
    print(json.dumps(dict({
        "rates": rates, "best": best, "value": rates[best],
        "seconds": secs, "cell_updates_per_repeat": cu,
        "sample": "first %d runs of the ensemble (%d points), %d steps "
                  "each" % (a.runs, cells, steps),
        "threads": threads, "flags": B.baseline_flags(),
        "pinning": "OMP_PROC_BIND=%s OMP_PLACES=%s" % (
            os.environ.get("OMP_PROC_BIND", "unset"),
            os.environ.get("OMP_PLACES", "unset")),
        "cpu": info}, **extra)))


if __name__ == "__main__":
    main()
