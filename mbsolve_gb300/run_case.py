"""Run one preset on the GPU and print its throughput (a command-line
counterpart of the reference tool's timing line, mbsolve-tool.cpp:672-696).

    python -m mbsolve_gb300.run_case --setup random_nlvl --levels 6 \\
        --points 65536 --steps 2000 --solver gpu-fdtd-6lvl-cvr-rodr-fp32 \\
        [--runs 8] [--tuning C,NT,DEPTH[,PERSISTENT]]

--setup ensemble_2lvl takes the first --runs runs of the batched 2-level
ensemble (seed --seed) for --steps steps.

Prints one JSON line: cell-updates/s over the timed steps (CUDA events on
the engine's stream, after autotuning and a warm-up of 10 % of the steps),
the tuning used and the device status.
"""
import argparse
import json

from . import ensemble
from . import lib as mb
from . import setups


def build(args, seed):
    if args.setup == "random_nlvl":
        return setups.random_nlvl(N=args.levels, num_gridpoints=args.points,
                                  num_timesteps=args.steps, seed=seed)
    if args.setup == "lambda_3lvl":
        return setups.lambda_3lvl(num_gridpoints=args.points,
                                  num_timesteps=args.steps)
    if args.setup == "sit_2lvl":
        return setups.sit_2lvl(args.points, args.steps)
    if args.setup == "ensemble_2lvl":
        return setups.ensemble_2lvl(num_runs=args.runs,
                                    num_timesteps=args.steps,
                                    seed=args.seed)[0]
    raise SystemExit("unknown setup " + args.setup)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--setup", default="random_nlvl",
                    choices=["random_nlvl", "lambda_3lvl", "sit_2lvl",
                             "ensemble_2lvl"])
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--points", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--solver", default="gpu-fdtd-6lvl-cvr-rodr-fp32")
    ap.add_argument("--tuning", default="",
                    help="C,NT,DEPTH[,PERSISTENT] (default: autotune; "
                         "PERSISTENT 1 = persistent kernel, 2 = one launch "
                         "per DEPTH steps)")
    a = ap.parse_args(argv)
    mb.material.clear_library()
    if a.setup == "ensemble_2lvl":
        runs = build(a, a.seed)
    else:
        runs = [build(a, seed) for seed in range(a.runs)]
    tun = None
    if a.tuning:
        v = [int(x) for x in a.tuning.split(",")]
        tun = ensemble.tuning(v[0], v[1], v[2],
                              persistent=v[3] if len(v) > 3 else 0)
    e = ensemble.ensemble(a.solver, runs, tun)
    warm = max(1, a.steps // 10)
    timed = a.steps - warm
    e.advance(warm)
    e.region_begin()
    e.advance(timed)
    ms = e.region_end()
    cells = sum(e.grid(r).num_gridpoints for r in range(len(runs)))
    print(json.dumps({"solver": a.solver, "setup": a.setup, "runs": a.runs,
                      "points": a.points, "timed_steps": timed,
                      "cell_updates_per_s": cells * timed / (ms * 1e-3),
                      "ms": ms, "tuning": e.info(), "status": e.status()}))
    e.close()


if __name__ == "__main__":
    main()
