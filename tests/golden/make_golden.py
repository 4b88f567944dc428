"""Generates the golden fixtures of tests/golden from the reference's own
code: mbsolve-lib and the solver_cpu_fdtd time loop compiled from the
reference tree (oracle/_ref, built by oracle/build_ref.sh), instantiated
with the oracle's Eigen-free Lindblad algorithms. One OpenMP thread (the
reference applies soft sources once per thread).

Usage: python tests/golden/make_golden.py [--reference ROOT] [case ...]
(default: every case)
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(
    __file__))))
sys.path.insert(0, ROOT)
os.environ["OMP_NUM_THREADS"] = "1"

import numpy as np  # noqa: E402

CASES = {
    "zio_cvr": ("cpu-fdtd-2lvl-cvr-rodr", "ziolkowski1995",
                dict(num_gridpoints=1024, endtime=60e-15)),
    "zio_cayley": ("cpu-fdtd-2lvl-reg-cayley", "ziolkowski1995",
                   dict(num_gridpoints=1024, endtime=60e-15)),
    "zio_noop": ("cpu-fdtd-noop", "ziolkowski1995",
                 dict(num_gridpoints=1024, endtime=60e-15)),
    "song_cvr": ("cpu-fdtd-3lvl-cvr-rodr", "song2005",
                 dict(endtime=80e-15, num_timesteps=3000)),
    "song_cayley": ("cpu-fdtd-3lvl-reg-cayley", "song2005",
                    dict(endtime=80e-15, num_timesteps=3000)),
    "marskar4_cvr": ("cpu-fdtd-4lvl-cvr-rodr", "marskar2011",
                     dict(N=4, num_gridpoints=256, endtime=1.5e-12)),
    "marskar6_cvr": ("cpu-fdtd-6lvl-cvr-rodr", "marskar2011",
                     dict(N=6, num_gridpoints=128, endtime=1.0e-12)),
    "marskar5_cayley": ("cpu-fdtd-5lvl-reg-cayley", "marskar2011",
                        dict(N=5, num_gridpoints=128, endtime=1.0e-12)),
    "sit_cvr": ("cpu-fdtd-2lvl-cvr-rodr", "sit_2lvl",
                dict(num_gridpoints=512, num_timesteps=4000)),
    "lambda_cayley": ("cpu-fdtd-3lvl-reg-cayley", "lambda_3lvl",
                      dict(num_gridpoints=512, num_timesteps=3000)),
    "lambda_cvr": ("cpu-fdtd-3lvl-cvr-rodr", "lambda_3lvl",
                   dict(num_gridpoints=512, num_timesteps=3000)),
    # the QCL comb preset at the reference's grid spacing on a 0.31 mm
    # device (random initial field, seeded), both forms
    "tzenov2016_cvr": ("cpu-fdtd-5lvl-cvr-rodr", "tzenov2016",
                       dict(num_gridpoints=512, endtime=12e-12, seed=1,
                            length=5e-3 * 511 / 8191)),
    "tzenov2016_cayley": ("cpu-fdtd-5lvl-reg-cayley", "tzenov2016",
                          dict(num_gridpoints=512, endtime=12e-12, seed=1,
                               length=5e-3 * 511 / 8191)),
    # colliding-pulse mode locking: gain, absorber, gain (random initial
    # field, seeded)
    "tzenov2018_cvr": ("cpu-fdtd-2lvl-cvr-rodr", "tzenov2018_cpml",
                       dict(num_gridpoints=512, endtime=30e-12, seed=1)),
}


def main(ref_root=None, only=()):
    if ref_root:
        os.environ["MBSOLVE_REFERENCE"] = ref_root
    from mbsolve_gb300 import lib as mb
    from tests import helpers
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for case, (solver, setup, kw) in CASES.items():
        if only and case not in only:
            continue
        mb.material.clear_library()
        spec = {"setup": setup, "kw": kw}
        dev, sce = helpers.build_setup(spec)
        grid, recs = helpers.reference_results(solver, dev, sce)
        meta = dict(solver=solver, spec=spec, num_records=len(recs),
                    num_gridpoints=grid.num_gridpoints,
                    num_timesteps=grid.num_timesteps,
                    gridpoint_size=grid.gridpoint_size,
                    timestep_size=grid.timestep_size,
                    generator="tests/golden/make_golden.py (reference "
                              "solver_cpu_fdtd via oracle/_ref)")
        arrays = {"rec%d" % k: r for k, r in enumerate(recs)}
        np.savez_compressed(os.path.join(out_dir, case + ".npz"),
                            meta=json.dumps(meta), **arrays)
        print(case, grid.num_gridpoints, grid.num_timesteps,
              [r.shape for r in recs])


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    main(a.reference, tuple(a.cases))
