"""Builds tests/golden/literature/traces.npz from the reference's literature
traces (tools/reference-data/*.csv of the mbsolve tree, digitised from the
papers its presets reproduce): x in um vs population inversion
(Ziolkowski 1995, fig. 2, compared at record row 75 = 187.5 fs), t in fs vs
rho11 (Song 2005, fig. 3a), t in ps vs rho55 and rho66 (Marskar 2011).

    python tests/golden/literature/make_traces.py [path/to/mbsolve]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    # default: $MBSOLVE_REFERENCE, else a checkout named "reference" beside
    # this repository
    root = sys.argv[1] if len(sys.argv) > 1 else (
        os.environ.get("MBSOLVE_REFERENCE") or
        os.path.join(HERE, "..", "..", "..", "..", "reference"))
    d = os.path.join(root, "tools", "reference-data")
    out = {}
    for key, name in [("ziolkowski1995_inv12_row75", "ziolkowski1995-2.csv"),
                      ("song2005_d11", "song2005-3a.csv"),
                      ("marskar2011_d55", "marskar2011-rho55.csv"),
                      ("marskar2011_d66", "marskar2011-rho66.csv")]:
        out[key] = np.loadtxt(os.path.join(d, name), delimiter=",")
    np.savez_compressed(os.path.join(HERE, "traces.npz"), **out)


if __name__ == "__main__":
    main()
