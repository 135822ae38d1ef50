"""Golden vectors for espins_gb300.optimize_t from the reference's own
utility/optimize-temperatures/optimize_T.py.

The reference script draws a plot with matplotlib, which this image lacks; a
stand-in module that accepts the plotting calls lets the script run unchanged.
The script's input (its shipped E.dat: temperature and energy per site) and
its converged temperatures (the array Tout, full precision) for two settings
are written to optimize_t_golden.json next to this file.

Run from the repository root:  python tests/golden/make_optimize_t_golden.py <reference_dir>
"""
import json
import os
import runpy
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    folder = os.path.join(ref_root, "utility", "optimize-temperatures")
    plt = types.ModuleType("matplotlib.pyplot")
    for name in ("plot", "xlabel", "ylabel", "legend", "savefig", "show"):
        setattr(plt, name, lambda *a, **k: None)
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = plt
    sys.modules["matplotlib"], sys.modules["matplotlib.pyplot"] = mpl, plt
    dat = np.loadtxt(os.path.join(folder, "E.dat"))
    out = {"source": "utility/optimize-temperatures", "T": dat[:, 0].tolist(), "E": dat[:, 1].tolist(), "runs": []}
    cwd = os.getcwd()
    try:
        os.chdir(folder)
        for alpha, eps in ((0.5, 1e-6), (0.9, 1e-8)):
            sys.argv = ["optimize_T.py", "--data", "E.dat", "--alpha", str(alpha), "--epsilon", str(eps)]
            ns = runpy.run_path("optimize_T.py", run_name="__main__")
            out["runs"].append({"alpha": alpha, "epsilon": eps, "tems": [float(x) for x in ns["Tout"]],
                                "iterations": int(ns["n_iter"])})
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "optimize_t_golden.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_optimize_t_golden.py <reference_dir>")
    main(sys.argv[1])
