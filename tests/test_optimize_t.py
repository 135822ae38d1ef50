"""The temperature optimiser (the reference's utility/optimize-temperatures)
against golden vectors made by running the reference's own optimize_T.py on
its shipped E.dat (tests/golden/make_optimize_t_golden.py), plus the property
it is for: equal exchange exponents Delta(beta) Delta(E) along the set."""
import json
import os

import numpy as np
import pytest

from espins_gb300.optimize_t import exchange_exponents, main, optimize_temperatures


def _golden(golden_dir):
    with open(os.path.join(golden_dir, "optimize_t_golden.json")) as fh:
        return json.load(fh)


def test_matches_reference_script(golden_dir):
    g = _golden(golden_dir)
    for run in g["runs"]:
        tems, it = optimize_temperatures(g["T"], g["E"], run["alpha"], run["epsilon"])
        # the same iteration, np.interp instead of scipy's interp1d
        assert np.max(np.abs(tems - np.array(run["tems"]))) < 1e-9, run["alpha"]
        assert abs(it - run["iterations"]) <= 2


def test_exchange_exponents_become_equal(golden_dir):
    g = _golden(golden_dir)
    T, E = np.array(g["T"]), np.array(g["E"])
    tems, _ = optimize_temperatures(T, E, 0.5, 1e-10)
    c = exchange_exponents(tems, np.interp(tems, T, E))
    c0 = exchange_exponents(T, E)
    assert np.std(c) / abs(np.mean(c)) < 1e-6 and np.std(c0) / abs(np.mean(c0)) > 0.1
    assert tems[0] == T[0] and tems[-1] == T[-1] and np.all(np.diff(tems) > 0)


def test_cli_prints_the_set(golden_dir, tmp_path, capsys):
    g = _golden(golden_dir)
    f = tmp_path / "E.dat"
    np.savetxt(f, np.column_stack([g["T"], g["E"]]))
    main(["--data", str(f)])
    out = capsys.readouterr().out
    line = [l for l in out.splitlines() if l.startswith("tems=")][0]
    assert [float(x) for x in line.split()[1:]] == pytest.approx(g["runs"][0]["tems"], abs=1e-4)
