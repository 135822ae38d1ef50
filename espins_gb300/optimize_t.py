"""Parallel-tempering temperature sets with equal swap acceptance.

The reference ships this as a separate script
(utility/optimize-temperatures/optimize_T.py:38-76): K. Hukushima's iteration
(Phys. Rev. E 60, 3606 (1999)) moves every interior temperature to the point
where the acceptance exponents Delta(beta) Delta(E) of its two neighbouring
pairs become equal, with E(T) interpolated linearly between the measured
points and the two end temperatures fixed:

    g(T1, T, T2) = (E1/T1 - E2/T2 - E(T) (1/T1 - 1/T2)) / (E1 - E2)
    1/T_out = (1/T + g(T_prev, T, T_next)) / 2
    T <- (1 - alpha) T + alpha T_out         until max |T - T_out| <= epsilon

Energies may be totals or per site (g does not depend on their scale).
`from_gpu_run` measures E(T) with a short run on the GPU first, so a user gets
an optimised set from an input file in one call.

    python -m espins_gb300.optimize_t --data E.dat [--alpha 0.5] [--epsilon 1e-6]
    python -m espins_gb300.optimize_t --mcin seed.mcin [--steps 20000]
"""
from __future__ import annotations

import argparse
from typing import Optional, Tuple

import numpy as np


def optimize_temperatures(T, E, alpha: float = 0.5, epsilon: float = 1e-6,
                          max_iter: int = 10_000_000) -> Tuple[np.ndarray, int]:
    """(optimised temperatures, iterations) for measured energies E at the
    ascending temperatures T."""
    T = np.asarray(T, dtype=float)
    E = np.asarray(E, dtype=float)
    if T.ndim != 1 or T.size < 3 or T.size != E.size:
        raise ValueError("need at least three (T, E) points")
    if np.any(np.diff(T) <= 0):
        raise ValueError("temperatures must be strictly ascending")

    def e_of(t):
        return np.interp(t, T, E)

    n = T.size
    t_in = T.copy()
    t_out = np.zeros(n)
    t_out[0], t_out[-1] = T[0], T[-1]
    it = 1
    while np.max(np.abs(t_in - t_out)) > epsilon:
        t1, t, t2 = t_in[:-2], t_in[1:-1], t_in[2:]
        e1, e, e2 = e_of(t1), e_of(t), e_of(t2)
        g = (1.0 / (e1 - e2)) * (e1 / t1 - e2 / t2 - e * (1.0 / t1 - 1.0 / t2))
        t_out[1:-1] = 1.0 / (0.5 * (1.0 / t + g))
        it += 1
        if it > max_iter:
            raise RuntimeError("temperatures did not converge; use a smaller alpha")
        t_in[1:-1] = (1.0 - alpha) * t_in[1:-1] + alpha * t_out[1:-1]
    return t_out.copy(), it


def exchange_exponents(T, E_of_T) -> np.ndarray:
    """Delta(beta) Delta(E) of neighbouring pairs (the quantity made equal)."""
    T = np.asarray(T, dtype=float)
    e = np.asarray(E_of_T, dtype=float)
    return (1.0 / T[:-1] - 1.0 / T[1:]) * (e[:-1] - e[1:])


def from_gpu_run(inp, steps_warmup: Optional[int] = None, steps_mc: Optional[int] = None,
                 alpha: float = 0.5, epsilon: float = 1e-6, seed: Optional[int] = None):
    """E(T) per site from a plain Metropolis run of `inp` on the GPU (its
    temperatures, shorter schedules if given), then the optimised set."""
    from . import mc
    if steps_warmup is not None:
        inp.steps_warmup = int(steps_warmup)
    if steps_mc is not None:
        inp.steps_mc = int(steps_mc)
    inp.pt = False
    r = mc.run(inp, seed=seed, write=False)
    T = np.asarray(r.tems, dtype=float)
    order = np.argsort(T)
    e = r.res["data"][:, 0] / r.ham.n
    tems, _ = optimize_temperatures(T[order], e[order], alpha, epsilon)
    return tems, T[order], e[order]


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--data", default=None, help="two columns: temperature and energy (the default is E.dat)")
    ap.add_argument("--mcin", default=None, help="measure E(T) with a short GPU run of this input instead")
    ap.add_argument("--steps", type=int, default=None, help="steps_mc of that run")
    ap.add_argument("--alpha", type=float, default=0.5, help="mixing parameter (smaller if it does not converge)")
    ap.add_argument("--epsilon", type=float, default=1e-6, help="convergence threshold")
    a = ap.parse_args(argv)
    if a.mcin:
        from .mcin import read_mcin
        tems, T, e = from_gpu_run(read_mcin(a.mcin), steps_mc=a.steps, alpha=a.alpha, epsilon=a.epsilon)
    else:
        dat = np.loadtxt(a.data or "E.dat")
        T, e = dat[:, 0], dat[:, 1]
        tems, _ = optimize_temperatures(T, e, a.alpha, a.epsilon)
    print("tems= " + " ".join("%5.4f" % t for t in tems))
    before = exchange_exponents(T, e)
    after = exchange_exponents(tems, np.interp(tems, T, e))
    print("# T_i   dbeta*dE (input set)   T_i   dbeta*dE (optimised set)")
    for k in range(before.size):
        print("%10.4f %14.6e %10.4f %14.6e" % (T[k + 1], before[k], tems[k + 1], after[k]))


if __name__ == "__main__":
    main()
