#!/usr/bin/env python
"""Throughput benchmark of the GB300 Monte Carlo path.

Workload (default ``batch512_pt``, the largest configuration that fits one
GPU): 512 independent simple-cubic lattices with L drawn uniformly from
{8, 12, ..., 48} (seed 3; 17.6 M sites), J1 = +1.0 meV, nearest-neighbour
biquadratic 0.1 meV and DM 0.2 meV along the unit bond vector, 16 parallel-
tempering replicas per lattice log-spaced 2-25 K (3.4 GB of FP32 spins),
every lattice advanced in replayed CUDA graphs with the sweep kernel chosen
per size by the library's autotuner.  Inputs are synthetic (the reference
ships no benchmark data): uniform random spins on S^2.

A step is one swap interval of the measurement phase for all replicas of all
lattices: 10 sweeps (every colour class), 10 measurements (energy and
magnetisation accumulators, binning, P(M)) and one exchange within each
lattice.  Metric: site updates/s = steps * 10 * sum(N * R) / time.

* ``value``: device time of the timed steps, CUDA events on the library's
  stream (the state is larger than L2; the single-lattice workloads flush L2
  with a 256 MB write before every timed step, outside the events).
* ``e2e``: the same metric through the C ABI with host buffers, as one job:
  every lattice's spin_matrix set from host memory, esp_begin, the steps,
  esp_collect and esp_get_spins of every lattice, wall clock.
* ``roofline``: the dominant sweep kernel (the largest lattice size), 24 B of
  compulsory spin traffic per site update (read + write of one FP32
  3-vector), against the measured HBM copy bandwidth; ``traffic`` from the
  ncu capture summarised in profiles/dram_traffic.json.
* ``cpu_baseline``: the FP64 oracle (a restatement of the reference's Fortran:
  typewriter sweeps, MT19937) on the host cores, one thread per block of
  temperatures as the reference's MPI ranks, on a bounded sample.
* ``secondary``: the HBM-resident single-lattice workload sc128_pt (SC 128^3
  x 64 replicas), device-timed, from a separate process.

``--impl reference`` times that CPU implementation alone on the same
workload (the reference itself is Fortran + MPI and cannot be built in this
image).  Other workloads: ``--workload bcc24_pt | sc16_plain |
sc48_frustrated_pt | sc128_pt``.

``--proposal compare`` (with ``--workload sc48_frustrated_pt``) measures the
learned proposal instead: it collects 10^7 (environment, spin) pairs from the
plain PT sampler, trains the network on the GPU, then runs the plain and the
learned sampler from the same state and reports independent samples/s =
sum over temperature slots of sweeps/s / (2 tau_int), tau_int the larger of
E's and |m|'s (Sokal windowing), for both.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", default="batch512_pt")
    p.add_argument("--secondary", dest="secondary", action="store_true", default=True,
                   help="with batch512_pt: also a short device-timed run of sc128_pt (separate process)")
    p.add_argument("--no-secondary", dest="secondary", action="store_false")
    p.add_argument("--L", type=int, default=None)
    p.add_argument("--replicas", type=int, default=None)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--geometry", default=None,
                   help="batch512_pt: cluster geometry CTAs,threads,sites for every size instead of the "
                        "autotuner (profiling)")
    p.add_argument("--tile", default=None,
                   help="tiled sweep with geometry edge,replicas,variant (every size of batch512_pt) instead of "
                        "the autotuner's choice (profiling)")
    p.add_argument("--only-L", type=int, default=None,
                   help="batch512_pt: run only the lattices of this size (profiling of a small case)")
    p.add_argument("--max-lattices", type=int, default=None,
                   help="batch512_pt: at most this many lattices per size (profiling of a small case)")
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--proposal", choices=["plain", "learned", "compare"], default="plain")
    p.add_argument("--lp-engine", choices=["mma", "tcgen05"], default="tcgen05")
    p.add_argument("--train-pairs", type=int, default=10_000_000)
    p.add_argument("--train-steps", type=int, default=3000)
    p.add_argument("--measure-sweeps", type=int, default=20000)
    p.add_argument("--chains", type=int, default=4,
                   help="--proposal compare: independent PT chains (replica groups) per sampler; the spread of "
                        "their averages is part of each observable's error")
    p.add_argument("--equil-sweeps", type=int, default=5000,
                   help="--proposal compare: learned-sampler sweeps after training that equilibrate the common start "
                        "of both measurement windows")
    p.add_argument("--plain-sweeps", type=int, default=100000,
                   help="--proposal compare: sweeps of the plain sampler's measurement window (its low-temperature "
                        "autocorrelation times reach ~2000 sweeps, so its window is longer than the learned one's)")
    return p.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _uniform_spins(R, n, mag, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(R, n, 3))
    v /= np.linalg.norm(v, axis=2, keepdims=True)
    return v * mag[None, :, None]


def _peaks(kind: str = "hbm"):
    """(peak, source): HBM GB/s, or dense BF16 TFLOP/s (burst) for kind 'tensor'."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"] if kind == "hbm" else d["bf16_tflops"]), "measured"
    return (6800.0 if kind == "hbm" else 1900.0), "fallback"


# network FLOPs of one learned proposal: 2 (12*128 + 128*128 + 128*20)
LP_FLOP = 2 * (12 * 128 + 128 * 128 + 128 * 20)


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0])); mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _oracle_lib():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ctypes as C

    import oracle as O
    lib = O.lib()
    lib.or_pt_bench.argtypes = [C.POINTER(O.OrHam), C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int64,
                                C.c_int64, C.c_int64, C.c_int, C.c_double, C.c_int32, C.POINTER(C.c_double)]
    lib.or_pt_bench.restype = C.c_int64
    return O, lib


class PortRun:
    """The oracle's PT main phase (the reference's algorithm: typewriter
    sweeps, MT19937, measurements after every steps_measure sweeps, pt_swap)
    on one lattice's replicas, block-split over host threads as the reference
    splits temperatures over MPI ranks.  Each call of run(k) times k swap
    intervals inside the C code, from the barrier after the threads' set-up to
    the last interval, so neither the initial energies nor the thread
    start-up are timed; the spins carry over between calls."""

    def __init__(self, inp, ham, threads, seed, tems=None):
        import ctypes as C
        O, self.lib = _oracle_lib()
        self.C = C
        self.H = O.Ham(ham)
        self.tems = np.ascontiguousarray(inp.tems if tems is None else tems, dtype=np.float64)
        self.R = self.tems.size
        self.spins = np.ascontiguousarray(_uniform_spins(self.R, ham.n, ham.mag, seed).reshape(-1))
        self.pss = inp.pt_steps_swap if inp.pt else 1
        self.measure = inp.steps_measure
        self.mode = 1 if inp.mcarlo_mode.startswith("const") else 0
        self.tilt = inp.tilt_angles_max
        self.threads = max(1, min(threads, self.R))
        self.seed = seed

    def run(self, k):
        secs = self.C.c_double(0.0)
        n = self.lib.or_pt_bench(self.H.ref, self.threads, self.R, self.tems.ctypes.data, self.spins.ctypes.data,
                                 int(k), self.pss, self.measure, self.mode, self.tilt, self.seed, self.C.byref(secs))
        return int(n), float(secs.value)


def cpu_baseline(inp, ham, seconds: float, threads: int, seed: int):
    """The oracle port on host threads for about `seconds` of sweeps."""
    pr = PortRun(inp, ham, threads, seed)
    n1, t1 = pr.run(1)
    k = max(1, int(seconds / max(t1, 1e-6)))
    n, t = pr.run(k)
    return n / t, {"swap_intervals": k, "updates": int(n), "seconds": t,
                   "sweeps_per_interval": pr.pss * pr.measure, "threads": pr.threads}


def batch_port_rate(sizes, threads, seed, intervals, warm_intervals=1):
    """The oracle port on the 512-lattice workload: one lattice of every size
    (its 16 temperatures on min(16, threads) threads) runs `intervals` swap
    intervals after `warm_intervals` untimed ones; the whole batch's time is
    the per-size time weighted by the number of lattices of that size.
    Returns (site updates/s, seconds per interval of the whole batch, detail)."""
    from espins_gb300.tables import build_hamiltonian
    from espins_gb300.workloads import batch_lattice_mcin
    tot_upd, tot_sec, detail = 0.0, 0.0, {}
    for L, count in sizes.items():
        inp = batch_lattice_mcin(L)
        ham = build_hamiltonian(inp, check=False)
        pr = PortRun(inp, ham, threads, seed + L)
        if warm_intervals:
            pr.run(warm_intervals)
        n, t = pr.run(intervals)
        tot_upd += count * n
        tot_sec += count * t
        detail[str(L)] = {"updates": n, "seconds": t, "threads": pr.threads}
    return tot_upd / tot_sec, tot_sec / intervals, detail


def reference_arm(a, ws, rank):
    """--impl reference: the CPU implementation of the path (the FP64 oracle
    port of the reference's Fortran, which cannot be built here) on all host
    threads, on the same workload, config and metric as our arm.  Warm-up
    intervals run first, untimed; the timed region is one call over all K
    intervals, timed inside the C code (sweeps, measurements and swaps only).
    The 512-lattice workload runs one lattice of every size and weights the
    sizes by their counts."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if a.workload == "batch512_pt":
        from espins_gb300.workloads import batch_lattice_sizes
        sizes = batch_lattice_sizes(512, 3)
        value, sec_per_step, detail = batch_port_rate(sizes, threads, a.seed, a.steps, a.warmup)
        config = _batch_config(sizes)
        sample = (f"one lattice of each of the {len(sizes)} sizes (16 temperatures on 16 threads) for "
                  f"{a.warmup} untimed + {a.steps} timed swap intervals of 10 sweeps; the batch's time is the "
                  "per-size time weighted by the lattice counts; FP64 C restatement of the Fortran "
                  "(typewriter order, MT19937)")
        t_tot = sec_per_step * a.steps
        threads_used = min(threads, 16)
    else:
        from espins_gb300.tables import build_hamiltonian
        from espins_gb300.workloads import workload
        inp = workload(a.workload, L=a.L, replicas=a.replicas)
        ham = build_hamiltonian(inp, check=False)
        pr = PortRun(inp, ham, threads, a.seed)
        if a.warmup:
            pr.run(a.warmup)
        n, t_tot = pr.run(a.steps)
        value = n / t_tot
        config = _config(inp, ham, a.workload) | {"proposal": a.proposal}
        sample = (f"{a.warmup} untimed + {a.steps} timed swap intervals of all {pr.R} temperatures "
                  "in one call; FP64 C restatement of the Fortran (typewriter order, MT19937), temperatures "
                  "block-split over threads")
        threads_used = pr.threads
    line = {
        "impl": "reference", "metric": "site updates/s", "value": value, "unit": "site updates/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * t_tot / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config,
        "cpu_baseline": {"value": value, "unit": "site updates/s", "cores": threads_used, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "site updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _batch_config(sizes):
    nsites = sum(L ** 3 * c for L, c in sizes.items())
    return {"workload": "batch512_pt", "lattices": sum(sizes.values()), "sizes": {str(k): v for k, v in sizes.items()},
            "sites": nsites, "replicas_per_lattice": 16, "temperatures_K": [2.0, 25.0],
            "pt_steps_swap": 10, "sweeps_per_step": 10,
            "l2": f"state {12 * nsites * 16 / 1e9:.2f} GB of spins, larger than L2 (no flush needed)",
            "parallelism": "all lattices in one device; independent jobs per GPU when n_gpus > 1"}


def _config(inp, ham, name):
    return {"workload": name, "sites": ham.n, "atoms_per_cell": ham.num_atoms,
            "supercell": list(inp.supercell_size), "replicas": inp.tems_num,
            "temperatures_K": [float(inp.tems[0]), float(inp.tems[-1])],
            "pt": bool(inp.pt), "pt_steps_swap": inp.pt_steps_swap, "steps_measure": inp.steps_measure,
            "sweeps_per_step": (inp.pt_steps_swap if inp.pt else 1) * inp.steps_measure,
            "l2": "flushed before every timed step (256 MB write, outside the events)",
            "parallelism": "all replicas in one device; independent jobs per GPU when n_gpus > 1"}


def learned_compare(a, rank, local):
    """Learned vs plain PT sampler: training, site updates/s, tau_int, independent samples/s."""
    import torch

    from espins_gb300 import analysis
    from espins_gb300.lib import Engine
    from espins_gb300.tables import build_hamiltonian
    from espins_gb300.workloads import workload
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    inp = workload(a.workload, L=a.L, replicas=a.replicas)
    ham = build_hamiltonian(inp, check=False)
    nT, N = inp.tems_num, ham.n
    C = max(1, a.chains)
    R = nT * C                      # chain c holds slots [c nT, (c+1) nT)
    pss = inp.pt_steps_swap if inp.pt else 1
    seed = 4 + 1000 * rank
    stream = torch.cuda.current_stream(dev)
    eng = Engine(N, ham.num_atoms, ham.supercell, R, inp.boundary_open)
    eng.upload(ham)
    eng.set_temperatures(np.tile(inp.tems, C))
    if C > 1:
        eng.set_pt_groups(nT)       # each chain exchanges only within itself
    eng.set_stream(stream.cuda_stream)
    _, ncol = eng.colouring()
    # plain PT warm-up from independent random configurations, then one
    # colour class of every replica per swap interval
    eng.set_spins(_uniform_spins(R, N, ham.mag, seed))
    warm = 2000
    n_coll = -(-a.train_pairs // (N * R // ncol))
    sched = eng.schedule(0, (warm // pss + n_coll + 1) * pss, 1, pt=inp.pt, pt_steps_swap=pss, seed=seed)
    eng.begin(sched)
    eng.advance(warm // pss)
    eng.lp_reserve(a.train_pairs)
    t0 = time.perf_counter()
    rows = 0
    for k in range(n_coll):
        eng.advance(1)
        rows = eng.lp_collect(k % ncol)
    torch.cuda.synchronize(dev)
    t_collect = time.perf_counter() - t0
    start = eng.get_spins()
    eng.lp_init(seed=seed)
    eng.lp_set_engine(a.lp_engine)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    loss = eng.lp_train(a.train_steps, batch=4096, lr=1e-3, seed=seed)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    t_train = ev0.elapsed_time(ev1) * 1e-3
    # a common, equilibrated start for both windows: the plain chains' slow
    # relaxation at low temperature (tau of thousands of sweeps) would
    # otherwise bias the plain window; a biased learned sampler would show as
    # a drift of the plain window away from this start (its two halves differ)
    eng.set_proposal("learned")
    eng.set_spins(start)
    eng.begin(eng.schedule(0, a.equil_sweeps + pss, 1, pt=inp.pt, pt_steps_swap=pss, seed=seed + 31))
    eng.advance(max(1, a.equil_sweeps // pss))
    start = eng.get_spins()
    out = {}
    from espins_gb300 import analysis as A
    for kind in ("plain", "learned"):
        sweeps = a.plain_sweeps if kind == "plain" else a.measure_sweeps
        eng.set_proposal(kind)
        eng.set_spins(start)
        eng.set_series(sweeps)
        sched = eng.schedule(0, sweeps, 1, pt=inp.pt, pt_steps_swap=pss, seed=seed + 17)
        eng.begin(sched)
        eng.advance(max(1, 500 // pss))          # settle after the switch (not in the series window)
        units = -(-sweeps // pss) - max(1, 500 // pss)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        eng.advance(units)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        secs = e0.elapsed_time(e1) * 1e-3
        res = eng.collect()
        ser = eng.series()[-units * pss:]
        tau_e = np.array([[analysis.tau_int(ser[:, c * nT + t, 0]) for t in range(nT)] for c in range(C)])
        tau_m = np.array([[analysis.tau_int(ser[:, c * nT + t, 1]) for t in range(nT)] for c in range(C)])
        tau = np.maximum(tau_e, tau_m).mean(axis=0)       # per slot, over the chains
        sweeps_per_s = units * pss / secs
        ups = sweeps_per_s * N * R
        trials = -(-sweeps // pss) * pss * N     # per temperature slot, whole run
        acc = (1.0 - res["rejected"][:, 1] / trials).reshape(C, nT).mean(axis=0)
        # the _mc.dat observables of the measurement window per chain
        # (jackknife errors), averaged over the chains; the error of the
        # average is the larger of the combined jackknife error and the
        # chains' spread, which also holds modes slower than the window
        obs = np.zeros((C, nT, 6)); err = np.zeros((C, nT, 6))
        for c in range(C):
            for t in range(nT):
                k = c * nT + t
                obs[c, t], err[c, t] = A.jackknife_observables(ser[:, k, 0], ser[:, k, 1], float(inp.tems[t]), N, 40)
        mean = obs.mean(axis=0)
        half = ser.shape[0] // 2
        e_halves = np.array([[ser[:half, c * nT + t, 0].mean() / N, ser[half:, c * nT + t, 0].mean() / N]
                             for t in range(nT) for c in range(C)]).reshape(nT, C, 2).mean(axis=1)
        sig = np.sqrt((err ** 2).sum(axis=0)) / C
        if C > 1:
            sig = np.maximum(sig, obs.std(axis=0, ddof=1) / np.sqrt(C))
        out[kind] = {
            "sweeps": int(units * pss), "seconds": secs, "chains": C,
            "site_updates_per_s": ups,
            # every chain yields an independent sample per 2 tau sweeps
            "independent_samples_per_s": float(np.sum(C * sweeps_per_s / (2.0 * tau))),
            "per_slot_samples_per_s": (C * sweeps_per_s / (2.0 * tau)).tolist(),
            "tau_int_E": tau_e.mean(axis=0).tolist(), "tau_int_absM": tau_m.mean(axis=0).tolist(),
            "tau_int_binning_E": [analysis.binning_tau(ser[:, t, 0]) for t in range(nT)],
            "acceptance": acc.tolist(), "kernel": eng.sweep_kernel()[0],
            "observables": mean.tolist(), "sigma": sig.tolist(),
            "E_per_site_first_second_half": e_halves.tolist(),
            "chain_spread_over_jackknife": (obs.std(axis=0, ddof=1) / np.maximum(err.mean(axis=0), 1e-300)).max(
                axis=1).tolist() if C > 1 else None,
        }
    eng.close()
    gains = np.asarray(out["learned"]["per_slot_samples_per_s"]) / np.asarray(out["plain"]["per_slot_samples_per_s"])
    # every observable of every slot, learned against plain at 3 sigma (the
    # criterion over K comparisons: |z| <= 3 except ceil(1 + 0.0027 K) of them,
    # none beyond the Bonferroni bound of two-sided 1%)
    zl = (np.asarray(out["learned"]["observables"]) - np.asarray(out["plain"]["observables"])) / np.sqrt(
        np.asarray(out["learned"]["sigma"]) ** 2 + np.asarray(out["plain"]["sigma"]) ** 2)
    K = zl.size
    az = np.abs(zl)
    over = int((az > 3.0).sum())
    allowed = int(np.ceil(1 + 0.0027 * K))
    import math
    lo, hi = 0.0, 10.0
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if K * math.erfc(mid / math.sqrt(2.0)) > 0.01:
            lo = mid
        else:
            hi = mid
    passed = bool(over <= allowed and np.all(az <= hi))
    if rank == 0:
        line = {
            "metric": "independent samples/s", "value": out["learned"]["independent_samples_per_s"],
            "unit": "samples/s", "n_gpus": 1, "steps": a.measure_sweeps, "warmup": 500,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32",
            "data": "synthetic",
            "config": _config(inp, ham, a.workload) | {"proposal": "learned vs plain", "independent_chains": C,
                                                       "plain_sweeps": a.plain_sweeps,
                                                       "equilibration_sweeps": a.equil_sweeps,
                                                       "learned_sweeps": a.measure_sweeps},
            "plain": out["plain"], "learned": out["learned"],
            "ratio_independent_samples": out["learned"]["independent_samples_per_s"]
            / out["plain"]["independent_samples_per_s"],
            # per temperature slot: learned / plain independent samples/s
            "gain_per_slot": gains.tolist(),
            "gain_geomean": float(np.exp(np.mean(np.log(gains)))),
            "gain_min": float(gains.min()), "gain_max": float(gains.max()),
            "slots_with_gain_ge_2": int((gains >= 2.0).sum()),
            "observables_3sigma": {"names": list(A.OBSERVABLES), "z": zl.tolist(), "comparisons": K,
                                   "over_3sigma": over, "allowed_over_3sigma": allowed, "bonferroni_z": hi,
                                   "worst_abs_z": float(az.max()), "pass": passed},
            "training": {"pairs": int(rows), "collect_s": t_collect, "steps": a.train_steps, "batch": 4096,
                         "seconds": t_train, "loss_first": float(np.mean(loss[:20])),
                         "loss_last": float(np.mean(loss[-50:]))},
        }
        print(json.dumps(line), flush=True)


def _traffic(key, units_per_launch):
    """DRAM bytes per launch of the dominant kernel from the ncu capture
    summarised in profiles/dram_traffic.json (bytes per site update of that
    kernel on a captured case, scaled by the site updates of one launch here;
    the traffic grows in proportion to the updates), or (None, None)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as fh:
        d = json.load(fh)
    e = d.get(key)
    if not e:
        return None, None
    return float(e["dram_bytes_per_update"]) * units_per_launch, e.get("capture")


def secondary_sc128(a, local):
    """The HBM-resident single-lattice workload (SC 128^3 x 64 replicas) as a
    second figure: a separate process of this script, device-timed steps only."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "sc128_pt", "--steps", "5", "--warmup", "3",
           "--no-cpu-baseline", "--no-secondary", "--no-e2e"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", str(local)))
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env)
    except subprocess.TimeoutExpired:
        return {"workload": "sc128_pt", "error": "timed out"}
    for ln in r.stdout.splitlines()[::-1]:
        if ln.startswith("{"):
            d = json.loads(ln)
            return {"workload": "sc128_pt", "value": d["value"], "unit": d["unit"], "ms_per_step": d["ms_per_step"],
                    "steps": d["steps"], "roofline": d["roofline"], "clocks": d.get("clocks"),
                    "config": d["config"]}
    return {"workload": "sc128_pt", "error": (r.stderr or r.stdout)[-400:]}


def batch_bench(a, ws, rank, local):
    """512 independent SC lattices (L in {8..48}, seed 3) x 16 PT replicas in
    one batch: one handle per lattice size, lattices of a size as replica
    groups, every swap interval of every lattice in replayed CUDA graphs, the
    sweep kernel per size and the units per graph chosen by the autotuner."""
    import torch

    from espins_gb300.lib import Batch, Engine
    from espins_gb300.tables import build_hamiltonian
    from espins_gb300.workloads import batch_lattice_mcin, batch_lattice_sizes
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sizes = batch_lattice_sizes(512, 3)
    if a.only_L is not None:
        sizes = {L: c for L, c in sizes.items() if L == a.only_L}
    if a.max_lattices is not None:
        sizes = {L: min(c, a.max_lattices) for L, c in sizes.items()}
    reduced = a.only_L is not None or a.max_lattices is not None
    stream = torch.cuda.Stream(dev)
    engines, upd_per_unit, nsites, starts_h = [], 0, 0, []
    total_units = a.warmup + a.steps + 64
    scheds = []
    for L, count in sizes.items():
        inp = batch_lattice_mcin(L)
        ham = build_hamiltonian(inp, check=False)
        R = 16 * count
        e = Engine(ham.n, ham.num_atoms, ham.supercell, R)
        e.upload(ham)
        e.set_temperatures(np.tile(inp.tems, count))
        e.set_pt_groups(16)
        e.set_stream(stream.cuda_stream)
        # one random configuration per lattice (pt.F90:448-459 starts every
        # replica of a lattice from the same one)
        s0 = _uniform_spins(count, ham.n, ham.mag, a.seed + 7 * L)
        starts_h.append(np.repeat(s0, 16, axis=0))
        e.set_spins(starts_h[-1])
        sched = e.schedule(0, total_units * 10, 1, pt=True, pt_steps_swap=10, seed=3000 + L + 1000 * rank,
                           binning_level=[1, 2, 3, 4, 5])
        scheds.append(sched)
        e.begin(sched)
        engines.append(e)
        upd_per_unit += 10 * ham.n * R
        nsites += ham.n * count
    b = Batch(engines, stream.cuda_stream)
    if a.geometry or a.tile:
        fixed = [int(x) for x in (a.geometry or a.tile).split(",")]
        for e in engines:
            if a.geometry:
                e.set_cluster_geometry(*fixed)
                e.set_sweep_kernel("cluster")
            else:
                e.set_tile_geometry(*fixed)
                e.set_sweep_kernel("tile")
        b.set_units_per_graph(1)
        tuning = {"units_per_graph": 1, "kernel": "cluster" if a.geometry else "tile", "fixed_geometry": fixed}
    else:
        tuning = b.tune(units=2)
    b.advance(a.warmup)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    l0 = sum(e.launch_count() for e in engines)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    torch.cuda.synchronize(dev)
    torch.cuda.nvtx.range_push("timed")     # lets a profiler take the timed launches only
    for k in range(a.steps):
        starts[k].record(stream)
        b.advance(1)
        ends[k].record(stream)
    torch.cuda.synchronize(dev)
    torch.cuda.nvtx.range_pop()
    launches = sum(e.launch_count() for e in engines) - l0
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    clocks = sampler.stop()
    b.close()
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())

    # the dominant kernel: the sweeps of the largest lattice size, timed live
    # on the same stream (whole sweeps of every replica, one launch of the
    # sweep kernel per call plus the slab transposes around it)
    big = int(np.argmax([e.n * e.R for e in engines]))
    eb = engines[big]
    kernel, _ = eb.sweep_kernel()
    nsw = 10
    eb.sweep(nsw, 10 ** 9, a.seed)
    torch.cuda.synchronize(dev)
    k0 = eb.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    ev0.record(stream)
    for r in range(reps):
        eb.sweep(nsw, 10 ** 9 + (r + 1) * nsw, a.seed)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    sweep_launches = eb.launch_count() - k0
    kern_launches = reps if kernel == "cluster" else sweep_launches
    per_launch_s = ev0.elapsed_time(ev1) * 1e-3 / kern_launches
    upd_per_launch = nsw * reps * eb.n * eb.R / kern_launches
    peak, peak_kind = _peaks()
    achieved = 24.0 * upd_per_launch / per_launch_s / 1e9
    # the capture of the kernel the autotuner chose for that size
    traffic, capture = _traffic(f"batch512_pt:L{list(sizes)[big]}" + ("" if kernel == "cluster" else f":{kernel}"),
                                upd_per_launch)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_capture": capture,
                "kernel": {"cluster": "k_sweep_cluster", "tile": "k_sweep_tile"}.get(kernel, "k_sweep_ell"),
                "lattice": f"L={list(sizes)[big]} x {eb.R} replicas",
                "site_updates_per_launch": upd_per_launch, "launch_us": per_launch_s * 1e6,
                "timing": "CUDA events around whole-sweep calls (each: the sweep kernel plus its two slab "
                          "transposes) on the launching stream",
                "peak_source": peak_kind, "step_rate_frac": 24.0 * (a.steps * upd_per_unit / (ms * 1e-3)) / 1e9 / peak}

    # end to end through the C ABI, one job: every lattice's spin_matrix from
    # host memory (FP64), esp_begin, the steps through a new batch, the
    # results of every lattice and its final spins back to host memory
    torch.cuda.synchronize(dev)
    t1 = time.perf_counter()
    for e, s0, sched in zip(engines, starts_h, scheds):
        e.set_spins(s0)
        e.begin(sched)
    b2 = Batch(engines, stream.cuda_stream)
    b2.set_units_per_graph(tuning["units_per_graph"])
    b2.advance(a.steps)
    res = [e.collect() for e in engines]
    outs = [e.get_spins() for e in engines]
    t_e2e = time.perf_counter() - t1
    b2.close()
    if ws > 1:
        import torch.distributed as dist
        te = torch.tensor([t_e2e], dtype=torch.float64)
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
        t_e2e = float(te.item())
    h2d = sum(x.nbytes for x in starts_h)
    d2h = sum(o.nbytes for o in outs) + sum(
        r["data"].nbytes + r["pm"].nbytes + r["binning"].nbytes + r["num_swaps"].nbytes + r["rejected"].nbytes
        + r["energy"].nbytes + r["map"].nbytes for r in res)
    for e in engines:
        e.close()
    value = a.steps * upd_per_unit / (ms * 1e-3)
    if rank == 0:
        line = {
            "metric": "site updates/s", "value": ws * value, "unit": "site updates/s", "n_gpus": ws,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _batch_config(sizes) | ({"reduced": "a subset of the 512 lattices (profiling case)"}
                                              if reduced else {}),
            "roofline": roofline,
            "e2e": {"value": ws * a.steps * upd_per_unit / t_e2e, "unit": "site updates/s",
                    "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps, "steps": a.steps,
                    "path": "per lattice size: esp_set_spins + esp_begin; esp_batch_advance; per lattice size: "
                            "esp_collect + esp_get_spins (one job: the spins cross once each way, FP64)"},
            "gpu_launches": int(launches), "clocks": clocks, "tuning": tuning,
        }
        if not a.no_cpu_baseline and not reduced:
            threads = os.cpu_count() or 1
            v, sec, detail = batch_port_rate(sizes, threads, a.seed, 2, 1)
            line["cpu_baseline"] = {"value": v, "unit": "site updates/s", "cores": min(threads, 16), "kind": "port",
                                    "sample": "one lattice of each size (16 temperatures on 16 threads), 1 untimed + "
                                              "2 timed swap intervals of 10 sweeps, weighted by the lattice counts"}
        if a.secondary and not reduced:
            line["secondary"] = secondary_sc128(a, local)
        print(json.dumps(line), flush=True)


def main():
    a = _args()
    ws, rank, local = _dist()
    if a.proposal == "compare":
        learned_compare(a, rank, local)
        return
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if a.workload == "batch512_pt" and a.impl == "ours":
        batch_bench(a, ws, rank, local)
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    if a.impl == "reference":
        reference_arm(a, ws, rank)
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch

    from espins_gb300.lib import Engine
    from espins_gb300.tables import build_hamiltonian
    from espins_gb300.workloads import workload
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    inp = workload(a.workload, L=a.L, replicas=a.replicas)
    ham = build_hamiltonian(inp, check=False)
    R, N = inp.tems_num, ham.n
    pss = inp.pt_steps_swap if inp.pt else 1
    sweeps_per_step = pss * inp.steps_measure
    updates_per_step = sweeps_per_step * N * R
    seed = a.seed + 1000 * rank
    spins0 = _uniform_spins(R, N, ham.mag, seed)
    stream = torch.cuda.current_stream(dev)
    eng = Engine(N, ham.num_atoms, ham.supercell, R, inp.boundary_open)
    eng.upload(ham)
    eng.set_temperatures(inp.tems)
    eng.set_stream(stream.cuda_stream)
    if a.proposal == "learned":
        # an untrained network (the learned sampler's cost does not depend on its weights)
        eng.lp_init(seed=seed)
        eng.lp_set_engine(a.lp_engine)
        eng.set_proposal("learned")
    _, ncol = eng.colouring()
    mode = 1 if inp.mcarlo_mode.startswith("const") else 0
    total_units = a.warmup + a.steps
    # the library's autotuner picks the sweep kernel and cluster geometry on
    # units that serve as extra warm-up; the run then starts over
    from espins_gb300.lib import Batch
    eng.set_spins(spins0)
    eng.begin(eng.schedule(0, 64 * pss, inp.steps_measure, pt=inp.pt, pt_steps_swap=pss, mode=mode,
                           tilt=inp.tilt_angles_max, seed=seed + 7))
    with Batch([eng]) as tb:
        tuning = tb.tune(units=2)
    if a.tile:
        eng.set_tile_geometry(*(int(x) for x in a.tile.split(",")))
        eng.set_sweep_kernel("tile")
    sched = eng.schedule(0, total_units * pss, inp.steps_measure, pt=inp.pt, pt_steps_swap=pss, mode=mode,
                         tilt=inp.tilt_angles_max, seed=seed, binning_level=[1, 2, 3, 4, 5])
    eng.set_spins(spins0)
    eng.begin(sched)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(a.warmup):
        eng.advance(1)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    l0 = eng.launch_count()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    torch.cuda.nvtx.range_push("timed")     # lets a profiler take the timed launches only
    for k in range(a.steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        eng.advance(1)
        ends[k].record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize(dev)
    launches = eng.launch_count() - l0
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    clocks = sampler.stop()
    res = eng.collect()

    # sweep-kernel duration, live: back-to-back sweeps on the same stream
    # (the ELL kernel runs one colour class per launch, the cluster-resident
    # kernel many whole sweeps per launch)
    kernel, csize = eng.sweep_kernel()
    nsw = max(4, min(200, int(2e8 // max(N * R, 1))))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    eng.sweep(2, 10 ** 9, seed)
    torch.cuda.synchronize(dev)
    k0 = eng.launch_count()
    ev0.record(stream)
    eng.sweep(nsw, 10 ** 9 + 2, seed)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    sweep_launches = eng.launch_count() - k0
    sweep_ms = ev0.elapsed_time(ev1)
    per_launch_s = sweep_ms * 1e-3 / sweep_launches
    bytes_per_launch = 24.0 * N * R * nsw / sweep_launches
    if kernel == "learned":
        flop_per_launch = float(LP_FLOP) * N * R * nsw / sweep_launches
        peak, peak_kind = _peaks("tensor")
        achieved = flop_per_launch / per_launch_s / 1e12
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": None,
                    "kernel": "k_sweep_lp_tc" if a.lp_engine == "tcgen05" else "k_sweep_lp",
                    "flop_per_launch": flop_per_launch, "sweeps_timed": nsw, "launch_us": per_launch_s * 1e6,
                    "peak_source": peak_kind,
                    "hbm_equivalent_GBps": bytes_per_launch / per_launch_s / 1e9}
    else:
        peak, peak_kind = _peaks()
        achieved = bytes_per_launch / per_launch_s / 1e9
        traffic, capture = _traffic(a.workload, bytes_per_launch / 24.0)
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": traffic, "traffic_capture": capture,
                    "kernel": {"cluster": "k_sweep_cluster", "tile": "k_sweep_tile"}.get(kernel, "k_sweep_ell"),
                    "cluster_geometry": list(eng.cluster_geometry()) if kernel == "cluster" else None,
                    "tile_geometry": list(eng.tile_geometry()) if kernel == "tile" else None,
                    "bytes_per_launch": bytes_per_launch, "sweeps_timed": nsw,
                    "launch_us": per_launch_s * 1e6, "peak_source": peak_kind,
                    "note": (f"state {12 * N * R / 1e6:.0f} MB of spins"
                             + (" (L2-resident inside a step)" if 12 * N * R < 100e6 else " (HBM-resident)"))}

    # end to end through the C ABI with host buffers
    e2e_steps = max(1, min(a.steps, 50))
    t_e2e = None
    if not a.no_e2e:
        eng2 = Engine(N, ham.num_atoms, ham.supercell, R, inp.boundary_open)
        eng2.upload(ham)
        eng2.set_temperatures(inp.tems)
        if a.proposal == "learned":
            eng2.lp_init(seed=seed)
            eng2.lp_set_engine(a.lp_engine)
            eng2.set_proposal("learned")
        elif kernel == "cluster":
            eng2.set_cluster_geometry(*eng.cluster_geometry())
            eng2.set_sweep_kernel("cluster")
        elif kernel == "tile":
            eng2.set_tile_geometry(*eng.tile_geometry())
            eng2.set_sweep_kernel("tile")
        elif kernel == "ell":
            eng2.set_sweep_kernel("ell")
        sched2 = eng2.schedule(0, e2e_steps * pss, inp.steps_measure, pt=inp.pt, pt_steps_swap=pss, mode=mode,
                               tilt=inp.tilt_angles_max, seed=seed)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        eng2.set_spins(spins0)
        eng2.begin(sched2)
        eng2.advance(e2e_steps)
        r2 = eng2.collect()
        out_spins = eng2.get_spins()
        t_e2e = time.perf_counter() - t0
        eng2.close()
    # spin_matrix crosses as FP64 (3 x 8 B per spin) both ways
    h2d = 24 * N * R + 8 * R
    d2h = 24 * N * R + 8 * R * (6 + 3 + 4) + 8 * R * eng.num_freq()

    t_local = ms / 1e3
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_local], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
        if t_e2e is not None:
            te = torch.tensor([t_e2e], dtype=torch.float64)
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
            t_e2e = float(te.item())
    else:
        t_max = t_local
    value = ws * a.steps * updates_per_step / t_max
    e2e_value = ws * e2e_steps * updates_per_step / t_e2e if t_e2e else None
    if rank == 0:
        line = {
            "metric": "site updates/s", "value": value, "unit": "site updates/s", "n_gpus": ws,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * t_max / a.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16+f32" if a.proposal == "learned" else "f32",
            "data": "synthetic", "config": _config(inp, ham, a.workload) | {"proposal": a.proposal},
            "roofline": roofline,
            "e2e": None if e2e_value is None else {
                "value": e2e_value, "unit": "site updates/s", "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps, "steps": e2e_steps,
                "path": "esp_set_spins + esp_begin + esp_advance + esp_collect + esp_get_spins (one job: the "
                        "spins cross once each way, FP64)"},
            "gpu_launches": int(launches), "colours": ncol,
            "autotuner": {"kernel": tuning["kernel"][0], "cluster_geometry": tuning["cluster_geometry"][0],
                          "ell_us_per_unit": tuning["ell_us"][0], "cluster_us_per_unit": tuning["cluster_us"][0]},
            "clocks": clocks,
            "swap_acceptance": float(np.mean(res["num_swaps"][:, 1] / np.maximum(res["num_swaps"][:, 0], 1))),
        }
        if not a.no_cpu_baseline:
            threads = os.cpu_count() or 1
            v, info = cpu_baseline(inp, ham, a.cpu_seconds, threads, a.seed)
            line["cpu_baseline"] = {"value": v, "unit": "site updates/s", "cores": threads, "kind": "port",
                                    "sample": f"{info['swap_intervals']} swap intervals x "
                                              f"{info['sweeps_per_interval']} sweeps of all {R} temperatures "
                                              f"({info['updates']} site updates, {info['seconds']:.1f} s)"}
        print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
