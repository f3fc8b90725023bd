"""Benchmark of the two-channel NRG sweep on GB300.

Workload (one "step"): the full NRG_main sweep of the two-channel Anderson
model in the (Q,S) basis -- Lambda=2.5, U=0.3, eps_d=-0.15, Gamma1=Gamma2=0.01,
50 Wilson iterations, 3000 kept multiplets -- run through the engine's C ABI.
Every step rebuilds all device state from the impurity H_{-1}; the H_N
blocks alone (~0.8 GB per iteration) exceed the 129 MB L2, so no flush is
needed between steps.

Prints one JSON line (rank 0).  `value` is the sweep time in seconds measured
with CUDA events on the engine's stream (mean over the timed steps, max over
ranks) in the headline arithmetic (--precision, default fp64, the faster
form on this workload; "mixed": the largest blocks' Householder reduction
blocked, its trailing updates as split-BF16 products on the tensor cores);
`e2e` is the host wall time of the same call including every host<->device
copy of inputs and results.  The other form is timed once after the timed
region, and both forms are
checked against the reference's own outputs for the first five iterations
at 3000 kept (tests/golden/cfg1_2chQS_n5_k3000.npz) and against each other
over the whole sweep ("accuracy").

The CPU baseline is the oracle port of the reference algorithm on the host
cores over iterations 0-3 of the same workload -- iteration 3 is the first at
the full 3000 kept multiplets -- measured iteration by iteration; the sweep
total derived from it is labelled an estimate.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision mixed|fp64]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(model="2chQS", nsites=50, ncutoff=3000, lam=2.5, U=0.3, ed=-0.15, gamma1=0.01,
                gamma2_or_B=0.01)
WORKLOAD_NAME = ("two-channel Anderson NRG sweep, (Q,S) basis: Lambda=2.5, U=0.3, ed=-0.15, "
                 "Gamma1=Gamma2=0.01, 50 iterations, 3000 kept multiplets")
# Warm-up steps: the first 6 Wilson iterations of the same workload (they
# reach the full block sizes, so every kernel, code path and buffer is hot).
WARMUP_NSITES = 6
# CPU sample: iterations 0-3 of the workload itself.  Iterations 0-2 grow the
# basis (35, 462, 6435 states); iteration 3 is the first at the full kept count
# (about 45 600 states, blocks up to 4341), and every later iteration has
# about the same size (44 600-47 700 states, largest block 4240-4651).
CPU_ITERS = 4
# The reference's own routines on one core, from the run that made the
# fixture tests/golden/cfg1_2chQS_n5_k3000.npz (build container, x86):
# seconds per iteration of the same workload.
REF_FIXTURE = "cfg1_2chQS_n5_k3000"
# DRAM traffic of the tridiagonalization, from the ncu capture summarised in
# profiles/tridiag_fp64_2chQS.md: one n = 2400 block read 23.3 MB (its lower
# triangle, n^2/2 doubles, touched once; the rest of the passes hit L2) and
# wrote 4.4 MB.  The traffic of a launch therefore scales with the n^2 of its
# blocks, not with the flops: 4 B x n^2 x (1 + 4.4/23.3).
TRIDIAG_DRAM_BYTES_PER_ELEMENT = 4.0 * (1.0 + 4.4 / 23.3)


def max_over_ranks(dist, *vals):
    """Each value's maximum over the ranks (replicas only: the ranks share
    nothing but this reduction and the barriers)."""
    if dist is None:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in t)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0])); mx.append(float(s[1]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def sum_n3(result) -> float:
    return float(sum(float((it.bsize.astype(float) ** 3).sum()) for it in result.iters))


def sum_n2(result) -> float:
    return float(sum(float((it.bsize.astype(float) ** 2).sum()) for it in result.iters))


def cpu_sample(nthreads: int):
    """The oracle port (the reference's algorithm: element-wise H_N, LAPACK
    dspev per block, dgemm rotations) on iterations 0-3 of the workload, the
    blocks of an iteration spread over `nthreads` host threads.  Returns the
    wall time and the oracle's sweep (with its per-iteration seconds)."""
    from oracle import oracle as orc
    W = WORKLOAD
    t = time.perf_counter()
    s = orc.run(W["model"], CPU_ITERS, W["ncutoff"], W["lam"], W["U"], W["ed"], W["gamma1"], W["gamma2_or_B"],
                nthreads=nthreads, blas_threads=1)
    return time.perf_counter() - t, s


def sweep_estimate(per_iter_s, nsites: int) -> float:
    """Sweep total from measured iterations: the measured ones plus, for each
    later iteration, the last (full-size) one's time.  Later iterations have
    the same kept count and 0.94-1.26 times its sum of n_b^3 (the GPU's own
    full-size iterations take 0.94-1.25 times iteration 3's time)."""
    return float(sum(per_iter_s) + (nsites - len(per_iter_s)) * per_iter_s[-1])


def load_fixture(name: str):
    """A reference fixture in the shape of a sweep result (tests/golden)."""
    import numpy as np
    g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))

    class It:
        pass

    its = []
    for n in range(int(g["niters"])):
        it = It()
        it.qn, it.bsize, it.en = g[f"qn_{n}"], g[f"bsize_{n}"], g[f"en_{n}"]
        it.nkept, it.ecut = int(g[f"nkept_{n}"]), float(g[f"ecut_{n}"])
        it.kept_bsize, it.thermo, it.opavg = g[f"kept_bsize_{n}"], g[f"thermo_{n}"], g[f"opavg_{n}"]
        it.seconds = float(g[f"seconds_{n}"]) if f"seconds_{n}" in g else None
        its.append(it)
    return its


def bookkeeping_exact(gpu_iters, ref_iters) -> bool:
    import numpy as np
    for a, b in zip(gpu_iters, ref_iters):
        if not (np.array_equal(a.bsize, b.bsize) and a.nkept == b.nkept
                and np.array_equal(a.kept_bsize, b.kept_bsize)):
            return False
    return True


def sweep_errors(gpu_iters, ref_iters) -> dict:
    """Largest deviations of a GPU sweep from a reference on the same
    inputs: block eigenvalues relative to each iteration's largest level,
    E_cut likewise, the thermodynamics (beta, T, T chi, S at four
    temperatures) and the operator averages (<n_d> first) relative to their
    size; and whether every integer of the block bookkeeping agrees."""
    import numpy as np
    eig = thermo = tchi = opavg = nd = ecut = 0.0
    for a, b in zip(gpu_iters, ref_iters):
        ecut = max(ecut, abs(a.ecut - b.ecut) / max(1.0, float(np.abs(b.en).max())))
        scale = max(1.0, float(np.abs(b.en).max()))
        eig = max(eig, float(np.abs(np.asarray(a.en) - np.asarray(b.en)).max()) / scale)
        ta, tb = np.asarray(a.thermo, dtype=float).ravel(), np.asarray(b.thermo, dtype=float).ravel()
        rel = np.abs(ta - tb) / np.maximum(np.abs(tb), 1e-300)
        thermo = max(thermo, float(rel.max()))
        tchi = max(tchi, float(rel.reshape(-1, 4)[:, 2].max()))
        oa, ob = np.asarray(a.opavg, dtype=float), np.asarray(b.opavg, dtype=float)
        if ob.size:
            r = np.abs(oa - ob) / np.maximum(np.abs(ob), 1e-300)
            opavg = max(opavg, float(r.max()))
            nd = max(nd, float(r[0]))
    return {"eigenvalues_rel_max": eig, "ecut_rel_max": ecut, "n_d_rel_max": nd, "T_chi_rel_max": tchi,
            "thermo_rel_max": thermo, "opavg_rel_max": opavg,
            "bookkeeping_exact": bookkeeping_exact(gpu_iters, ref_iters),
            "iterations": min(len(gpu_iters), len(ref_iters))}


def run_reference_arm(args, rank: int):
    """The reference's algorithm on the host cores: the oracle port over
    iterations 0-3 of the workload (3 = the first at 3000 kept), measured
    iteration by iteration once; `value` is the sweep total derived from those
    measurements (labelled an estimate).  The reference's own binaries are
    built from its sources in the build container only (the sources are not
    on the GPU host, and x86 binaries do not run on its Arm cores); the
    fixture made there records the reference's own per-iteration seconds on
    one core, reported beside the port's."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    wall, s = cpu_sample(cores)
    per = [it.seconds for it in s.iters]
    value = sweep_estimate(per, WORKLOAD["nsites"])
    line = {"metric": "2ch NRG sweep s", "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": 1, "warmup": 0, "ms_per_step": value * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD_NAME, "parallelism": f"host threads over blocks ({cores})"},
            "estimate": {"value_is": "sweep total estimated from measured iterations: iterations 0-3 as "
                                     "measured plus 46 more at the measured time of iteration 3 (the first "
                                     "at 3000 kept)",
                         "measured_iterations": list(range(len(per))), "measured_s": per,
                         "timed_region_s": wall,
                         "passes": "the sample runs once: --steps/--warmup would repeat ~minutes of CPU work"},
            "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port",
                             "sample": (f"oracle port, iterations 0-3 of the workload measured "
                                        f"({', '.join(f'{x:.2f}' for x in per)} s; {wall:.1f} s in all), "
                                        "sweep total estimated as above")},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    ref = reference_seconds()
    if ref:
        line["reference_one_core"] = ref
    cbs, cdt, cn, _ = cpu_batch_sample(cores)
    line["batched"] = {"metric": "batched solves/s", "value": cbs, "unit": "solves/s",
                       "instances": cn, "seconds": cdt, "workload": BATCH_NAME,
                       "sample": f"oracle port on the first {cn} of {BATCH_INSTANCES} instances, one per thread"}
    print(json.dumps(line), flush=True)


def reference_seconds():
    """The reference's own per-iteration seconds (one core, build container)
    recorded in the full-size fixture."""
    try:
        its = load_fixture(REF_FIXTURE)
    except (OSError, KeyError):
        return None
    sec = [it.seconds for it in its if it.seconds is not None]
    if not sec:
        return None
    return {"iterations": list(range(len(sec))), "seconds": sec,
            "where": "reference routines (oracle/ref_harness), one core of the build container (x86)"}


BATCH_INSTANCES = 256
BATCH_SEED = 2024
BATCH_NAME = ("independent one-channel Anderson solves, (Q,Sz) basis: U~U[0.1,1], ed=-U/2+U[-0.1,0.1], "
              "Gamma log-U[1e-3,5e-2], B log-U[1e-8,1e-3], kept U{200..1000}, Lambda=2.5, 40 iterations, "
              f"seed {BATCH_SEED}")


def cpu_batch_sample(cores: int):
    """Oracle port on the first `cores` instances, one per host thread."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as orc
    from twochnrg_gb300.workloads import batched_qsz
    inst = batched_qsz(BATCH_INSTANCES, seed=BATCH_SEED)[:cores]
    orc.lib()
    t = time.perf_counter()
    with ThreadPoolExecutor(max_workers=cores) as ex:
        res = list(ex.map(lambda c: orc.run(c["model"], c["nsites"], c["ncutoff"], c["lam"], c["U"], c["ed"],
                                            c["gamma1"], c["gamma2_or_B"], nthreads=1), inst))
    dt = time.perf_counter() - t
    return len(inst) / dt, dt, len(inst), res


def batch_errors(gpu, refs) -> dict:
    """Errors of the GPU batch against the oracle on the instances the CPU
    sample ran: <n_d> and T chi (CalcSuscep at the four temperatures of each
    iteration) relative, and the kept counts."""
    import numpy as np
    nd = tchi = 0.0
    nk_ok = True
    for i, o in enumerate(refs):
        for n, it in enumerate(o.iters):
            nk_ok &= int(gpu.nkept[i, n]) == it.nkept
            a, b = gpu.thermo[i, n][:, 2], np.asarray(it.thermo)[:, 2]
            tchi = max(tchi, float((np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max()))
            nd = max(nd, abs(float(gpu.opavg[i, n, 0]) - it.opavg[0]) / max(abs(it.opavg[0]), 1e-300))
    return {"n_d_rel_max": nd, "T_chi_rel_max": tchi, "nkept_exact": bool(nk_ok), "instances": len(refs),
            "iterations": 40}


DM_WORKLOAD = dict(nsites=40, ncutoff=500, lam=2.5, U=0.5, ed=-0.25, gamma=0.02)
DM_TEMP, DM_BROAD, DM_NOMEGA = 1e-8, 0.6, 2000
DM_NAME = ("DM-NRG (FDM) spectral function of c_d, one-channel Anderson (Q,S): Lambda=2.5, U=0.5, ed=-0.25, "
           "Gamma=0.02, 40 iterations, 500 kept; T=1e-8, log-Gaussian b=0.6, 2000 frequencies "
           "+-logspace(-10, 0, 1000)")
DM_SAMPLE = dict(nsites=16, ncutoff=150, lam=2.5, U=0.5, ed=-0.25, gamma=0.02)
DM_SAMPLE_NOMEGA = 200
# The two-channel DM-NRG spectral function (--dm2ch): the two-channel sweep's
# model and kept count, T = 1e-8, b = 0.6, 2000 frequencies.
DM2_WORKLOAD = dict(nsites=50, ncutoff=3000, lam=2.5, U=0.3, ed=-0.15, gamma=0.01, gamma2=0.01, model="2chQS")
DM2_NAME = ("DM-NRG (FDM) spectral function of c_d, two-channel Anderson (Q,S): Lambda=2.5, U=0.3, ed=-0.15, "
            "Gamma1=Gamma2=0.01, 50 iterations, {ncutoff} kept; T=1e-8, log-Gaussian b=0.6, 2000 frequencies "
            "+-logspace(-10, 0, 1000)")
DM2_SAMPLE = dict(nsites=6, ncutoff=100, lam=2.5, U=0.3, ed=-0.15, gamma=0.01, gamma2=0.01, model="2chQS")


def dm_omegas(n):
    import numpy as np
    h = n // 2
    return np.concatenate([-np.logspace(0, -10, h), np.logspace(-10, 0, h)])


def gpu_dm(eng, W, nomega):
    """Forward sweep keeping the DM-NRG shells, backward sweep, Lehmann sums;
    device times of each phase (CUDA events on the engine stream)."""
    eng.sweep_dm(**W)
    fwd = eng.timing()["device_ms"]
    prm = eng.dm_params(temp=DM_TEMP, bbroad=DM_BROAD)
    eng.dm_backprop(prm)
    back = eng.timing()["dm_backprop_ms"]
    om, A = eng.lehmann(prm, omegas=dm_omegas(nomega))
    t = eng.timing()
    return fwd, back, t["dm_spectral_ms"], t["lehmann_ms"], t["lehmann_pairs"], t["lehmann_evals"], A


# The derivatives (--grad): d/d(eps_d, U, Gamma, B) of the one-channel
# Anderson model at Lambda=2.5, U=0.4, eps_d=-0.2, Gamma=0.015, B=1e-6, 1000
# kept, 45 iterations: <n_d> and T chi (four temperatures per iteration, 180
# from 1e-10 to 1) from the (Q,Sz) sweep, which carries the field, and
# A(omega) on 512 frequencies from the (Q,S) DM-NRG (T = 1e-8, b = 0.6), in
# which B does not enter.
GRAD_WORKLOAD = dict(nsites=45, ncutoff=1000, lam=2.5, U=0.4, ed=-0.2, gamma=0.015, B=1e-6)
GRAD_NOMEGA = 512
GRAD_NAME = ("derivatives of <n_d>, T chi(T) and A(omega) with respect to (eps_d, U, Gamma, B), one-channel "
             "Anderson: Lambda=2.5, U=0.4, ed=-0.2, Gamma=0.015, B=1e-6, 45 iterations, 1000 kept; (Q,Sz) sweep "
             "for <n_d> and T chi, (Q,S) DM-NRG (FDM, T=1e-8, b=0.6) for A(omega) on 512 frequencies "
             "+-logspace(-10, 0, 256)")


def fd_error(an, fd, floor=1e-3):
    """max |analytic - central difference| over max(max |fd|, floor)."""
    import numpy as np
    return float(np.abs(an - fd).max() / max(float(np.abs(fd).max()), floor))


def gpu_grad(local: int) -> dict:
    """The derivatives of the fifth configuration with their cost against
    the plain runs, checked against central differences of the GPU runs
    (step 1e-5 |p|; 1e-7 for B) and against the Hellmann-Feynman averages of
    the last iteration.  Runs on its own context, closed afterwards."""
    import numpy as np
    import twochnrg_gb300 as tg
    eng = tg.Engine(local)
    W = GRAD_WORKLOAD
    args_qsz = ("1chQSz", W["nsites"], W["ncutoff"], W["lam"], W["U"], W["ed"], W["gamma"], W["B"])
    k0 = eng.kernel_count
    t0 = time.perf_counter()
    g = eng.grad_forward(*args_qsz)
    grad_ms = eng.timing()["device_ms"]
    grad_wall = time.perf_counter() - t0
    launches = eng.kernel_count - k0
    eng.sweep(*args_qsz, fetch=False)
    plain_ms = eng.timing()["device_ms"]
    params = [W["ed"], W["U"], W["gamma"], W["B"]]
    names = ["eps_d", "U", "Gamma", "B"]
    fd_sweep = {}
    for k in range(4):
        h = 1e-7 if k == 3 else 1e-5 * abs(params[k])
        pp, pm = list(params), list(params)
        pp[k] += h
        pm[k] -= h
        rp = eng.sweep("1chQSz", W["nsites"], W["ncutoff"], W["lam"], pp[1], pp[0], pp[2], pp[3])
        rm = eng.sweep("1chQSz", W["nsites"], W["ncutoff"], W["lam"], pm[1], pm[0], pm[2], pm[3])
        # the derivatives are those of a fixed kept set: compare the
        # iterations before the first one at which a displaced sweep keeps
        # another set
        n = 0
        for a, b, c in zip(rp.iters, rm.iters, g.sweep.iters):
            if not (np.array_equal(a.kept_bsize, c.kept_bsize) and np.array_equal(b.kept_bsize, c.kept_bsize)):
                break
            n += 1
        fd_t = np.array([(a.thermo[:, 2] - b.thermo[:, 2]) / (2 * h) for a, b in zip(rp.iters[:n], rm.iters[:n])])
        fd_n = np.array([(a.opavg[0] - b.opavg[0]) / (2 * h) for a, b in zip(rp.iters[:n], rm.iters[:n])])
        fd_sweep[names[k]] = {"step": h, "iterations_compared": n,
                              "tchi_rel_err": fd_error(g.d_thermo[:n, k, :, 2], fd_t) if n else None,
                              "nd_rel_err": fd_error(g.d_opavg[:n, k, 0], fd_n) if n else None,
                              "max_abs_dtchi": float(np.abs(fd_t).max()) if n else None,
                              "tchi_abs_err_by_iteration": [float(f"{x:.3g}") for x in
                                                            np.abs(g.d_thermo[:n, k, :, 2] - fd_t).max(axis=1)]}
    # T chi and its derivatives on 64 temperatures log-spaced over [1e-10, 1e-2]
    # (the sweep's own temperatures reach down to about 3e-9 in 45 iterations;
    # below that the entries are null)
    temps = np.logspace(-10, -2, 64)
    tchi64, dtchi64 = g.tchi_on(temps)
    nul = lambda a: [None if not np.isfinite(x) else float(x) for x in a]  # noqa: E731
    tchi_grid = {"T": temps.tolist(), "tchi": nul(tchi64), "d_tchi": [nul(r) for r in dtchi64],
                 "covered": int(np.isfinite(tchi64).sum())}
    last = g.sweep.iters[-1]
    hf = {"dEgs_deps_d": float(g.d_egs[-1, 0]), "nd": float(last.opavg[0]),
          "dEgs_dB": float(g.d_egs[-1, 3]), "Szdot": float(last.opavg[1])}
    # A(omega): forward sweep with tangents, backward sweep, Lehmann sums
    om = dm_omegas(GRAD_NOMEGA)
    t1 = time.perf_counter()
    eng.grad_forward_dm(W["nsites"], W["ncutoff"], W["lam"], W["U"], W["ed"], W["gamma"])
    dm_fwd = eng.timing()["device_ms"]
    prm = eng.dm_params(temp=DM_TEMP, bbroad=DM_BROAD)
    eng.dm_backprop(prm)
    dm_back = eng.timing()["dm_backprop_ms"]
    _, A, dA = eng.lehmann_grad(prm, omegas=om)
    dm_spec = eng.timing()["dm_spectral_ms"]
    dm_wall = time.perf_counter() - t1
    plain = gpu_dm(eng, dict(nsites=W["nsites"], ncutoff=W["ncutoff"], lam=W["lam"], U=W["U"], ed=W["ed"],
                             gamma=W["gamma"]), GRAD_NOMEGA)
    kept0 = [it.kept_bsize for it in eng.fetch().iters]
    fd_dm = {}
    for k in range(3):
        h = 1e-5 * abs(params[k])
        out, same = [], True
        for sgn in (1, -1):
            q = list(params)
            q[k] += sgn * h
            out.append(gpu_dm(eng, dict(nsites=W["nsites"], ncutoff=W["ncutoff"], lam=W["lam"], U=q[1], ed=q[0],
                                        gamma=q[2]), GRAD_NOMEGA)[-1])
            same = same and all(np.array_equal(a.kept_bsize, b) for a, b in zip(eng.fetch().iters, kept0))
        fd = (out[0] - out[1]) / (2 * h)
        fd_dm[names[k]] = {"step": h, "kept_sets_equal": bool(same), "rel_err": fd_error(dA[k], fd, 0.0),
                           "max_abs_dA": float(np.abs(fd).max())}
    eng.close()
    return {"workload": GRAD_NAME, "unit": "s",
            "total_s": (grad_ms + dm_fwd + dm_back + dm_spec) * 1e-3,
            "sweep_grad_s": grad_ms * 1e-3, "sweep_plain_s": plain_ms * 1e-3, "sweep_grad_wall_s": grad_wall,
            "dm_grad_forward_s": dm_fwd * 1e-3, "dm_grad_backprop_s": dm_back * 1e-3,
            "dm_grad_spectral_s": dm_spec * 1e-3, "dm_grad_wall_s": dm_wall,
            "dm_plain_s": (plain[0] + plain[1] + plain[2]) * 1e-3,
            "fd_sweep": fd_sweep, "fd_spectral": fd_dm, "hellmann_feynman_last_iteration": hf,
            "tchi_64T": tchi_grid,
            "sweep_grad_launches": launches}


def run_grad(args, rank: int, local: int) -> None:
    """gpu_grad as its own JSON line."""
    import torch
    if rank != 0:
        return
    torch.cuda.set_device(local)
    d = gpu_grad(local)
    line = {"metric": "derivatives of the sweep observables and of A(omega)", "value": d.pop("total_s"),
            "unit": d.pop("unit"), "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
            "data": "synthetic (flat band Wilson chain)", "config": {"workload": d.pop("workload")}}
    line.update(d)
    print(json.dumps(line), flush=True)


def run_dm2ch(args, rank: int, local: int) -> None:
    """One pass of the two-channel DM-NRG spectral function: forward sweep
    keeping the shells, density-matrix backward sweep, Lehmann sums.  The
    reference's DM_NRG is one-channel only, so the CPU figure is the oracle's
    restatement on a reduced case."""
    import numpy as np
    import torch
    import twochnrg_gb300 as tg
    if rank != 0:
        return
    W = dict(DM2_WORKLOAD, ncutoff=args.dm2ch_ncutoff)
    torch.cuda.set_device(local)
    eng = tg.Engine(local)
    free0, _ = torch.cuda.mem_get_info(local)
    k0 = eng.kernel_count
    t0 = time.perf_counter()
    fwd, back, spec, leh, recs, evals, A = gpu_dm(eng, W, DM_NOMEGA)
    wall = time.perf_counter() - t0
    free1, _ = torch.cuda.mem_get_info(local)
    om = dm_omegas(DM_NOMEGA)
    k = int(np.argmin(np.abs(om - 1e-6)))
    line = {"metric": "two-channel DM-NRG spectral function", "value": (fwd + back + spec) * 1e-3, "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "dtype": "f64", "data": "synthetic (flat band Wilson chain)",
            "config": {"workload": DM2_NAME.format(ncutoff=W["ncutoff"])},
            "forward_sweep_s": fwd * 1e-3, "backprop_s": back * 1e-3, "spectral_s": spec * 1e-3,
            "lehmann_kernel_s": leh * 1e-3, "lehmann_records": recs, "lehmann_evals": evals,
            "lehmann_evals_per_s": evals / (leh * 1e-3) if leh > 0 else None, "wall_s": wall,
            "device_gb_held": (free0 - free1) / 1e9,
            "friedel_pi_gamma_A_1e-6": float(np.pi * (W["gamma"] + W["gamma2"]) * A[k]),
            "gpu_launches": eng.kernel_count - k0}
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        g = gpu_dm(eng, DM2_SAMPLE, DM_SAMPLE_NOMEGA)
        S = DM2_SAMPLE
        t = time.perf_counter()
        orc.dm_spectral(S["nsites"], S["ncutoff"], S["lam"], S["U"], S["ed"], S["gamma"], DM_TEMP, DM_BROAD,
                        omegas=dm_omegas(DM_SAMPLE_NOMEGA), model="2chQS", gamma2=S["gamma2"])
        line["cpu_baseline"] = {
            "value": time.perf_counter() - t, "unit": "s", "cores": 1, "kind": "port",
            "sample": (f"oracle restatement (single thread) on {S['nsites']} iterations, {S['ncutoff']} kept, "
                       f"{DM_SAMPLE_NOMEGA} frequencies, same T and b; GPU on that case: "
                       f"{(g[0] + g[1] + g[2]) * 1e-3:.3f} s")}
    print(json.dumps(line), flush=True)
    eng.close()


def gpu_batch(workers: int, device: int):
    import twochnrg_gb300 as tg
    from twochnrg_gb300.workloads import batched_qsz
    inst = batched_qsz(BATCH_INSTANCES, seed=BATCH_SEED)
    tg.sweep_batch(inst[:workers], nworkers=workers, device=device)  # warm-up
    res = tg.sweep_batch(inst, nworkers=workers, device=device)
    return BATCH_INSTANCES / res.seconds, res.seconds, res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-workers", type=int, default=8)
    ap.add_argument("--dm2ch", action="store_true",
                    help="only the two-channel DM-NRG spectral function (about 8 minutes and 190 GB at 3000 kept)")
    ap.add_argument("--dm2ch-ncutoff", type=int, default=DM2_WORKLOAD["ncutoff"])
    ap.add_argument("--grad", action="store_true",
                    help="the derivatives (sweep observables and A(omega)) with their checks, one JSON line")
    ap.add_argument("--precision", default="fp64", choices=["mixed", "fp64"],
                    help="arithmetic of the timed sweeps (the other form is timed once after them)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    if args.dm2ch:
        run_dm2ch(args, rank, local)
        return
    if args.grad:
        run_grad(args, rank, local)
        return
    dist = None
    if ws > 1:
        import torch.distributed as dist  # replicas only: used for barriers and the max over ranks
        dist.init_process_group("gloo")
    import numpy as np
    import twochnrg_gb300 as tg
    eng = tg.Engine(local)
    W = dict(WORKLOAD)
    prec = tg.PREC_MIXED if args.precision == "mixed" else tg.PREC_FP64
    other = tg.PREC_FP64 if prec == tg.PREC_MIXED else tg.PREC_MIXED
    warm = dict(W, nsites=WARMUP_NSITES)
    for i in range(args.warmup):
        # the first warm-up step is the whole sweep, so that every device buffer
        # has reached its final size before the timed steps (a buffer that grows
        # is freed and reallocated, and cudaFree synchronises the device)
        eng.sweep(**(W if i == 0 else warm), fetch=False, precision=prec)
    peak = eng.fp64_peak()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    k0 = eng.kernel_count
    dev_ms, wall, tim = [], [], []
    res = None
    for _ in range(args.steps):
        t = time.perf_counter()
        res = eng.sweep(**W, fetch=True, precision=prec)
        wall.append(time.perf_counter() - t)
        dev_ms.append(res.timing["device_ms"])
        tim.append(res.timing)
    launches = eng.kernel_count - k0
    ck = clocks.stop()
    value = statistics.mean(dev_ms) / 1e3
    e2e = statistics.mean(wall)
    value, e2e = max_over_ranks(dist, value, e2e)
    if rank != 0:
        return
    T = tim[-1]
    tri_ms = T["tridiag_ms"]
    achieved = T["tridiag_flops"] / (tri_ms * 1e-3) / 1e12
    traffic = None
    if T["tridiag_launches"] and prec == tg.PREC_FP64:
        traffic = TRIDIAG_DRAM_BYTES_PER_ELEMENT * sum_n2(res) / T["tridiag_launches"]
    w_full = sum_n3(res)
    names = {tg.PREC_MIXED: "mixed", tg.PREC_FP64: "fp64"}
    line = {
        "metric": "2ch NRG sweep s", "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+bf16 (split-BF16 tensor-core products, FP64 elsewhere)" if prec == tg.PREC_MIXED else "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "precision": names[prec], "parallelism": f"replicas x{args.gpus}",
                   "l2": "working set (H_N blocks ~0.8 GB per iteration) larger than L2; no flush",
                   "warmup_step": f"the whole sweep once, then its first {WARMUP_NSITES} iterations"},
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(T["h2d_bytes"]),
                "d2h_bytes_per_step": int(T["d2h_bytes"])},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "kernel": ("Householder reduction, blocked: FP64 panels + tensor-core "
                                                 "trailing products" if prec == tg.PREC_MIXED else
                                                 "Householder reduction (FP64)"),
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "peak_source": "measured by bench.py: DFMA register loop on all SMs (FP64 has no "
                                    "entry in MEASURED_PEAKS.json)",
                     "algorithmic": "4/3 sum_b n_b^3 flops per iteration"},
        "clocks": ck,
        "phases_ms": {k: T[k] for k in ("assemble_ms", "tridiag_ms", "tridiag_eig_ms", "vectors_ms",
                                          "backtransform_ms", "cut_ms", "update_ms")},
        "sum_n3": w_full,
        "gpu_iteration_ms": [round(it.device_ms, 3) for it in res.iters],
    }
    # the other arithmetic, once, and the two forms against each other
    r2 = eng.sweep(**W, fetch=True, precision=other)
    line[names[other]] = {"value": r2.timing["device_ms"] / 1e3, "unit": "s",
                          "e2e_s": r2.timing["total_ms"] / 1e3,
                          "phases_ms": {k: r2.timing[k] for k in ("tridiag_ms", "tridiag_eig_ms", "vectors_ms",
                                                                  "backtransform_ms", "update_ms")}}
    mixed_s = value if prec == tg.PREC_MIXED else r2.timing["device_ms"] / 1e3
    fp64_s = value if prec == tg.PREC_FP64 else r2.timing["device_ms"] / 1e3
    line["mixed_vs_fp64"] = {"speedup": fp64_s / mixed_s, "mixed_s": mixed_s, "fp64_s": fp64_s}
    rm, rf = (res, r2) if prec == tg.PREC_MIXED else (r2, res)
    line["accuracy"] = {"mixed_vs_fp64_sweep": dict(sweep_errors(rm.iters, rf.iters),
                                                    sample="whole 50-iteration sweep, mixed against FP64 GPU")}
    # both forms against the reference's own outputs at 3000 kept
    try:
        ref_its = load_fixture(REF_FIXTURE)
    except OSError:
        ref_its = None
    if ref_its:
        for p, nm in ((tg.PREC_FP64, "fp64"), (tg.PREC_MIXED, "mixed")):
            g = eng.sweep(**dict(W, nsites=len(ref_its)), fetch=True, precision=p)
            line["accuracy"][f"sweep_full_{nm}"] = dict(
                sweep_errors(g.iters, ref_its),
                sample=f"iterations 0-{len(ref_its) - 1} of the workload at 3000 kept, GPU against the "
                       "reference's own routines (fixture tests/golden/cfg1_2chQS_n5_k3000.npz)")
    # second half of the metric: batched independent solves per second
    bs, bsec, bres = gpu_batch(args.batch_workers, local)
    line["batched"] = {"metric": "batched solves/s", "value": bs * (ws if dist else 1), "unit": "solves/s",
                       "instances": BATCH_INSTANCES, "seconds": bsec, "workers": args.batch_workers,
                       "workload": BATCH_NAME, "timing": "host wall time of nrg_sweep_batch"}
    # DM-NRG spectral function (one-channel: the reference's DM_NRG is d = 4 only)
    gpu_dm(eng, DM_WORKLOAD, 200)  # warm-up
    fwd, back, spec, leh, pairs, evals, _ = gpu_dm(eng, DM_WORKLOAD, DM_NOMEGA)
    line["dm_spectral"] = {
        "workload": DM_NAME, "unit": "ms", "forward_sweep_ms": fwd, "backprop_ms": back, "spectral_ms": spec,
        "total_ms": fwd + back + spec, "lehmann_kernel_ms": leh, "lehmann_pairs": pairs,
        "lehmann_evals": evals, "lehmann_evals_per_s": evals / (leh * 1e-3) if leh > 0 else None,
        "lehmann_bound": "fp64 (one exp per nonzero Lehmann record and frequency)"}
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        cwall, cs = cpu_sample(cores)
        per = [it.seconds for it in cs.iters]
        est = sweep_estimate(per, W["nsites"])
        gpu_first = [it.device_ms / 1e3 for it in res.iters[:len(per)]]
        line["cpu_baseline"] = {
            "value": est, "unit": "s", "cores": cores, "kind": "port",
            "estimate": True,
            "sample": (f"oracle port on iterations 0-{len(per) - 1} of the workload (iteration 3: the first at "
                       f"3000 kept), measured per iteration: {', '.join(f'{x:.2f}' for x in per)} s; sweep total "
                       f"estimated as those plus {W['nsites'] - len(per)} iterations at iteration 3's time"),
            "measured_s": per, "timed_region_s": cwall,
            "gpu_same_iterations_s": gpu_first,
            "measured_ratio_same_iterations": sum(per) / max(sum(gpu_first), 1e-12),
            "measured_ratio_full_size_iteration": per[-1] / max(gpu_first[-1], 1e-12)}
        ref = reference_seconds()
        if ref:
            line["cpu_baseline"]["reference_one_core"] = ref
        # the port's sample against the GPU on the same iterations (both forms above)
        line["accuracy"]["port_vs_gpu_first_iterations"] = dict(
            sweep_errors(res.iters[:len(cs.iters)], cs.iters),
            sample=f"iterations 0-{len(per) - 1} at 3000 kept, GPU ({names[prec]}) against the oracle port")
        cbs, cdt, cn, crefs = cpu_batch_sample(cores)
        line["batched"]["cpu_baseline"] = {
            "value": cbs, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"oracle port on the first {cn} instances, one per thread: {cdt:.2f} s"}
        line["batched"]["accuracy"] = dict(batch_errors(bres, crefs),
                                           sample=f"the first {cn} instances, GPU batch against the oracle")
        # DM-NRG: GPU and the oracle port on the same reduced case (the port
        # evaluates every frequency with dense products, as DM_NRG does)
        from oracle import oracle as orc
        g = gpu_dm(eng, DM_SAMPLE, DM_SAMPLE_NOMEGA)
        t = time.perf_counter()
        o_dm = orc.dm_spectral(DM_SAMPLE["nsites"], DM_SAMPLE["ncutoff"], DM_SAMPLE["lam"], DM_SAMPLE["U"],
                               DM_SAMPLE["ed"], DM_SAMPLE["gamma"], DM_TEMP, DM_BROAD,
                               omegas=dm_omegas(DM_SAMPLE_NOMEGA))
        cdm = (time.perf_counter() - t) * 1e3
        A_gpu, A_ref = np.asarray(g[6]), np.asarray(o_dm[1])
        line["accuracy"]["dm_spectral"] = {
            "A_rel_max": float((np.abs(A_gpu - A_ref) / np.maximum(np.abs(A_ref), 1e-300)).max()),
            "A_abs_max_over_max_A": float(np.abs(A_gpu - A_ref).max() / np.abs(A_ref).max()),
            "sample": (f"one-channel DM-NRG, {DM_SAMPLE['nsites']} iterations, {DM_SAMPLE['ncutoff']} kept, "
                       f"{DM_SAMPLE_NOMEGA} frequencies, GPU against the FP64 oracle")}
        line["dm_spectral"]["cpu_baseline"] = {
            "value": cdm, "unit": "ms", "cores": 1, "kind": "port",
            "sample": (f"oracle port (single thread) on {DM_SAMPLE['nsites']} iterations, {DM_SAMPLE['ncutoff']} "
                       f"kept, {DM_SAMPLE_NOMEGA} frequencies, same T and b; GPU on that case: "
                       f"{g[0] + g[1] + g[2]:.1f} ms")}
    if not dist:
        # the derivatives (fifth configuration) on a context of their own;
        # a failure there is reported in the line, not raised
        try:
            line["derivatives"] = gpu_grad(local)
        except Exception as e:  # noqa: BLE001
            line["derivatives"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
