"""Benchmark of the two-channel NRG sweep on GB300.

Workload (one "step"): the full NRG_main sweep of the two-channel Anderson
model in the (Q,S) basis -- Lambda=2.5, U=0.3, eps_d=-0.15, Gamma1=Gamma2=0.01,
50 Wilson iterations, 3000 kept multiplets -- run through the engine's C ABI.
Every step rebuilds all device state from the impurity H_{-1}; the H_N
blocks alone (~0.8 GB per iteration) exceed the 129 MB L2, so no flush is
needed between steps.

Prints one JSON line (rank 0).  `value` is the sweep time in seconds measured
with CUDA events on the engine's stream (mean over the timed steps, max over
ranks); `e2e` is the host wall time of the same call including every
host<->device copy of inputs and results.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
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
# CPU sample: the same model and parameters with 600 kept multiplets, 8
# iterations; scaled to the full sweep by the ratio of sum_b n_b^3 (the
# dspev cost that dominates the CPU path).
CPU_SAMPLE = dict(model="2chQS", nsites=8, ncutoff=600, lam=2.5, U=0.3, ed=-0.15, gamma1=0.01,
                  gamma2_or_B=0.01)
# DRAM traffic of the tridiagonalization, from the ncu capture summarised in
# profiles/tridiag_fp64_2chQS.md: one n = 2400 block read 46 MB (its n^2
# doubles, touched once; the rest of the passes hit L2) and wrote 5 MB.  The
# traffic of a launch therefore scales with the n^2 of its blocks, not with
# the flops: 8 B x n^2 x (1 + 5/46).
TRIDIAG_DRAM_BYTES_PER_ELEMENT = 8.0 * (1.0 + 5.0 / 46.0)


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


def cpu_sample(nthreads: int, want_result: bool = False):
    """Time the oracle port (the reference's algorithm on the host cores)."""
    from oracle import oracle as orc
    t = time.perf_counter()
    s = orc.run(CPU_SAMPLE["model"], CPU_SAMPLE["nsites"], CPU_SAMPLE["ncutoff"], CPU_SAMPLE["lam"],
                CPU_SAMPLE["U"], CPU_SAMPLE["ed"], CPU_SAMPLE["gamma1"], CPU_SAMPLE["gamma2_or_B"],
                nthreads=nthreads, blas_threads=1)
    dt = time.perf_counter() - t
    return (dt, sum_n3(s), s) if want_result else (dt, sum_n3(s))


def sweep_errors(gpu, ref) -> dict:
    """Largest deviations of a GPU sweep from the oracle's on the same
    inputs: block eigenvalues relative to each iteration's largest level,
    the thermodynamics (beta, T, T chi, S at four temperatures) and the
    operator averages (<n_d> first) relative to their size."""
    import numpy as np
    eig = thermo = tchi = opavg = nd = 0.0
    for a, b in zip(gpu.iters, ref.iters):
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
    return {"eigenvalues_rel_max": eig, "n_d_rel_max": nd, "T_chi_rel_max": tchi, "thermo_rel_max": thermo,
            "opavg_rel_max": opavg, "iterations": min(len(gpu.iters), len(ref.iters))}


# sum_b n_b^3 over the 50 iterations of the full workload, from the block
# sizes the sweep produces (identical on CPU and GPU: the bookkeeping is exact).
def full_sum_n3_from(result) -> float:
    return sum_n3(result)


def run_reference_arm(args, rank: int):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    steps = []
    for _ in range(args.warmup):
        cpu_sample(cores)
    for _ in range(args.steps):
        steps.append(cpu_sample(cores))
    dt = statistics.mean(s[0] for s in steps)
    w_sample = steps[0][1]
    w_full = FULL_SUM_N3
    value = dt * w_full / w_sample
    sample = (f"oracle port of the reference sweep (same model/parameters, 600 kept, 8 iterations) "
              f"timed at {dt:.2f} s on {cores} threads, scaled by sum n^3 ratio {w_full / w_sample:.1f}")
    line = {"metric": "2ch NRG sweep s", "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD_NAME, "parallelism": "host threads over blocks"},
            "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    cbs, cdt, cn = cpu_batch_sample(cores)
    line["batched"] = {"metric": "batched solves/s", "value": cbs, "unit": "solves/s",
                       "instances": cn, "seconds": cdt, "workload": BATCH_NAME,
                       "sample": f"oracle port on the first {cn} of {BATCH_INSTANCES} instances, one per thread"}
    print(json.dumps(line), flush=True)


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
        list(ex.map(lambda c: orc.run(c["model"], c["nsites"], c["ncutoff"], c["lam"], c["U"], c["ed"],
                                      c["gamma1"], c["gamma2_or_B"], nthreads=1), inst))
    dt = time.perf_counter() - t
    return len(inst) / dt, dt, len(inst)


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
    return BATCH_INSTANCES / res.seconds, res.seconds


# Fixed by the workload: sum over the 50 iterations of n_b^3 for the block
# structure the sweep produces (the bookkeeping is exact, so CPU and GPU agree;
# the GPU arm reports the value it measured as "sum_n3").
FULL_SUM_N3 = 1.6993633731293001e13


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-workers", type=int, default=16)
    ap.add_argument("--dm2ch", action="store_true",
                    help="only the two-channel DM-NRG spectral function (about 8 minutes and 190 GB at 3000 kept)")
    ap.add_argument("--dm2ch-ncutoff", type=int, default=DM2_WORKLOAD["ncutoff"])
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    if args.dm2ch:
        run_dm2ch(args, rank, local)
        return
    dist = None
    if ws > 1:
        import torch.distributed as dist  # replicas only: used for barriers and the max over ranks
        dist.init_process_group("gloo")
    import twochnrg_gb300 as tg
    eng = tg.Engine(local)
    W = dict(WORKLOAD)
    warm = dict(W, nsites=WARMUP_NSITES)
    for _ in range(args.warmup):
        eng.sweep(**warm, fetch=False)
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
        res = eng.sweep(**W, fetch=True)
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
    if T["tridiag_launches"]:
        traffic = TRIDIAG_DRAM_BYTES_PER_ELEMENT * sum_n2(res) / T["tridiag_launches"]
    w_full = sum_n3(res)
    line = {
        "metric": "2ch NRG sweep s", "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "parallelism": f"replicas x{args.gpus}",
                   "l2": "working set (H_N blocks ~0.8 GB per iteration) larger than L2; no flush",
                   "warmup_step": f"first {WARMUP_NSITES} iterations of the same workload"},
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(T["h2d_bytes"]),
                "d2h_bytes_per_step": int(T["d2h_bytes"])},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "kernel": "tridiag (Householder, FP64)", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured by bench.py: DFMA register loop on all SMs (FP64 has no "
                                    "entry in MEASURED_PEAKS.json)",
                     "algorithmic": "4/3 sum_b n_b^3 flops per iteration"},
        "clocks": ck,
        "phases_ms": {k: T[k] for k in ("assemble_ms", "tridiag_ms", "tridiag_eig_ms", "vectors_ms",
                                          "backtransform_ms", "cut_ms", "update_ms")},
        "sum_n3": w_full,
    }
    # second half of the metric: batched independent solves per second
    bs, bsec = gpu_batch(args.batch_workers, local)
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
        dt, w_s, ref = cpu_sample(cores, want_result=True)
        line["cpu_baseline"] = {
            "value": dt * w_full / w_s, "unit": "s", "cores": cores, "kind": "port",
            "sample": (f"oracle port, same model/parameters with 600 kept and 8 iterations: {dt:.2f} s on "
                       f"{cores} threads, scaled by the sum n^3 ratio {w_full / w_s:.1f}")}
        # The GPU sweep against the FP64 oracle on that sample.
        C = CPU_SAMPLE
        gs = eng.sweep(C["model"], C["nsites"], C["ncutoff"], C["lam"], C["U"], C["ed"], C["gamma1"],
                      C["gamma2_or_B"])
        line["accuracy"] = {"sweep": dict(sweep_errors(gs, ref), sample=(
            "two-channel sweep, same model/parameters, 600 kept, 8 iterations, GPU against the FP64 oracle"))}
        cbs, cdt, cn = cpu_batch_sample(cores)
        line["batched"]["cpu_baseline"] = {
            "value": cbs, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"oracle port on the first {cn} instances, one per thread: {cdt:.2f} s"}
        # DM-NRG: GPU and the oracle port on the same reduced case (the port
        # evaluates every frequency with dense products, as DM_NRG does)
        from oracle import oracle as orc
        g = gpu_dm(eng, DM_SAMPLE, DM_SAMPLE_NOMEGA)
        t = time.perf_counter()
        o_dm = orc.dm_spectral(DM_SAMPLE["nsites"], DM_SAMPLE["ncutoff"], DM_SAMPLE["lam"], DM_SAMPLE["U"],
                               DM_SAMPLE["ed"], DM_SAMPLE["gamma"], DM_TEMP, DM_BROAD,
                               omegas=dm_omegas(DM_SAMPLE_NOMEGA))
        cdm = (time.perf_counter() - t) * 1e3
        import numpy as np
        A_gpu, A_ref = np.asarray(g[6]), np.asarray(o_dm[1])
        line.setdefault("accuracy", {})["dm_spectral"] = {
            "A_rel_max": float((np.abs(A_gpu - A_ref) / np.maximum(np.abs(A_ref), 1e-300)).max()),
            "A_abs_max_over_max_A": float(np.abs(A_gpu - A_ref).max() / np.abs(A_ref).max()),
            "sample": (f"one-channel DM-NRG, {DM_SAMPLE['nsites']} iterations, {DM_SAMPLE['ncutoff']} kept, "
                       f"{DM_SAMPLE_NOMEGA} frequencies, GPU against the FP64 oracle")}
        line["dm_spectral"]["cpu_baseline"] = {
            "value": cdm, "unit": "ms", "cores": 1, "kind": "port",
            "sample": (f"oracle port (single thread) on {DM_SAMPLE['nsites']} iterations, {DM_SAMPLE['ncutoff']} "
                       f"kept, {DM_SAMPLE_NOMEGA} frequencies, same T and b; GPU on that case: "
                       f"{g[0] + g[1] + g[2]:.1f} ms")}
    print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
