"""Batched independent sweeps (nrg_sweep_batch, one context per worker thread)
against the oracle, instance by instance: kept counts exact, thermodynamics
and <n_d>, <S_z> within 1e-8 relative.  <S_z> at fields of 1e-8 is itself
~1e-7, a cancellation between O(1) Boltzmann terms, so averages also get an
absolute floor of 1e-12 (the round-off of the O(1) sums)."""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc
from twochnrg_gb300.workloads import batched_qsz

pytestmark = pytest.mark.gpu


def test_batch_matches_oracle():
    inst = batched_qsz(n=6, seed=11, nsites=10, kmin=60, kmax=160)
    res = tg.sweep_batch(inst, nworkers=3)
    assert res.seconds > 0
    for i, c in enumerate(inst):
        o = orc.run(c["model"], c["nsites"], c["ncutoff"], c["lam"], c["U"], c["ed"], c["gamma1"],
                    c["gamma2_or_B"], nthreads=min(4, os.cpu_count() or 1))
        for n, it in enumerate(o.iters):
            assert res.nkept[i, n] == it.nkept, f"instance {i} N={n}"
            np.testing.assert_allclose(res.thermo[i, n], it.thermo, rtol=1e-8, atol=1e-14)
            np.testing.assert_allclose(res.opavg[i, n, :len(it.opavg)], it.opavg, rtol=1e-8, atol=1e-12)


def test_batch_of_mixed_models():
    inst = [dict(model="1chQS", nsites=6, ncutoff=80, lam=2.5, U=0.5, ed=-0.25, gamma1=0.02, gamma2_or_B=0.0),
            dict(model="2chQS", nsites=4, ncutoff=40, lam=2.5, U=0.3, ed=-0.15, gamma1=0.01, gamma2_or_B=0.01)]
    res = tg.sweep_batch(inst, nworkers=2)
    for i, c in enumerate(inst):
        o = orc.run(c["model"], c["nsites"], c["ncutoff"], c["lam"], c["U"], c["ed"], c["gamma1"],
                    c["gamma2_or_B"])
        for n, it in enumerate(o.iters):
            assert res.nkept[i, n] == it.nkept
            np.testing.assert_allclose(res.thermo[i, n], it.thermo, rtol=1e-8, atol=1e-14)


def test_batch_full_size_instances():
    """Four instances of the batched workload itself (seed 2024: 40 iterations,
    kept counts drawn from 200..1000), including its largest kept count, against
    the oracle on host threads: kept counts exact; <n_d>, <S_z> and T chi (with
    the CalcSuscep quirk of the reference, <S_z^2> without <S_z>^2) 1e-8."""
    from concurrent.futures import ThreadPoolExecutor
    allinst = batched_qsz(256, seed=2024)
    pick = sorted(range(256), key=lambda i: allinst[i]["ncutoff"])
    idx = [pick[0], pick[85], pick[170], pick[255]]
    inst = [allinst[i] for i in idx]
    res = tg.sweep_batch(inst, nworkers=4)

    def oracle(c):
        return orc.run(c["model"], c["nsites"], c["ncutoff"], c["lam"], c["U"], c["ed"], c["gamma1"],
                       c["gamma2_or_B"], nthreads=2)

    with ThreadPoolExecutor(max_workers=4) as ex:
        refs = list(ex.map(oracle, inst))
    for i, o in enumerate(refs):
        assert len(o.iters) == 40
        for n, it in enumerate(o.iters):
            assert res.nkept[i, n] == it.nkept, f"instance {idx[i]} N={n}"
            np.testing.assert_allclose(res.thermo[i, n], it.thermo, rtol=1e-8, atol=1e-14)
            np.testing.assert_allclose(res.opavg[i, n, :len(it.opavg)], it.opavg, rtol=1e-8, atol=1e-12)
