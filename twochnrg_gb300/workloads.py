"""Synthetic workloads (seeded parameter draws) used by the tests and bench.

batched_qsz(): independent one-channel Anderson instances in the (Q,Sz)
basis: U ~ Uniform[0.1, 1], eps_d = -U/2 + Uniform[-0.1, 0.1],
Gamma log-uniform on [1e-3, 5e-2], B log-uniform on [1e-8, 1e-3], kept states
uniform on {200..1000}, Lambda = 2.5, 40 Wilson iterations.
"""
from __future__ import annotations

import numpy as np


def batched_qsz(n: int = 256, seed: int = 2024, nsites: int = 40, kmin: int = 200, kmax: int = 1000):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        U = rng.uniform(0.1, 1.0)
        ed = -U / 2 + rng.uniform(-0.1, 0.1)
        gamma = float(np.exp(rng.uniform(np.log(1e-3), np.log(5e-2))))
        B = float(np.exp(rng.uniform(np.log(1e-8), np.log(1e-3))))
        K = int(rng.integers(kmin, kmax + 1))
        out.append(dict(model="1chQSz", nsites=nsites, ncutoff=K, lam=2.5, U=float(U), ed=float(ed),
                        gamma1=gamma, gamma2_or_B=B))
    return out
