"""GB300-native engine for the TwoChNRG iterative-diagonalization hot path.

The compute path is the CUDA library ``_build/libtwochnrg_gb300.so`` (sm_103a),
driven through its C ABI (``include/twochnrg_gb300.h``).  This module is the
Python mirror of that ABI: it loads the library with ctypes and converts the
results to numpy arrays.  There is no CPU fallback: if the library or a usable
GB300 device is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

MODEL_1CH_QS, MODEL_1CH_QSZ, MODEL_2CH_QS = 0, 1, 2
MODELS = {"1chQS": MODEL_1CH_QS, "1chQSz": MODEL_1CH_QSZ, "2chQS": MODEL_2CH_QS}
PREC_FP64 = 0

STATUS = {0: "ok", 1: "bad argument", 2: "CUDA error", 3: "out of memory", 4: "not converged",
          5: "size limit exceeded", 6: "block structures out of sync", 7: "device wait timed out",
          8: "bad call order"}


class NRGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class SweepConfig(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("nsites", ctypes.c_int), ("ncutoff", ctypes.c_int),
                ("lambda_", ctypes.c_double), ("U", ctypes.c_double), ("ed", ctypes.c_double),
                ("gamma1", ctypes.c_double), ("gamma2_or_B", ctypes.c_double),
                ("degen_eps", ctypes.c_double), ("precision", ctypes.c_int)]


class _Iteration(ctypes.Structure):
    _fields_ = [("nblocks", ctypes.c_int), ("qnumbers", ctypes.POINTER(ctypes.c_double)),
                ("block_size", ctypes.POINTER(ctypes.c_int)), ("nstates", ctypes.c_int),
                ("en", ctypes.POINTER(ctypes.c_double)), ("emin", ctypes.c_double),
                ("ecut", ctypes.c_double), ("nkept", ctypes.c_int), ("nkept_blocks", ctypes.c_int),
                ("kept_block_size", ctypes.POINTER(ctypes.c_int)),
                ("thermo", ctypes.POINTER(ctypes.c_double)), ("nops", ctypes.c_int),
                ("opavg", ctypes.POINTER(ctypes.c_double)), ("params", ctypes.POINTER(ctypes.c_double))]


class Timing(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("assemble_ms", ctypes.c_double),
                ("tridiag_ms", ctypes.c_double), ("tridiag_eig_ms", ctypes.c_double),
                ("backtransform_ms", ctypes.c_double), ("cut_ms", ctypes.c_double),
                ("update_ms", ctypes.c_double), ("tridiag_flops", ctypes.c_double),
                ("update_flops", ctypes.c_double), ("backtransform_flops", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("tridiag_launches", ctypes.c_int64),
                ("device_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the engine library; raise if it is not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise NRGError(2, f"engine library not built: {LIB_PATH} (run __graft_entry__.build())")
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    L.nrg_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.nrg_destroy.argtypes = [ctypes.c_void_p]
    L.nrg_last_error.argtypes = [ctypes.c_void_p]
    L.nrg_last_error.restype = ctypes.c_char_p
    L.nrg_status_string.restype = ctypes.c_char_p
    L.nrg_kernel_count.argtypes = [ctypes.c_void_p]
    L.nrg_kernel_count.restype = ctypes.c_int64
    L.nrg_sweep_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig)]
    L.nrg_sweep_num_iterations.argtypes = [ctypes.c_void_p]
    L.nrg_sweep_iteration.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Iteration)]
    L.nrg_sweep_opavg_initial.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    L.nrg_sweep_timing.argtypes = [ctypes.c_void_p, ctypes.POINTER(Timing)]
    L.nrg_fp64_peak.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    _dp = ctypes.POINTER(ctypes.c_double)
    _ip = ctypes.POINTER(ctypes.c_int)
    L.nrg_diag_blocks.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp, _dp, _dp]
    L.nrg_sweep_batch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(SweepConfig), ctypes.c_int,
                                  ctypes.c_int, _dp, _dp, _ip, _dp]
    _lib = L
    return L


@dataclass
class Iteration:
    params: np.ndarray
    qn: np.ndarray
    bsize: np.ndarray
    en: np.ndarray
    emin: float
    ecut: float
    nkept: int
    thermo: np.ndarray
    opavg: np.ndarray
    kept_bsize: np.ndarray


@dataclass
class SweepResult:
    iters: list = field(default_factory=list)
    opavg_m1: np.ndarray | None = None
    timing: dict | None = None


def _arr(ptr, n, dtype):
    if n <= 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Engine:
    """One engine context (one CUDA stream on one device)."""

    def __init__(self, device: int = 0):
        self.L = load_library()
        h = ctypes.c_void_p()
        st = self.L.nrg_create(int(device), ctypes.byref(h))
        if st != 0:
            raise NRGError(st, "nrg_create failed (no usable sm_103 device?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.nrg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != 0:
            raise NRGError(st, self.L.nrg_last_error(self.h).decode())

    @property
    def kernel_count(self) -> int:
        return int(self.L.nrg_kernel_count(self.h))

    def diag_blocks(self, sizes, packed_upper):
        """DiagBlock for a batch of blocks in the reference's packed-upper
        storage.  Returns (eigenvalues per block, eigenvector matrices per
        block with row k = eigenvector k)."""
        sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        packed = np.ascontiguousarray(packed_upper, dtype=np.float64)
        need = int(sum(int(n) * (int(n) + 1) // 2 for n in sizes))
        if packed.size != need:
            raise ValueError(f"packed storage has {packed.size} elements, expected {need}")
        ev = np.empty(int(sizes.sum()), dtype=np.float64)
        vec = np.empty(int((sizes.astype(np.int64) ** 2).sum()), dtype=np.float64)
        P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
        self._check(self.L.nrg_diag_blocks(self.h, len(sizes), P(sizes, ctypes.c_int),
                                           P(packed, ctypes.c_double), P(ev, ctypes.c_double),
                                           P(vec, ctypes.c_double)))
        out_e, out_v, so, vo = [], [], 0, 0
        for n in sizes:
            n = int(n)
            out_e.append(ev[so:so + n]); out_v.append(vec[vo:vo + n * n].reshape(n, n))
            so += n; vo += n * n
        return out_e, out_v

    def fp64_peak(self) -> float:
        """Measured FP64 FMA throughput of the device, TFLOP/s."""
        v = ctypes.c_double()
        self._check(self.L.nrg_fp64_peak(self.h, ctypes.byref(v)))
        return v.value

    def sweep(self, model: str, nsites: int, ncutoff: int, lam: float, U: float, ed: float,
              gamma1: float, gamma2_or_B: float = 0.0, degen_eps: float = 0.0,
              precision: int = PREC_FP64, fetch: bool = True) -> SweepResult:
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, U, ed, gamma1, gamma2_or_B,
                          degen_eps, precision)
        self._check(self.L.nrg_sweep_run(self.h, ctypes.byref(cfg)))
        out = SweepResult()
        tm = Timing()
        self._check(self.L.nrg_sweep_timing(self.h, ctypes.byref(tm)))
        out.timing = tm.as_dict()
        if not fetch:
            return out
        nops = ctypes.c_int()
        vals = ctypes.POINTER(ctypes.c_double)()
        self._check(self.L.nrg_sweep_opavg_initial(self.h, ctypes.byref(nops), ctypes.byref(vals)))
        out.opavg_m1 = _arr(vals, nops.value, np.float64)
        for n in range(self.L.nrg_sweep_num_iterations(self.h)):
            it = _Iteration()
            self._check(self.L.nrg_sweep_iteration(self.h, n, ctypes.byref(it)))
            out.iters.append(Iteration(
                params=_arr(it.params, 4, np.float64),
                qn=_arr(it.qnumbers, 2 * it.nblocks, np.float64).reshape(it.nblocks, 2),
                bsize=_arr(it.block_size, it.nblocks, np.int64),
                en=_arr(it.en, it.nstates, np.float64),
                emin=it.emin, ecut=it.ecut, nkept=it.nkept,
                thermo=_arr(it.thermo, 16, np.float64).reshape(4, 4),
                opavg=_arr(it.opavg, it.nops, np.float64),
                kept_bsize=_arr(it.kept_block_size, it.nkept_blocks, np.int64)))
        return out


@dataclass
class BatchResult:
    thermo: np.ndarray   # (ninst, max_sites, 4, 4)
    opavg: np.ndarray    # (ninst, max_sites, 4)
    nkept: np.ndarray    # (ninst, max_sites)
    seconds: float


def sweep_batch(instances, nworkers: int = 16, device: int = 0, precision: int = PREC_FP64) -> BatchResult:
    """Run independent sweeps (dicts with the Engine.sweep keywords) on one
    GPU through nrg_sweep_batch."""
    L = load_library()
    n = len(instances)
    cfgs = (SweepConfig * max(n, 1))()
    max_sites = max([int(c["nsites"]) for c in instances] + [1])
    for i, c in enumerate(instances):
        cfgs[i] = SweepConfig(MODELS[c["model"]], int(c["nsites"]), int(c["ncutoff"]), float(c["lam"]),
                              float(c["U"]), float(c["ed"]), float(c["gamma1"]),
                              float(c.get("gamma2_or_B", 0.0)), float(c.get("degen_eps", 0.0)), precision)
    thermo = np.zeros((n, max_sites, 16))
    opavg = np.zeros((n, max_sites, 4))
    nkept = np.zeros((n, max_sites), dtype=np.int32)
    sec = ctypes.c_double()
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    st = L.nrg_sweep_batch(int(device), n, cfgs, int(nworkers), max_sites, P(thermo, ctypes.c_double),
                           P(opavg, ctypes.c_double), P(nkept, ctypes.c_int), ctypes.byref(sec))
    if st != 0:
        raise NRGError(st, "nrg_sweep_batch: " + L.nrg_last_error(None).decode())
    return BatchResult(thermo.reshape(n, max_sites, 4, 4), opavg, nkept, sec.value)


__all__ = ["Engine", "NRGError", "SweepResult", "Iteration", "BatchResult", "load_library", "sweep_batch",
           "MODELS"]
