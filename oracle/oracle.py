"""ctypes wrapper of the C++ oracle restatement (oracle/nrg_oracle.cpp).

Test infrastructure only.  ``build()`` compiles the oracle in-tree with g++;
``run()`` executes one NRG sweep and returns per-iteration numpy arrays.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "libnrg_oracle.so")

MODEL_1CHQS, MODEL_1CHQSZ, MODEL_2CHQS, MODEL_1CHQ, MODEL_1CHS, MODEL_1CHSZ = 0, 1, 2, 3, 4, 5
MODELS = {"1chQS": MODEL_1CHQS, "1chQSz": MODEL_1CHQSZ, "2chQS": MODEL_2CHQS, "1chQ": MODEL_1CHQ,
          "1chS": MODEL_1CHS, "1chSz": MODEL_1CHSZ}


class _Cfg(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("nsites", ctypes.c_int), ("ncutoff", ctypes.c_int),
                ("lambda_", ctypes.c_double), ("U", ctypes.c_double), ("ed", ctypes.c_double),
                ("gamma1", ctypes.c_double), ("gamma2_or_B", ctypes.c_double),
                ("degen_eps", ctypes.c_double), ("nthreads", ctypes.c_int),
                ("capture_iter", ctypes.c_int), ("dm", ctypes.c_int), ("chain", ctypes.c_int),
                ("delta_sc", ctypes.c_double), ("chain_chi", ctypes.POINTER(ctypes.c_double)),
                ("chain_en", ctypes.POINTER(ctypes.c_double)), ("chain_len", ctypes.c_int),
                ("chain_alambda", ctypes.c_int)]


class _DmParams(ctypes.Structure):
    _fields_ = [("temp", ctypes.c_double), ("betabar", ctypes.c_double), ("bbroad", ctypes.c_double),
                ("twindow", ctypes.c_double), ("broadtemp", ctypes.c_double), ("site_dim", ctypes.c_double),
                ("nw", ctypes.c_int), ("mtemp", ctypes.c_int)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "nrg_oracle.cpp")
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", SO,
                               "-ldl", "-lpthread"])
    return SO


def openblas_path() -> str:
    """OpenBLAS bundled with scipy (LP64, symbols prefixed ``scipy_``)."""
    import scipy
    root = os.path.dirname(os.path.dirname(scipy.__file__))
    libs = sorted(glob.glob(os.path.join(root, "scipy.libs", "libscipy_openblas*.so")))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS not found")
    return libs[0]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(SO)
        L.oracle_run.restype = ctypes.c_void_p
        L.oracle_run.argtypes = [ctypes.POINTER(_Cfg)]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_cgordan.restype = ctypes.c_double
        L.oracle_cgordan.argtypes = [ctypes.c_double] * 6
        L.oracle_seconds.restype = ctypes.c_double
        L.oracle_op_name.restype = ctypes.c_char_p
        for name in ("oracle_iter_emin", "oracle_iter_ecut", "oracle_iter_seconds"):
            getattr(L, name).restype = ctypes.c_double
        for name in ("oracle_iter_qn", "oracle_iter_en", "oracle_iter_thermo", "oracle_iter_opavg",
                     "oracle_iter_params", "oracle_iter_H", "oracle_iter_basis_en", "oracle_opavg_m1"):
            getattr(L, name).restype = ctypes.POINTER(ctypes.c_double)
        for name in ("oracle_iter_bsize", "oracle_iter_kept_bsize", "oracle_iter_basis_itype",
                     "oracle_iter_basis_stcf"):
            getattr(L, name).restype = ctypes.POINTER(ctypes.c_int)
        L.oracle_cap_d.restype = ctypes.POINTER(ctypes.c_double)
        L.oracle_cap_i.restype = ctypes.POINTER(ctypes.c_int)
        for name in ("oracle_cap_d", "oracle_cap_i"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p,
                                         ctypes.POINTER(ctypes.c_int)]
        L.oracle_dm_spectral.argtypes = [ctypes.c_void_p, ctypes.POINTER(_DmParams),
                                          ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.oracle_dm_d.restype = ctypes.POINTER(ctypes.c_double)
        L.oracle_dm_i.restype = ctypes.POINTER(ctypes.c_int)
        for name in ("oracle_dm_d", "oracle_dm_i"):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p,
                                         ctypes.POINTER(ctypes.c_int)]
        L.oracle_diag_block.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        rc = L.oracle_load_lapack(openblas_path().encode())
        if rc != 0:
            raise RuntimeError("oracle: " + L.oracle_last_error().decode())
        _lib = L
    return _lib


@dataclass
class Iteration:
    params: np.ndarray
    qn: np.ndarray          # (nblocks, 2)
    bsize: np.ndarray       # (nblocks,)
    en: np.ndarray          # (nstates,)
    emin: float
    ecut: float
    nkept: int
    thermo: np.ndarray      # (4, 4): beta, T, suscep, entropy
    opavg: np.ndarray
    kept_bsize: np.ndarray
    H: np.ndarray | None = None
    basis_itype: np.ndarray | None = None
    basis_stcf: np.ndarray | None = None
    basis_en: np.ndarray | None = None
    seconds: float = 0.0    # wall time of the iteration
    # capture iteration only: every input/output of DiagHN, SetKept, CutStates
    # and UpdateMatrices by name (old_*, basis_*, eig_*, kept*, cut_*, new_*;
    # per-operator arrays end in .<operator index>)
    cap: dict | None = None


@dataclass
class Sweep:
    iters: list = field(default_factory=list)
    opnames: list = field(default_factory=list)
    opavg_m1: np.ndarray | None = None
    seconds: float = 0.0


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def run(model: str, nsites: int, ncutoff: int, lam: float, U: float, ed: float, gamma1: float,
        gamma2_or_B: float = 0.0, nthreads: int = 1, capture_iter: int = -1,
        degen_eps: float = 0.0, blas_threads: int = 1, chain: bool = False, delta_sc: float = 0.0,
        wilson=None, alambda: bool = True) -> Sweep:
    """One sweep.  chain=True: the free Wilson chain of calcdens = 3 (U, ed and
    the couplings are ignored; iteration 0 is the first site alone).  delta_sc:
    the leads' gap of the superconducting-lead models.  wilson: a chain (chi, en)
    other than the flat band's."""
    L = lib()
    L.oracle_blas_threads(int(blas_threads))
    cfg = _Cfg(MODELS[model], nsites, ncutoff, lam, U, ed, gamma1, gamma2_or_B, degen_eps,
               nthreads, capture_iter, 0, 1 if chain else 0, delta_sc)
    if wilson is not None:
        wc = np.ascontiguousarray(wilson[0], dtype=np.float64)
        we = np.ascontiguousarray(wilson[1], dtype=np.float64)
        cfg.chain_chi = wc.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        cfg.chain_en = we.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        cfg.chain_len = len(wc)
        cfg.chain_alambda = 1 if alambda else 0
    h = L.oracle_run(ctypes.byref(cfg))
    if not h:
        raise RuntimeError("oracle: " + L.oracle_last_error().decode())
    h = ctypes.c_void_p(h)
    try:
        out = Sweep()
        nops = L.oracle_num_ops(h)
        out.opnames = [L.oracle_op_name(h, k).decode() for k in range(nops)]
        out.opavg_m1 = _arr(L.oracle_opavg_m1(h), nops, np.float64)
        out.seconds = L.oracle_seconds(h)
        nq = L.oracle_nqn(h)
        for n in range(L.oracle_num_iters(h)):
            nb = L.oracle_iter_nblocks(h, n)
            ns = L.oracle_iter_nstates(h, n)
            it = Iteration(
                params=_arr(L.oracle_iter_params(h, n), L.oracle_iter_nparams(h, n), np.float64),
                qn=_arr(L.oracle_iter_qn(h, n), nq * nb, np.float64).reshape(nb, nq),
                bsize=_arr(L.oracle_iter_bsize(h, n), nb, np.int64),
                en=_arr(L.oracle_iter_en(h, n), ns, np.float64),
                emin=L.oracle_iter_emin(h, n), ecut=L.oracle_iter_ecut(h, n),
                nkept=L.oracle_iter_nkept(h, n),
                thermo=_arr(L.oracle_iter_thermo(h, n), 16, np.float64).reshape(4, 4),
                opavg=_arr(L.oracle_iter_opavg(h, n), nops, np.float64),
                kept_bsize=_arr(L.oracle_iter_kept_bsize(h, n), L.oracle_iter_nkeptblocks(h, n), np.int64),
                seconds=L.oracle_iter_seconds(h, n))
            if n == capture_iter:
                it.H = _arr(L.oracle_iter_H(h, n), L.oracle_iter_H_size(h, n), np.float64)
                it.basis_itype = _arr(L.oracle_iter_basis_itype(h, n), ns, np.int64)
                it.basis_stcf = _arr(L.oracle_iter_basis_stcf(h, n), ns, np.int64)
                it.basis_en = _arr(L.oracle_iter_basis_en(h, n), ns, np.float64)
                it.cap = _captures(L, h, n)
            out.iters.append(it)
        return out
    finally:
        L.oracle_free(h)


_CAP_D = ("old_qn", "basis_qn", "basis_en", "eig_en", "eig_evec", "params", "kept_en", "cut_qn",
          "cut_en", "cut_evec")
_CAP_I = ("old_bbe", "basis_bbe", "basis_itype", "basis_stcf", "kept", "cut_bbe", "cut_bbe_bc",
          "cut_bbe_eig", "cut_stcf", "cut_kept")


def _captures(L, h, n) -> dict:
    out = {}
    ln = ctypes.c_int(0)

    def get(fn, name, dtype):
        p = fn(h, n, name.encode(), ctypes.byref(ln))
        if ln.value < 0:
            return None
        return _arr(p, ln.value, dtype)

    for name in _CAP_D:
        out[name] = get(L.oracle_cap_d, name, np.float64)
    for name in _CAP_I:
        out[name] = get(L.oracle_cap_i, name, np.int64)
    o = 0
    while True:
        el = get(L.oracle_cap_d, f"old_el.{o}", np.float64)
        if el is None:
            break
        out[f"old_el.{o}"] = el
        for pre in ("old", "new"):
            out[f"{pre}_map.{o}"] = get(L.oracle_cap_i, f"{pre}_map.{o}", np.int64)
            out[f"{pre}_mbe.{o}"] = get(L.oracle_cap_i, f"{pre}_mbe.{o}", np.int64)
        out[f"new_el.{o}"] = get(L.oracle_cap_d, f"new_el.{o}", np.float64)
        o += 1
    out["nmats"] = o
    return out


def dm_temp_default(lam: float, nsites: int, betabar: float = 0.727) -> float:
    """DM_NRG's temperature when Mtemp >= Nsitesmax-1 (DM_NRG.cpp:112-121):
    D_{Nsitesmax+199} / betabar."""
    hlf = 0.5 * (1.0 + 1.0 / lam)
    return hlf * lam ** ((-(nsites + 199 - 1) / 2.0) - 1.0 + 1.0) / betabar


def dm_spectral(nsites: int, ncutoff: int, lam: float, U: float, ed: float, gamma: float, temp: float,
                bbroad: float, nw: int = 4, omegas=None, betabar: float = 0.727, twindow: float = 2.0,
                broadtemp: float = 0.8, site_dim: float | None = None, nthreads: int = 1, mtemp: int = -1,
                model: str = "1chQS", gamma2: float = 0.0):
    """|Q S> Anderson model (one channel, or "2chQS" with Gamma1 = gamma and
    Gamma2 = gamma2): forward sweep saving the DM-NRG shells (UpdateBefCut =
    1, c_d), then the FDM density-matrix backward sweep and the c_d spectral
    function.  site_dim defaults to 4 (16 for two channels).  Returns
    (omega, A, rho_trace per shell)."""
    L = lib()
    if model not in ("1chQS", "2chQS"):
        raise ValueError(f"DM-NRG is restated for 1chQS and 2chQS, not {model!r}")
    two = model == "2chQS"
    if site_dim is None:
        site_dim = 16.0 if two else 4.0
    cfg = _Cfg(MODEL_2CHQS if two else MODEL_1CHQS, nsites, ncutoff, lam, U, ed, gamma, gamma2 if two else 0.0,
               0.0, nthreads, -1, 1)
    h = L.oracle_run(ctypes.byref(cfg))
    if not h:
        raise RuntimeError("oracle: " + L.oracle_last_error().decode())
    h = ctypes.c_void_p(h)
    try:
        prm = _DmParams(temp, betabar, bbroad, twindow, broadtemp, site_dim, nw, mtemp)
        P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        if omegas is None:
            cap = 2 * nw * nsites + 8
            om_in, n_in = None, 0
        else:
            om_arr = np.ascontiguousarray(omegas, dtype=np.float64)
            cap, om_in, n_in = len(om_arr), P(om_arr), len(om_arr)
        om = np.zeros(cap)
        A = np.zeros(cap)
        tr = np.zeros(nsites)
        n = L.oracle_dm_spectral(h, ctypes.byref(prm), om_in, n_in, P(om), P(A), cap, P(tr))
        if n < 0:
            raise RuntimeError("oracle: " + L.oracle_last_error().decode())
        return om[:n], A[:n], tr
    finally:
        L.oracle_free(h)


_DM_D = ("basis_qn", "basis_en", "qn", "en", "evec", "cd_el")
_DM_I = ("basis_bbe", "basis_itype", "basis_stcf", "bbe", "kept", "cd_map", "cd_mbe")


def dm_shells(nsites: int, ncutoff: int, lam: float, U: float, ed: float, gamma: float, nthreads: int = 1,
              model: str = "1chQS", gamma2: float = 0.0):
    """The DM-NRG shells of the |Q S> Anderson sweep (one channel, or "2chQS"
    with Gamma2 = gamma2; UpdateBefCut = 1, c_d), one dict of arrays per shell
    (Abasis_N: basis_*; Acut_N: qn, bbe, en, kept, evec; c_d: cd_*)."""
    L = lib()
    two = model == "2chQS"
    cfg = _Cfg(MODEL_2CHQS if two else MODEL_1CHQS, nsites, ncutoff, lam, U, ed, gamma, gamma2 if two else 0.0,
               0.0, nthreads, -1, 1)
    h = L.oracle_run(ctypes.byref(cfg))
    if not h:
        raise RuntimeError("oracle: " + L.oracle_last_error().decode())
    h = ctypes.c_void_p(h)
    try:
        out = []
        ln = ctypes.c_int(0)
        for N in range(nsites):
            d = {}
            for k in _DM_D:
                p = L.oracle_dm_d(h, N, k.encode(), ctypes.byref(ln))
                d[k] = _arr(p, ln.value, np.float64)
            for k in _DM_I:
                p = L.oracle_dm_i(h, N, k.encode(), ctypes.byref(ln))
                d[k] = _arr(p, ln.value, np.int64)
            out.append(d)
        return out
    finally:
        L.oracle_free(h)


def diag_block(packed: np.ndarray, n: int):
    """The reference's DiagBlock: LAPACK dspev on the packed upper triangle."""
    L = lib()
    packed = np.ascontiguousarray(packed, dtype=np.float64)
    w = np.empty(n, dtype=np.float64)
    Z = np.empty(n * n, dtype=np.float64)
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    info = L.oracle_diag_block(n, P(packed), P(w), P(Z))
    if info != 0:
        raise RuntimeError(f"dspev info={info}")
    return w, Z.reshape(n, n)


def pack_upper(A: np.ndarray) -> np.ndarray:
    """Row-major packed upper triangle (ij2rUpTr order)."""
    n = A.shape[0]
    return np.concatenate([A[i, i:] for i in range(n)]) if n else np.zeros(0)
