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

MODEL_1CH_QS, MODEL_1CH_QSZ, MODEL_2CH_QS, MODEL_1CH_Q, MODEL_1CH_S, MODEL_1CH_SZ = 0, 1, 2, 3, 4, 5
MODELS = {"1chQS": MODEL_1CH_QS, "1chQSz": MODEL_1CH_QSZ, "2chQS": MODEL_2CH_QS, "1chQ": MODEL_1CH_Q,
          "1chS": MODEL_1CH_S, "1chSz": MODEL_1CH_SZ}
PREC_FP64 = 0
PREC_MIXED = 1  # blocked reduction of the large blocks with tensor-core trailing products

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
                ("degen_eps", ctypes.c_double), ("precision", ctypes.c_int), ("delta_sc", ctypes.c_double)]


class _Iteration(ctypes.Structure):
    _fields_ = [("nblocks", ctypes.c_int), ("qnumbers", ctypes.POINTER(ctypes.c_double)),
                ("block_size", ctypes.POINTER(ctypes.c_int)), ("nstates", ctypes.c_int),
                ("en", ctypes.POINTER(ctypes.c_double)), ("emin", ctypes.c_double),
                ("ecut", ctypes.c_double), ("nkept", ctypes.c_int), ("nkept_blocks", ctypes.c_int),
                ("kept_block_size", ctypes.POINTER(ctypes.c_int)),
                ("thermo", ctypes.POINTER(ctypes.c_double)), ("nops", ctypes.c_int),
                ("opavg", ctypes.POINTER(ctypes.c_double)), ("params", ctypes.POINTER(ctypes.c_double)),
                ("wall_ms", ctypes.c_double), ("device_ms", ctypes.c_double)]


class _Grad(ctypes.Structure):
    _fields_ = [("nsites", ctypes.c_int), ("nparams", ctypes.c_int), ("nops", ctypes.c_int),
                ("d_thermo", ctypes.POINTER(ctypes.c_double)), ("d_opavg", ctypes.POINTER(ctypes.c_double)),
                ("d_emin", ctypes.POINTER(ctypes.c_double)), ("egs", ctypes.POINTER(ctypes.c_double)),
                ("d_egs", ctypes.POINTER(ctypes.c_double))]


@dataclass
class GradResult:
    """nrg_grad_forward: the sweep and the derivatives of its reported values
    with respect to (eps_d, U, Gamma1, B), parameter on the second axis."""
    sweep: "SweepResult"
    d_thermo: np.ndarray   # (nsites, 4, 4, 4): d thermo (beta, T, T chi, S at 4 temperatures)
    d_opavg: np.ndarray    # (nsites, 4, nops)
    d_emin: np.ndarray     # (nsites, 4)
    egs: np.ndarray        # (nsites,) absolute ground-state energy
    d_egs: np.ndarray      # (nsites, 4)

    def tchi_on(self, temps):
        """T chi and d T chi / d p at the temperatures `temps`, linear in ln T
        between the sweep's own temperatures (four per iteration, strictly
        decreasing along the sweep); the derivatives are interpolated alike,
        the interpolation being linear in the values.  The free chain's part
        of T chi does not depend on the parameters, so d T chi is also the
        derivative of the impurity's T chi.  Temperatures outside the sweep's
        range get NaN.  Returns (tchi (m,), d_tchi (4, m))."""
        T = np.array([it.thermo[:, 1] for it in self.sweep.iters]).ravel()
        v = np.array([it.thermo[:, 2] for it in self.sweep.iters]).ravel()
        d = self.d_thermo[:, :, :, 2].transpose(1, 0, 2).reshape(self.d_thermo.shape[1], -1)
        o = np.argsort(T)
        lt = np.log(T[o])
        x = np.log(np.asarray(temps, dtype=np.float64))
        out = (x < lt[0]) | (x > lt[-1])
        tchi = np.interp(x, lt, v[o])
        dt = np.array([np.interp(x, lt, dk[o]) for dk in d])
        tchi[out] = np.nan
        dt[:, out] = np.nan
        return tchi, dt


class Timing(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("assemble_ms", ctypes.c_double),
                ("tridiag_ms", ctypes.c_double), ("tridiag_eig_ms", ctypes.c_double),
                ("backtransform_ms", ctypes.c_double), ("cut_ms", ctypes.c_double),
                ("update_ms", ctypes.c_double), ("tridiag_flops", ctypes.c_double),
                ("update_flops", ctypes.c_double), ("backtransform_flops", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("tridiag_launches", ctypes.c_int64),
                ("device_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("dm_backprop_ms", ctypes.c_double), ("dm_spectral_ms", ctypes.c_double),
                ("lehmann_ms", ctypes.c_double), ("lehmann_pairs", ctypes.c_int64),
                ("lehmann_evals", ctypes.c_int64), ("vectors_ms", ctypes.c_double)]


    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class DmParams(ctypes.Structure):
    """DM_NRG's command-line parameters (nrg_dm_params)."""
    _fields_ = [("temp", ctypes.c_double), ("mtemp", ctypes.c_int), ("betabar", ctypes.c_double),
                ("bbroad", ctypes.c_double), ("twindow", ctypes.c_double), ("broadtemp", ctypes.c_double),
                ("site_dim", ctypes.c_double), ("nw", ctypes.c_int)]


_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_ubyte)


class _Blocks(ctypes.Structure):
    _fields_ = [("nblocks", ctypes.c_int), ("nqn", ctypes.c_int), ("qnumbers", _DP), ("block_beg_end", _IP)]


class _Basis(ctypes.Structure):
    _fields_ = [("blocks", _Blocks), ("itype", _IP), ("st_came_from", _IP), ("en", _DP)]


class _Matrix(ctypes.Structure):
    _fields_ = [("nmatblocks", ctypes.c_int), ("mat_block_map", _IP), ("mat_block_beg_end", _IP),
                ("mat_el", _DP)]


class _EigCut(ctypes.Structure):
    _fields_ = [("blocks", _Blocks), ("block_beg_end_bc", _IP), ("block_beg_end_eigvec", _IP),
                ("st_came_from", _IP), ("en", _DP), ("kept", _UP), ("eigvec", _DP)]


class _CutResult(ctypes.Structure):
    _fields_ = [("en", _DP), ("kept", _UP), ("nkept", ctypes.c_int), ("ecut", ctypes.c_double),
                ("cut", _EigCut)]


class DmShell(ctypes.Structure):
    _fields_ = [("nshell", ctypes.c_int), ("basis", _Basis), ("blocks", _Blocks), ("en", _DP), ("kept", _UP),
                ("eigvec", _DP), ("cd", _Matrix)]


class _Keep:
    """Holds the numpy arrays a ctypes structure points into."""

    def __init__(self):
        self.refs = []

    def d(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.refs.append(a)
        return a.ctypes.data_as(_DP)

    def i(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.refs.append(a)
        return a.ctypes.data_as(_IP)

    def blocks(self, qn, bbe):
        qn = np.asarray(qn, dtype=np.float64).reshape(-1)
        return _Blocks(len(qn) // 2, 2, self.d(qn), self.i(bbe))

    def matrix(self, m):
        mp, mbe, el = m
        return _Matrix(len(mp) // 2, self.i(mp), self.i(mbe), self.d(el))


_lib = None


def write_dm_shell(directory: str, name: str, nshell: int, shell: dict) -> None:
    """Write one DM-NRG shell (dict with basis_qn/bbe/itype/stcf/en, qn, bbe, en,
    kept, evec, cd_map/cd_mbe/cd_el) as the reference's Abasis/Acut/Mat0 .bin
    files.  Needs no device."""
    L = load_library()
    k = _Keep()
    kept = np.ascontiguousarray(shell["kept"], dtype=np.uint8)
    k.refs.append(kept)
    s = DmShell(nshell,
                _Basis(k.blocks(shell["basis_qn"], shell["basis_bbe"]), k.i(shell["basis_itype"]),
                       k.i(shell["basis_stcf"]), k.d(shell["basis_en"])),
                k.blocks(shell["qn"], shell["bbe"]), k.d(shell["en"]), kept.ctypes.data_as(_UP),
                k.d(shell["evec"]), k.matrix((shell["cd_map"], shell["cd_mbe"], shell["cd_el"])))
    st = L.nrg_write_dm_shell(directory.encode(), name.encode(), ctypes.byref(s))
    if st != 0:
        raise NRGError(st, f"cannot write shell {nshell} into {directory}")


def write_code_pars(directory: str, lam: float, nsites: int, name: str) -> None:
    st = load_library().nrg_write_code_pars(directory.encode(), float(lam), int(nsites), name.encode())
    if st != 0:
        raise NRGError(st, f"cannot write ThisCodePars.dat into {directory}")


BAND_CONST, BAND_LORENTZIAN, BAND_TABLE = 0, 1, 2
BANDS = {"const": BAND_CONST, "lorentzian": BAND_LORENTZIAN, "table": BAND_TABLE}


class _Band(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("nparams", ctypes.c_int), ("params", _DP), ("lambda_", ctypes.c_double),
                ("z", ctypes.c_double), ("disc_scheme", ctypes.c_int), ("band_offset", ctypes.c_double)]


def chain_lanczos(kind: str, nsites: int, lam: float, params=(), z: float = 1.0, disc_scheme: int = 0,
                  band_offset: float = 0.0):
    """Wilson chain of a band by the reference's Lanczos procedure
    (nrg_chain_lanczos): returns (chi, en, Fsq).  Needs no device."""
    L = load_library()
    p = np.ascontiguousarray(params, dtype=np.float64)
    chi = np.zeros(int(nsites)); en = np.zeros(int(nsites)); fsq = ctypes.c_double()
    b = _Band(BANDS[kind], len(p), p.ctypes.data_as(_DP) if len(p) else None, float(lam), float(z),
              int(disc_scheme), float(band_offset))
    st = L.nrg_chain_lanczos(ctypes.byref(b), int(nsites), chi.ctypes.data_as(_DP), en.ctypes.data_as(_DP),
                             ctypes.byref(fsq))
    if st != 0:
        raise NRGError(st, "nrg_chain_lanczos failed")
    return chi, en, fsq.value


class _Thermo(ctypes.Structure):
    _fields_ = [("nvalues", ctypes.c_int), ("temp", _DP), ("suscep", _DP), ("suscep_chain", _DP),
                ("suscep_imp", _DP), ("entropy", _DP), ("entropy_chain", _DP), ("entropy_imp", _DP),
                ("chain_reused", ctypes.c_int), ("chain_ms", ctypes.c_double), ("imp_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double)]


# Thermodynamics files of CNRGCodeHandler::ModelSwitch
# (CodeHandler_ModelSwitch.cpp:202-216, 810-822, 585-593, 1187-1188), as
# {quantity: (impurity file, chain file)}; "{z}" becomes the z-string ("_zEQ1"
# for z = 1).  NRG_main has no two-channel Anderson model; its impurity file
# follows the one-channel Anderson pattern.  The |Q> symmetry has the entropy
# only, without a z-string.
THERMO_FILES = {
    "1chQS": {"Suscep": ("SuscepImp1ChQS_Anderson{z}.dat", "SuscepChain1Ch_QS{z}.dat"),
              "Entropy": ("EntropyImp1ChQS_Anderson{z}.dat", "EntropyChain1Ch_QS{z}.dat")},
    "1chQSz": {"Suscep": ("SuscepImp1ChQSz{z}.dat", "SuscepChain1Ch_QSz{z}.dat"),
               "Entropy": ("EntropyImp1ChQSz{z}.dat", "EntropyChain1Ch_QSz{z}.dat")},
    "2chQS": {"Suscep": ("SuscepImp2ChQS_Anderson{z}.dat", "SuscepChain2Ch_QS{z}.dat"),
              "Entropy": ("EntropyImp2ChQS_Anderson{z}.dat", "EntropyChain2Ch_QS{z}.dat")},
    "1chQ": {"Entropy": ("EntropyImp1Ch_Anderson_Q.dat", "EntropyChain1Ch_Q.dat")},
}


def write_thermo(path: str, temp, value, chain=None) -> None:
    """One file in the layout of CNRGthermo::SaveNValue: T value chain value-chain
    per line (chain=None: a chain file, third column 0).  Needs no device."""
    L = load_library()
    t = np.ascontiguousarray(temp, dtype=np.float64)
    v = np.ascontiguousarray(value, dtype=np.float64)
    c = None if chain is None else np.ascontiguousarray(chain, dtype=np.float64)
    if len(v) != len(t) or (c is not None and len(c) != len(t)):
        raise NRGError(1, "temp, value and chain must have the same length")
    st = L.nrg_write_thermo(path.encode(), len(t), t.ctypes.data_as(_DP), v.ctypes.data_as(_DP),
                            None if c is None else c.ctypes.data_as(_DP))
    if st != 0:
        raise NRGError(st, f"cannot write {path}")


@dataclass
class ThermoResult:
    """T chi and S of the impurity sweep, of the free chain, and their
    difference, at T_M = D_N / betabar_nc (value k = 4 N + nc - 1)."""
    temp: np.ndarray
    suscep: np.ndarray
    suscep_chain: np.ndarray
    suscep_imp: np.ndarray
    entropy: np.ndarray
    entropy_chain: np.ndarray
    entropy_imp: np.ndarray
    chain_reused: bool
    chain_ms: float
    imp_ms: float
    total_ms: float
    model: str = "1chQS"

    def save(self, directory: str, z: str = "1") -> list:
        """The reference's files (SuscepImp*, EntropyImp*, SuscepChain*,
        EntropyChain*) in `directory`; returns their paths."""
        out = []
        for kind, val, ch in (("Suscep", self.suscep, self.suscep_chain),
                              ("Entropy", self.entropy, self.entropy_chain)):
            names = THERMO_FILES[self.model].get(kind)
            if names is None:
                continue
            p_imp, p_ch = (os.path.join(directory, n.format(z="_zEQ" + z)) for n in names)
            write_thermo(p_imp, self.temp, val, ch)
            write_thermo(p_ch, self.temp, ch, None)
            out += [p_imp, p_ch]
        return out


# ---- model plug-in (nrg_model_desc) -----------------------------------------
HN_ONE_OP, HN_SPIN_SUM, HN_CHANNEL_SUM = 0, 1, 2
OP_SITE, OP_IMPURITY, OP_IMPURITY_DIAG = 0, 1, 2
_HN_COEF_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int, ctypes.c_int)
_OP_FACTOR_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_int, ctypes.c_int)
_OP_CHECK_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double))


class _ModelDesc(ctypes.Structure):
    _fields_ = [("total_spin", ctypes.c_int), ("site_nqn", ctypes.c_int), ("site_nblocks", ctypes.c_int),
                ("site_qn", ctypes.POINTER(ctypes.c_double)), ("site_bsize", ctypes.POINTER(ctypes.c_int)),
                ("hn_form", ctypes.c_int), ("onsite", ctypes.c_int), ("hn_coef", _HN_COEF_FN),
                ("nops", ctypes.c_int), ("op_class", ctypes.POINTER(ctypes.c_int)),
                ("op_avg", ctypes.POINTER(ctypes.c_int)), ("op_factor", _OP_FACTOR_FN),
                ("op_check", _OP_CHECK_FN), ("start_nblocks", ctypes.c_int),
                ("start_qn", ctypes.POINTER(ctypes.c_double)), ("start_bsize", ctypes.POINTER(ctypes.c_int)),
                ("start_en", ctypes.POINTER(ctypes.c_double)), ("start_npairs", ctypes.POINTER(ctypes.c_int)),
                ("start_pairs", ctypes.POINTER(ctypes.c_int)), ("start_el", ctypes.POINTER(ctypes.c_double)),
                ("user", ctypes.c_void_p)]


@dataclass
class ModelPlugin:
    """A model supplied from Python through nrg_sweep_run_model: the
    reference's CalcHNMatEl / CalcMatEl / CheckForMatEl rules
    (include/NRGclasses.hpp:612-634) as callables, its single-site basis and
    its H_{-1} set-up.

    hn_coef(S, ti, tj, channel, sigma, dir) -> float
    op_factor(op, S_i, S_j, ti, tj) -> float          (NRG_OP_SITE / NRG_OP_IMPURITY)
    op_check(op, qn_i, qn_j) -> bool                   (qn: (Q, S or S_z) of a kept block)
    start_ops[o]: list of (bi, bj, dense block) of operator o at H_{-1}."""
    total_spin: bool
    site_qn: list
    site_bsize: list
    hn_form: int
    onsite: bool
    hn_coef: object
    op_class: list
    op_avg: list
    op_factor: object
    op_check: object
    start_qn: list
    start_bsize: list
    start_en: list
    start_ops: list

    def _desc(self, keep: list, errors: list) -> "_ModelDesc":
        def guard(fn, bad):
            def call(*a):
                try:
                    return fn(*a)
                except BaseException as e:  # surfaced after the sweep returns
                    errors.append(e)
                    return bad
            return call

        def dbl(v):
            a = np.ascontiguousarray(v, dtype=np.float64).ravel()
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

        def ints(v):
            a = np.ascontiguousarray(v, dtype=np.int32).ravel()
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))

        d = _ModelDesc()
        d.total_spin = 1 if self.total_spin else 0
        d.site_nqn = 3 if self.total_spin else 2
        d.site_nblocks = len(self.site_bsize)
        d.site_qn = dbl(self.site_qn)
        d.site_bsize = ints(self.site_bsize)
        d.hn_form = self.hn_form
        d.onsite = 1 if self.onsite else 0
        hc = guard(lambda u, S, ti, tj, ch, sg, dr: float(self.hn_coef(S, ti, tj, ch, sg, dr)), float("nan"))
        of = guard(lambda u, o, si, sj, ti, tj: float(self.op_factor(o, si, sj, ti, tj)), float("nan"))
        oc = guard(lambda u, o, qi, qj: 1 if self.op_check(o, (qi[0], qi[1]), (qj[0], qj[1])) else 0, 0)
        d.hn_coef = _HN_COEF_FN(hc)
        d.op_factor = _OP_FACTOR_FN(of)
        d.op_check = _OP_CHECK_FN(oc)
        keep.extend([d.hn_coef, d.op_factor, d.op_check])
        d.nops = len(self.op_class)
        d.op_class = ints(self.op_class)
        d.op_avg = ints(self.op_avg)
        d.start_nblocks = len(self.start_bsize)
        d.start_qn = dbl(self.start_qn)
        d.start_bsize = ints(self.start_bsize)
        d.start_en = dbl(self.start_en)
        d.start_npairs = ints([len(p) for p in self.start_ops])
        d.start_pairs = ints([[bi, bj] for p in self.start_ops for bi, bj, _ in p] or [0])
        d.start_el = dbl(np.concatenate([np.asarray(b, dtype=np.float64).ravel()
                                         for p in self.start_ops for _, _, b in p] or [np.zeros(1)]))
        return d


_dp_ = ctypes.POINTER(ctypes.c_double)


class ModelTables:
    """The host tables of a model (nrg_model_hn_table / nrg_model_op_factor /
    nrg_model_op_check): a built-in model by name or a ModelPlugin.  Needs no
    device."""

    def __init__(self, model):
        self.L = load_library()
        self._keep, self._errors = [], []
        if isinstance(model, ModelPlugin):
            self.model, self.desc = -1, ctypes.byref(model._desc(self._keep, self._errors))
        else:
            self.model, self.desc = MODELS[model], None

    def _call(self, st):
        if self._errors:
            raise self._errors.pop(0)
        if st != 0:
            raise NRGError(st, STATUS.get(st, "error"))

    def hn_table(self, s_block: float) -> np.ndarray:
        n = ctypes.c_int()
        self._call(self.L.nrg_model_hn_table(self.model, self.desc, s_block, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        self._call(self.L.nrg_model_hn_table(self.model, self.desc, s_block,
                                             out.ctypes.data_as(_dp_), n.value, ctypes.byref(n)))
        return out

    def op_factor(self, op: int, s_i: float, s_j: float, ti: int, tj: int) -> float:
        v = ctypes.c_double()
        self._call(self.L.nrg_model_op_factor(self.model, self.desc, op, s_i, s_j, ti, tj, ctypes.byref(v)))
        return v.value

    def op_check(self, op: int, qn_i, qn_j) -> bool:
        a = (ctypes.c_double * 2)(*qn_i)
        b = (ctypes.c_double * 2)(*qn_j)
        v = ctypes.c_int()
        self._call(self.L.nrg_model_op_check(self.model, self.desc, op, a, b, ctypes.byref(v)))
        return bool(v.value)


def clebsch(j1: float, m1: float, j2: float, m2: float, j: float, m: float) -> float:
    """nrg_clebsch: <j1 m1; j2 m2 | j m> as the engine computes it."""
    return load_library().nrg_clebsch(j1, m1, j2, m2, j, m)


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
    L.nrg_sweep_run_model.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig), ctypes.POINTER(_ModelDesc)]
    L.nrg_model_hn_table.argtypes = [ctypes.c_int, ctypes.POINTER(_ModelDesc), ctypes.c_double, _dp_, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int)]
    L.nrg_model_op_factor.argtypes = [ctypes.c_int, ctypes.POINTER(_ModelDesc), ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp_]
    L.nrg_model_op_check.argtypes = [ctypes.c_int, ctypes.POINTER(_ModelDesc), ctypes.c_int, _dp_, _dp_,
                                     ctypes.POINTER(ctypes.c_int)]
    L.nrg_clebsch.argtypes = [ctypes.c_double] * 6
    L.nrg_clebsch.restype = ctypes.c_double
    L.nrg_sweep_num_iterations.argtypes = [ctypes.c_void_p]
    L.nrg_sweep_iteration.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Iteration)]
    L.nrg_sweep_opavg_initial.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
    L.nrg_sweep_timing.argtypes = [ctypes.c_void_p, ctypes.POINTER(Timing)]
    L.nrg_fp64_peak.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    _dp = ctypes.POINTER(ctypes.c_double)
    _ip = ctypes.POINTER(ctypes.c_int)
    L.nrg_diag_blocks.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp, _dp, _dp]
    L.nrg_set_precision.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.nrg_grad_forward.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig), ctypes.POINTER(_Grad)]
    L.nrg_grad_backward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_double)]
    L.nrg_dm_load_bin.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    L.nrg_gemm_f64_tensor.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
    L.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    L.cudaFree.argtypes = [ctypes.c_void_p]
    L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    L.nrg_diag_hn.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int, ctypes.POINTER(_Blocks),
                              ctypes.c_int, ctypes.POINTER(_Matrix), ctypes.POINTER(_Basis), _dp, _dp, _dp]
    L.nrg_diag_hn_model.argtypes = [ctypes.c_void_p, ctypes.POINTER(_ModelDesc), _dp, ctypes.c_int,
                                    ctypes.POINTER(_Blocks), ctypes.c_int, ctypes.POINTER(_Matrix),
                                    ctypes.POINTER(_Basis), _dp, _dp, _dp]
    L.nrg_update_ops_model.argtypes = [ctypes.c_void_p, ctypes.POINTER(_ModelDesc), ctypes.POINTER(_Blocks),
                                       ctypes.POINTER(_Basis), ctypes.POINTER(_EigCut), ctypes.c_int,
                                       ctypes.POINTER(_Matrix), ctypes.POINTER(_Matrix)]
    L.nrg_cut_states.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Blocks), _dp, _dp, ctypes.c_int,
                                 ctypes.c_double, ctypes.POINTER(_CutResult)]
    L.nrg_update_ops.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Blocks), ctypes.POINTER(_Basis),
                                 ctypes.POINTER(_EigCut), ctypes.c_int, ctypes.POINTER(_Matrix),
                                 ctypes.POINTER(_Matrix)]
    L.nrg_sweep_run_dm.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig)]
    L.nrg_dm_num_shells.argtypes = [ctypes.c_void_p]
    L.nrg_dm_backprop.argtypes = [ctypes.c_void_p, ctypes.POINTER(DmParams), _dp]
    L.nrg_lehmann.argtypes = [ctypes.c_void_p, ctypes.POINTER(DmParams), ctypes.c_int, _dp, _dp, _ip]
    L.nrg_grad_forward_dm.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig), ctypes.POINTER(_Grad)]
    L.nrg_lehmann_grad.argtypes = [ctypes.c_void_p, ctypes.POINTER(DmParams), ctypes.c_int, _dp, _dp, _dp, _ip]
    L.nrg_lehmann_grad_backward.argtypes = [ctypes.c_void_p, _dp, _dp]
    L.nrg_write_dm_shell.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(DmShell)]
    L.nrg_write_code_pars.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_int, ctypes.c_char_p]
    L.nrg_dm_save_bin.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]
    L.nrg_sweep_run_chain.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig)]
    L.nrg_thermo_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(SweepConfig), ctypes.c_int,
                                 ctypes.POINTER(_Thermo)]
    L.nrg_write_thermo.argtypes = [ctypes.c_char_p, ctypes.c_int, _dp, _dp, _dp]
    L.nrg_set_chain.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_int]
    L.nrg_chain_lanczos.argtypes = [ctypes.POINTER(_Band), ctypes.c_int, _dp, _dp, _dp]
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
    wall_ms: float = 0.0     # host wall time of the iteration
    device_ms: float = 0.0   # CUDA-event span of the iteration on the engine stream


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

    def set_precision(self, precision: int) -> None:
        """Arithmetic of diag_blocks / diag_hn on this context (PREC_FP64 or
        PREC_MIXED); a sweep sets it from its own argument."""
        self._check(self.L.nrg_set_precision(self.h, int(precision)))

    def gemm_f64_tensor(self, A, B, C, alpha: float = 1.0, slices: int = 6):
        """C + alpha A B^T through nrg_gemm_f64_tensor (split-BF16 products on
        the tensor cores); A (m, k), B (n, k), C (m, n) host arrays, copied to
        and from device buffers allocated for the call.  Returns the new C."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        C = np.array(C, dtype=np.float64, order="C", copy=True)
        m, k = A.shape
        n = B.shape[0]
        L = self.L
        bufs = []
        try:
            for arr in (A, B, C):
                p = ctypes.c_void_p()
                if L.cudaMalloc(ctypes.byref(p), max(arr.nbytes, 8)) != 0:
                    raise NRGError(3, "cudaMalloc failed")
                bufs.append(p)
                if L.cudaMemcpy(p, arr.ctypes.data, arr.nbytes, 1) != 0:
                    raise NRGError(2, "cudaMemcpy failed")
            self._check(L.nrg_gemm_f64_tensor(self.h, m, n, k, float(alpha), bufs[0], k, bufs[1], k, bufs[2], n,
                                              int(slices)))
            if L.cudaMemcpy(C.ctypes.data, bufs[2], C.nbytes, 2) != 0:
                raise NRGError(2, "cudaMemcpy failed")
        finally:
            for p in bufs:
                L.cudaFree(p)
        return C

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

    # ---- per-step drop-ins (the NRG_main call sites) ----------------------
    # Arrays follow the reference containers: qn (nblocks, 2) QNumbers,
    # bbe [2*nblocks] inclusive BlockBegEnd, operators as (MatBlockMap,
    # MatBlockBegEnd, MatEl) triples in the model's operator order.

    def diag_hn(self, model, params, old_qn, old_bbe, ops, basis_qn, basis_bbe, itype, stcf, basis_en):
        """CNRGmatrix::DiagHN + SetE0zero for a built-in model (its name) or a
        ModelPlugin (nrg_diag_hn_model).  Returns (en, eigvec, emin): en the
        E_min-shifted eigenvalues (ascending per block), eigvec the
        block-concatenated n x n matrices (row k = eigenvector k)."""
        k = _Keep()
        params = np.ascontiguousarray(params, dtype=np.float64)
        old = k.blocks(old_qn, old_bbe)
        mats = (_Matrix * len(ops))(*[k.matrix(m) for m in ops])
        basis = _Basis(k.blocks(basis_qn, basis_bbe), k.i(itype), k.i(stcf), k.d(basis_en))
        bbe = np.asarray(basis_bbe, dtype=np.int64)
        sizes = bbe[1::2] - bbe[0::2] + 1
        en = np.empty(int(sizes.sum()), dtype=np.float64)
        vec = np.empty(int((sizes ** 2).sum()), dtype=np.float64)
        emin = ctypes.c_double()
        if isinstance(model, ModelPlugin):
            keep, errors = [], []
            desc = model._desc(keep, errors)
            st = self.L.nrg_diag_hn_model(self.h, ctypes.byref(desc), params.ctypes.data_as(_DP), len(params),
                                          ctypes.byref(old), len(ops), mats, ctypes.byref(basis),
                                          en.ctypes.data_as(_DP), vec.ctypes.data_as(_DP), ctypes.byref(emin))
            if errors:
                raise errors[0]
            self._check(st)
        else:
            self._check(self.L.nrg_diag_hn(self.h, MODELS[model], params.ctypes.data_as(_DP), len(params),
                                           ctypes.byref(old), len(ops), mats, ctypes.byref(basis),
                                           en.ctypes.data_as(_DP), vec.ctypes.data_as(_DP), ctypes.byref(emin)))
        return en, vec, emin.value

    def cut_states(self, qn, bbe, en, eigvec, ncutoff: int, degen_eps: float = 0.0) -> dict:
        """SetKept + CutStates on Aeig.  Returns a dict with en/kept/nkept/ecut
        (Aeig after SetKept) and AeigCut's qn, bbe, bbe_bc, bbe_eig, stcf,
        cut_en, cut_kept, eigvec."""
        k = _Keep()
        blk = k.blocks(qn, bbe)
        en = np.ascontiguousarray(en, dtype=np.float64)
        evp = k.d(eigvec) if eigvec is not None else None
        r = _CutResult()
        self._check(self.L.nrg_cut_states(self.h, ctypes.byref(blk), en.ctypes.data_as(_DP), evp,
                                          int(ncutoff), float(degen_eps), ctypes.byref(r)))
        ns = len(en)
        c = r.cut
        nb = c.blocks.nblocks
        bbe_c = _arr(c.blocks.block_beg_end, 2 * nb, np.int64)
        nk = int(bbe_c[-1] + 1) if nb else 0
        bbe_eig = _arr(c.block_beg_end_eigvec, 2 * nb, np.int64)
        out = dict(en=_arr(r.en, ns, np.float64), kept=_arr(r.kept, ns, np.int64), nkept=r.nkept, ecut=r.ecut,
                   qn=_arr(c.blocks.qnumbers, 2 * nb, np.float64), bbe=bbe_c,
                   bbe_bc=_arr(c.block_beg_end_bc, 2 * nb, np.int64), bbe_eig=bbe_eig,
                   stcf=_arr(c.st_came_from, nk, np.int64), cut_en=_arr(c.en, nk, np.float64),
                   cut_kept=_arr(c.kept, nk, np.int64), eigvec=None)
        if eigvec is not None:
            out["eigvec"] = _arr(c.eigvec, int(bbe_eig[-1] + 1) if nb else 0, np.float64)
        return out

    def update_ops(self, model, old_qn, old_bbe, basis_qn, basis_bbe, itype, stcf, basis_en,
                   cut_qn, cut_bbe, cut_bbe_eig, cut_eigvec, ops):
        """UpdateMatrices for all of the model's operators, a built-in model
        (its name) or a ModelPlugin (nrg_update_ops_model).  Returns the new
        operators as (MatBlockMap, MatBlockBegEnd, MatEl) triples."""
        k = _Keep()
        old = k.blocks(old_qn, old_bbe)
        basis = _Basis(k.blocks(basis_qn, basis_bbe), k.i(itype), k.i(stcf), k.d(basis_en))
        cut = _EigCut(k.blocks(cut_qn, cut_bbe), None, k.i(cut_bbe_eig), None, None, None, k.d(cut_eigvec))
        mats = (_Matrix * len(ops))(*[k.matrix(m) for m in ops])
        new = (_Matrix * len(ops))()
        if isinstance(model, ModelPlugin):
            keep, errors = [], []
            desc = model._desc(keep, errors)
            st = self.L.nrg_update_ops_model(self.h, ctypes.byref(desc), ctypes.byref(old), ctypes.byref(basis),
                                             ctypes.byref(cut), len(ops), mats, new)
            if errors:
                raise errors[0]
            self._check(st)
        else:
            self._check(self.L.nrg_update_ops(self.h, MODELS[model], ctypes.byref(old), ctypes.byref(basis),
                                              ctypes.byref(cut), len(ops), mats, new))
        res = []
        for m in new:
            nmb = m.nmatblocks
            mbe = _arr(m.mat_block_beg_end, 2 * nmb, np.int64)
            nel = int(mbe.max() + 1) if nmb else 0
            res.append((_arr(m.mat_block_map, 2 * nmb, np.int64), mbe, _arr(m.mat_el, nel, np.float64)))
        return res

    # ---- DM-NRG spectral function ---------------------------------------
    def sweep_dm(self, nsites: int, ncutoff: int, lam: float, U: float, ed: float, gamma: float,
                 degen_eps: float = 0.0, model: str = "1chQS", gamma2: float = 0.0) -> int:
        """Forward sweep of the |Q S> Anderson model (model "1chQS", or "2chQS"
        with Gamma1 = gamma and Gamma2 = gamma2) keeping the DM-NRG shells on
        the device; returns the number of shells."""
        if model not in ("1chQS", "2chQS"):
            raise NRGError(f"DM-NRG shells are available for 1chQS and 2chQS, not {model!r}")
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, U, ed, gamma, gamma2 if model == "2chQS" else 0.0,
                          degen_eps, PREC_FP64)
        self._check(self.L.nrg_sweep_run_dm(self.h, ctypes.byref(cfg)))
        self._dm_site_dim = 16.0 if model == "2chQS" else 4.0
        return int(self.L.nrg_dm_num_shells(self.h))

    def dm_params(self, temp: float = 0.0, mtemp: int = -1, betabar: float = 0.727, bbroad: float = 0.6,
                  twindow: float = 2.0, broadtemp: float = 0.8, site_dim: float | None = None,
                  nw: int = 4) -> DmParams:
        """DM_NRG's parameters; site_dim (states per Wilson site in the FDM
        weights) defaults to that of the last sweep_dm: 4, or 16 for two
        channels."""
        if site_dim is None:
            site_dim = getattr(self, "_dm_site_dim", 4.0)
        return DmParams(temp, mtemp, betabar, bbroad, twindow, broadtemp, site_dim, nw)

    def dm_backprop(self, prm: DmParams) -> np.ndarray:
        """Density-matrix backward sweep; returns the trace per shell."""
        n = int(self.L.nrg_dm_num_shells(self.h))
        tr = np.zeros(max(n, 1))
        self._check(self.L.nrg_dm_backprop(self.h, ctypes.byref(prm), tr.ctypes.data_as(_DP)))
        return tr[:n]

    def lehmann(self, prm: DmParams, omegas=None, capacity: int = 0):
        """A(omega) of c_d; omegas=None uses the reference's grid.
        Returns (omega, A)."""
        n_sh = int(self.L.nrg_dm_num_shells(self.h))
        if omegas is None:
            cap = capacity or 2 * prm.nw * n_sh + 8
            om_ptr = None
        else:
            om = np.ascontiguousarray(omegas, dtype=np.float64)
            cap = len(om)
            om_ptr = om.ctypes.data_as(_DP)
        out = np.zeros(2 * max(cap, 1))
        nout = ctypes.c_int(0)
        self._check(self.L.nrg_lehmann(self.h, ctypes.byref(prm), cap, om_ptr, out.ctypes.data_as(_DP),
                                       ctypes.byref(nout)))
        n = nout.value
        return out[:n].copy(), out[cap:cap + n].copy()

    def grad_forward_dm(self, nsites: int, ncutoff: int, lam: float, U: float, ed: float, gamma: float,
                        degen_eps: float = 0.0) -> GradResult:
        """nrg_grad_forward_dm: sweep_dm of the one-channel |Q S> model with the
        tangent pass; afterwards dm_backprop also builds the density matrices'
        tangents and lehmann_grad gives d A(omega) / d (eps_d, U, Gamma, B)."""
        cfg = SweepConfig(MODELS["1chQS"], nsites, ncutoff, lam, U, ed, gamma, 0.0, degen_eps, PREC_FP64, 0.0)
        g = _Grad()
        self._check(self.L.nrg_grad_forward_dm(self.h, ctypes.byref(cfg), ctypes.byref(g)))
        self._dm_site_dim = 4.0
        n, k, no = g.nsites, g.nparams, g.nops
        return GradResult(self._fetch(True), _arr(g.d_thermo, n * k * 16, np.float64).reshape(n, k, 4, 4),
                          _arr(g.d_opavg, n * k * no, np.float64).reshape(n, k, no),
                          _arr(g.d_emin, n * k, np.float64).reshape(n, k), _arr(g.egs, n, np.float64),
                          _arr(g.d_egs, n * k, np.float64).reshape(n, k))

    def lehmann_grad(self, prm: DmParams, omegas=None, capacity: int = 0):
        """nrg_lehmann_grad after grad_forward_dm and dm_backprop: returns
        (omega, A, dA) with dA[k, j] = d A(omega_j) / d p_k, p = (eps_d, U,
        Gamma, B)."""
        n_sh = int(self.L.nrg_dm_num_shells(self.h))
        if omegas is None:
            cap = capacity or 2 * prm.nw * n_sh + 8
            om_ptr = None
        else:
            om = np.ascontiguousarray(omegas, dtype=np.float64)
            cap = len(om)
            om_ptr = om.ctypes.data_as(_DP)
        out = np.zeros(2 * max(cap, 1))
        dout = np.zeros(4 * max(cap, 1))
        nout = ctypes.c_int(0)
        self._check(self.L.nrg_lehmann_grad(self.h, ctypes.byref(prm), cap, om_ptr, out.ctypes.data_as(_DP),
                                            dout.ctypes.data_as(_DP), ctypes.byref(nout)))
        n = nout.value
        self._lehmann_grad_n = n
        return out[:n].copy(), out[cap:cap + n].copy(), dout.reshape(4, max(cap, 1))[:, :n].copy()

    def lehmann_grad_backward(self, g_rhow) -> np.ndarray:
        """nrg_lehmann_grad_backward: sum_j g_rhow[j] d A(omega_j) / d p over the
        frequencies of the last lehmann_grad."""
        g = np.ascontiguousarray(g_rhow, dtype=np.float64)
        if g.shape != (getattr(self, "_lehmann_grad_n", -1),):
            raise ValueError("g_rhow must hold one weight per frequency of the last lehmann_grad")
        out = np.zeros(4)
        self._check(self.L.nrg_lehmann_grad_backward(self.h, g.ctypes.data_as(_DP), out.ctypes.data_as(_DP)))
        return out

    def dm_save_bin(self, directory: str, name: str) -> None:
        """The DM-NRG shells as the reference's .bin files plus ThisCodePars.dat."""
        self._check(self.L.nrg_dm_save_bin(self.h, directory.encode(), name.encode()))

    def dm_load_bin(self, directory: str, name: str, nshells: int = 0) -> int:
        """DM-NRG shells from the reference's .bin files (NRG_main with the
        spectral density on, or dm_save_bin) and ThisCodePars.dat; afterwards
        dm_backprop and lehmann run on them.  Returns the number of shells."""
        self._check(self.L.nrg_dm_load_bin(self.h, directory.encode(), name.encode(), int(nshells)))
        return int(self.L.nrg_dm_num_shells(self.h))

    def timing(self) -> dict:
        t = Timing()
        self._check(self.L.nrg_sweep_timing(self.h, ctypes.byref(t)))
        return t.as_dict()

    def fp64_peak(self) -> float:
        """Measured FP64 FMA throughput of the device, TFLOP/s."""
        v = ctypes.c_double()
        self._check(self.L.nrg_fp64_peak(self.h, ctypes.byref(v)))
        return v.value

    def set_chain(self, chi=None, en=None, alambda: bool = True):
        """Use the chain (chi_N, e_N) in the following sweeps (nrg_set_chain);
        no arguments: back to the flat band's Wilson chain."""
        if chi is None:
            self._check(self.L.nrg_set_chain(self.h, 0, None, None, 1))
            return
        self._chain = (np.ascontiguousarray(chi, dtype=np.float64), np.ascontiguousarray(en, dtype=np.float64))
        c, e = self._chain
        if len(c) != len(e):
            raise ValueError("chi and en must have the same length")
        self._check(self.L.nrg_set_chain(self.h, len(c), c.ctypes.data_as(_DP), e.ctypes.data_as(_DP),
                                         1 if alambda else 0))

    def sweep_chain(self, model: str, nsites: int, ncutoff: int, lam: float, degen_eps: float = 0.0,
                    precision: int = PREC_FP64, fetch: bool = True) -> SweepResult:
        """The free Wilson chain (calcdens = 3): iteration 0 is the first site
        alone, iterations 1 .. nsites-1 add one site each."""
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, 0.0, 0.0, 0.0, 0.0, degen_eps, precision)
        self._check(self.L.nrg_sweep_run_chain(self.h, ctypes.byref(cfg)))
        return self._fetch(fetch)

    def thermo(self, model: str, nsites: int, ncutoff: int, lam: float, U: float, ed: float,
               gamma1: float, gamma2_or_B: float = 0.0, degen_eps: float = 0.0,
               precision: int = PREC_FP64, reuse_chain: bool = True) -> ThermoResult:
        """Impurity T chi and S with the free chain subtracted (calcdens = 3
        then 2): the chain sweep runs beside the impurity sweep on a second
        stream, or is reused from the last call with the same chain
        parameters.  The impurity sweep stays readable through fetch()."""
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, U, ed, gamma1, gamma2_or_B,
                          degen_eps, precision)
        t = _Thermo()
        self._check(self.L.nrg_thermo_run(self.h, ctypes.byref(cfg), 1 if reuse_chain else 0, ctypes.byref(t)))
        n = t.nvalues
        return ThermoResult(_arr(t.temp, n, np.float64), _arr(t.suscep, n, np.float64),
                            _arr(t.suscep_chain, n, np.float64), _arr(t.suscep_imp, n, np.float64),
                            _arr(t.entropy, n, np.float64), _arr(t.entropy_chain, n, np.float64),
                            _arr(t.entropy_imp, n, np.float64), bool(t.chain_reused), t.chain_ms,
                            t.imp_ms, t.total_ms, model)

    def sweep(self, model: str, nsites: int, ncutoff: int, lam: float, U: float, ed: float,
              gamma1: float, gamma2_or_B: float = 0.0, degen_eps: float = 0.0,
              precision: int = PREC_FP64, fetch: bool = True, delta_sc: float = 0.0) -> SweepResult:
        """One sweep (nrg_sweep_run).  gamma2_or_B: Gamma2 (2chQS) or the field B
        (1chQSz, 1chSz); delta_sc: the leads' gap (1chS, 1chSz)."""
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, U, ed, gamma1, gamma2_or_B,
                          degen_eps, precision, delta_sc)
        self._check(self.L.nrg_sweep_run(self.h, ctypes.byref(cfg)))
        return self._fetch(fetch)

    def sweep_model(self, plugin: ModelPlugin, nsites: int, ncutoff: int, lam: float, gamma1: float,
                    gamma2: float = 0.0, degen_eps: float = 0.0, precision: int = PREC_FP64,
                    fetch: bool = True) -> SweepResult:
        """One sweep of a caller-described model (nrg_sweep_run_model);
        gamma1 (and gamma2 with two channels) give chi_{-1}."""
        cfg = SweepConfig(-1, nsites, ncutoff, lam, 0.0, 0.0, gamma1, gamma2, degen_eps, precision, 0.0)
        keep, errors = [], []
        desc = plugin._desc(keep, errors)
        st = self.L.nrg_sweep_run_model(self.h, ctypes.byref(cfg), ctypes.byref(desc))
        if errors:
            raise errors[0]
        self._check(st)
        return self._fetch(fetch)

    def grad_forward(self, model: str, nsites: int, ncutoff: int, lam: float, U: float, ed: float,
                     gamma1: float, B: float = 0.0, degen_eps: float = 0.0) -> GradResult:
        """nrg_grad_forward: the sweep of the one-channel Anderson model ("1chQS"
        or "1chQSz") and the derivatives of every iteration's reported values
        with respect to (eps_d, U, Gamma1, B) at its kept-state set."""
        cfg = SweepConfig(MODELS[model], nsites, ncutoff, lam, U, ed, gamma1, B, degen_eps, PREC_FP64, 0.0)
        g = _Grad()
        self._check(self.L.nrg_grad_forward(self.h, ctypes.byref(cfg), ctypes.byref(g)))
        n, k, no = g.nsites, g.nparams, g.nops
        return GradResult(self._fetch(True), _arr(g.d_thermo, n * k * 16, np.float64).reshape(n, k, 4, 4),
                          _arr(g.d_opavg, n * k * no, np.float64).reshape(n, k, no),
                          _arr(g.d_emin, n * k, np.float64).reshape(n, k), _arr(g.egs, n, np.float64),
                          _arr(g.d_egs, n * k, np.float64).reshape(n, k))

    def grad_backward(self, g_thermo=None, g_opavg=None, g_egs=None) -> np.ndarray:
        """nrg_grad_backward: the gradient of sum(g_thermo * thermo) +
        sum(g_opavg * opavg) + sum(g_egs * egs) over the iterations of the last
        grad_forward, with respect to (eps_d, U, Gamma1, B)."""
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data_as(ctypes.c_void_p)

        out = np.zeros(4)
        self._check(self.L.nrg_grad_backward(self.h, ptr(g_thermo), ptr(g_opavg), ptr(g_egs),
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def fetch(self) -> SweepResult:
        """The iterations of the last sweep on this context."""
        return self._fetch(True)

    def _fetch(self, fetch: bool) -> SweepResult:
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
                kept_bsize=_arr(it.kept_block_size, it.nkept_blocks, np.int64),
                wall_ms=it.wall_ms, device_ms=it.device_ms))
        return out


@dataclass
class BatchResult:
    thermo: np.ndarray   # (ninst, max_sites, 4, 4)
    opavg: np.ndarray    # (ninst, max_sites, 4)
    nkept: np.ndarray    # (ninst, max_sites)
    seconds: float


def sweep_batch(instances, nworkers: int = 8, device: int = 0, precision: int = PREC_FP64) -> BatchResult:
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


__all__ = ["Engine", "NRGError", "SweepResult", "Iteration", "BatchResult", "GradResult", "load_library", "sweep_batch",
           "MODELS"]
