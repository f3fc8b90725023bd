"""Built-in models restated as caller-supplied plug-ins (nrg_model_desc).

Each function returns a twochnrg_gb300.ModelPlugin whose rules are written
here in Python from the reference's model code, the way a user would add a
model: the site basis (SetSingleSite), the H_N rule (CalcHNMatEl), the
operator rules (CalcMatEl) and selection rules (CheckForMatEl), and H_{-1}
(*_SetAnderson_Hm1).  Sums and products follow the reference's order, so the
coefficient tables equal the built-in models' bit for bit.
"""
import math

import numpy as np

import twochnrg_gb300 as tg


def _deq(a, b):  # dEqual.cpp:6
    return abs(a - b) < 1.0e-20


def _find(qn, q):
    """GetBlockFromQNumbers over the site blocks: index or -1."""
    for b, x in enumerate(qn):
        if all(_deq(x[k], q[k]) for k in range(len(q))):
            return b
    return -1


def _fd(sigma, ti, tj):
    """OneCh_fd_table (OpTables.cpp:8-33): <t_i| f^dagger_sigma |t_j> in
    |0>, |up>, |dn>, |up dn>."""
    if sigma == 1:
        return 1.0 if (ti == 1 and tj == 0) or (ti == 3 and tj == 2) else 0.0
    if sigma == -1:
        if ti == 2 and tj == 0:
            return 1.0
        if ti == 3 and tj == 1:
            return -1.0
    return 0.0


def _start_ops_diag(sizes, values):
    return [(b, b, np.array([[v]])) for b, v in enumerate(values)]


def one_channel_qs(U, ed, lam):
    """One-channel Anderson model in the |Q S> basis (SymNo 0)."""
    cg = tg.clebsch
    site = [(-1.0, 0.0, 0.0), (0.0, 0.5, 0.5), (0.0, 0.5, -0.5), (1.0, 0.0, 0.0)]  # OneChQS_SetSingleSite

    def coef(Si, typep, typ):
        # OneChQS_HN_MatEl (OpMatRules.cpp:1473-1523) for the site pair
        # (typep, typ) in a multiplet of spin Si, times the fermion sign
        Qtp, Stp, Sztp = site[typep]
        Qt, Stt, Szt = site[typ]
        Scfp, Scf = Si - Sztp, Si - Szt
        fermi = -1.0 if _deq(Qt, 0.0) else 1.0
        acc = 0.0
        Sz = -Stt
        while Sz <= Stt:
            sst = _find(site, (Qt, Stt, Sz))
            for sigma in (-1, 1):
                dS = 0.5 * sigma
                Szcf = Si - Sz
                Szcfp, Szp = Szcf - dS, Sz + dS
                sstp = _find(site, (Qtp, Stp, Sz + dS))
                a0 = cg(Scf, Szcf, Stt, Sz, Si, Si)
                a1 = cg(Scfp, Szcfp, Stp, Szp, Si, Si)
                a2 = cg(Scfp, Szcfp, 0.5, dS, Scf, Szcf)
                a3 = _fd(sigma, sstp, sst)
                acc += a0 * a1 * a2 * a3
            Sz += 1.0
        return acc * fermi

    def hn_coef(S, ti, tj, ch, sg, dr):
        return coef(S, ti, tj) if dr == 0 else coef(S, tj, ti)

    def op_factor(o, Si, Sj, ti, tj):
        # OneChQS_fN_MatEl (OpMatRules.cpp:1167-1244)
        Qi, Sti, Szti = site[ti]
        Qj, Stj, Sztj = site[tj]
        Scfi, Scfj = Si - Szti, Sj - Sztj
        acc = 0.0
        sigma = Sj - Si
        Sz = -Stj
        while Sz <= Stj:
            sj = _find(site, (Qj, Stj, Sz))
            si = _find(site, (Qi, Sti, Sz - sigma))
            c0 = cg(Scfi, Si - Sz + sigma, Sti, Sz - sigma, Si, Si)
            c1 = cg(Scfj, Sj - Sz, Stj, Sz, Sj, Sj)
            acc += _fd(int(sigma / 0.5), sj, si) * c0 * c1
            Sz += 1.0
        n0 = cg(Si, Si, 0.5, sigma, Sj, Sj)
        return acc / n0 if not _deq(n0, 0.0) else 0.0

    def op_check(o, qi, qj):
        if o == 0:  # OneChQS_cd_check (OpMatRules.cpp:106)
            return _deq(qj[0], qi[0] + 1.0) and (_deq(qj[1], qi[1] + 0.5) or _deq(qj[1], qi[1] - 0.5))
        return qi == qj  # Diag_check (OpMatRules.cpp:12): the same kept block

    # OneChQS_SetAnderson_Hm1 (Main/Main_SetH0.cpp:1794-1969)
    scale = lam * 0.5 * (1.0 + 1.0 / lam)
    blocks = [(-1.0, 0.0), (0.0, 0.5), (1.0, 0.0)]
    n = [q + 1.0 for q, _ in blocks]
    return tg.ModelPlugin(
        total_spin=True, site_qn=site, site_bsize=[1, 1, 1, 1], hn_form=tg.HN_ONE_OP, onsite=True,
        hn_coef=hn_coef, op_class=[tg.OP_SITE, tg.OP_IMPURITY_DIAG, tg.OP_IMPURITY_DIAG, tg.OP_IMPURITY_DIAG],
        op_avg=[0, 1, 1, 1], op_factor=op_factor, op_check=op_check,
        start_qn=blocks, start_bsize=[1, 1, 1],
        start_en=[0.5 * U / scale, (ed + 0.5 * U) / scale, (2.0 * ed + 1.5 * U) / scale],
        start_ops=[[(0, 1, np.array([[1.0]])), (1, 2, np.array([[-math.sqrt(2.0)]]))],
                   _start_ops_diag(3, n), _start_ops_diag(3, [x * x for x in n]),
                   _start_ops_diag(3, [S * (S + 1.0) for _, S in blocks])])


def one_channel_qsz(U, ed, B, lam):
    """One-channel Anderson model in the |Q Sz> basis with a Zeeman field (SymNo 2)."""
    site = [(-1.0, 0.0), (0.0, 0.5), (0.0, -0.5), (1.0, 0.0)]  # OneChQSz_SetSingleSite

    def charge_sign(t):
        return -1.0 if _deq(site[t][0], 0.0) else 1.0

    def hn_coef(S, ti, tj, ch, sg, dr):
        # OneChQSz_HN_MatEl (OpMatRules.cpp:468-531): per spin, the fermion
        # sign of the "type" state times <typep| f^dagger_sigma |type>
        sigma = 1 if sg == 0 else -1
        return charge_sign(tj) * _fd(sigma, ti, tj) if dr == 0 else charge_sign(ti) * _fd(sigma, tj, ti)

    def op_factor(o, Si, Sj, ti, tj):  # OneChQ_fN_MatEl (OpMatRules.cpp:1003-1033)
        return _fd(1 if o == 0 else -1, tj, ti)

    def op_check(o, qi, qj):
        if o < 2:  # OneChQ_cd_check (OpMatRules.cpp:92)
            return _deq(qj[0], qi[0] + 1.0)
        return qi == qj

    # OneChQSz_SetAnderson_Hm1 (Main/Main_SetH0.cpp:421-660), hz = B/2
    scale = lam * 0.5 * (1.0 + 1.0 / lam)
    hz = 0.5 * B
    blocks = [(-1.0, 0.0), (0.0, 0.5), (0.0, -0.5), (1.0, 0.0)]
    one = lambda i, j, v: (i, j, np.array([[v]]))  # noqa: E731
    return tg.ModelPlugin(
        total_spin=False, site_qn=site, site_bsize=[1, 1, 1, 1], hn_form=tg.HN_SPIN_SUM, onsite=True,
        hn_coef=hn_coef, op_class=[tg.OP_SITE, tg.OP_SITE, tg.OP_IMPURITY_DIAG, tg.OP_IMPURITY_DIAG],
        op_avg=[0, 0, 1, 1], op_factor=op_factor, op_check=op_check,
        start_qn=blocks, start_bsize=[1, 1, 1, 1],
        start_en=[0.5 * U / scale, (ed + 0.5 * U - hz) / scale, (ed + 0.5 * U + hz) / scale,
                  (2.0 * ed + 1.5 * U) / scale],
        start_ops=[[one(0, 1, 1.0), one(2, 3, 1.0)], [one(0, 2, 1.0), one(1, 3, -1.0)],
                   _start_ops_diag(4, [q + 1.0 for q, _ in blocks]), _start_ops_diag(4, [s for _, s in blocks])])
