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


def _two_channel_tables():
    """TwoChQS_fd_table (TwoChQS_OpTables.cpp:20-130): f^dagger_{ch,sigma} in
    the 16-state two-channel site basis, fd[ch-1][sigma == +1][ti][tj]; and
    TwoChQS_SpSm_table (:140-185), which links the members of a multiplet."""
    fd = np.zeros((2, 2, 16, 16))
    r, mr = 1.0 / math.sqrt(2.0), -1.0 / math.sqrt(2.0)
    u1, d1, u2, d2 = fd[0][1], fd[0][0], fd[1][1], fd[1][0]
    for (i, j), v in {(2, 0): 1, (10, 1): 1, (9, 3): r, (11, 6): 1, (5, 3): r, (7, 4): 1, (12, 9): r, (12, 5): mr,
                      (14, 8): 1, (15, 13): 1}.items():
        u1[i, j] = v
    for (i, j), v in {(4, 0): 1, (9, 1): r, (5, 1): mr, (8, 3): 1, (13, 6): 1, (7, 2): -1, (12, 10): -1,
                      (14, 9): mr, (14, 5): mr, (15, 11): -1}.items():
        d1[i, j] = v
    for (i, j), v in {(1, 0): 1, (6, 3): 1, (10, 2): -1, (11, 9): mr, (11, 5): mr, (9, 4): mr, (5, 4): r,
                      (13, 8): -1, (12, 7): 1, (15, 14): 1}.items():
        u2[i, j] = v
    for (i, j), v in {(3, 0): 1, (6, 1): -1, (9, 2): mr, (11, 10): 1, (5, 2): mr, (8, 4): -1, (13, 9): r,
                      (13, 5): mr, (14, 7): 1, (15, 12): -1}.items():
        d2[i, j] = v
    spsm = np.eye(16)
    for i, j in [(1, 3), (2, 4), (11, 13), (12, 14), (8, 9), (9, 10), (8, 10)]:
        spsm[i, j] = spsm[j, i] = 1.0

    def f(ch, sigma, ti, tj):
        if ti < 0 or tj < 0 or ti > 15 or tj > 15 or ch not in (1, 2) or sigma not in (1, -1):
            return 0.0
        return float(fd[ch - 1][1 if sigma == 1 else 0][ti][tj])
    return f, spsm


def two_channel_qs(U, ed, lam):
    """Two-channel Anderson model in the |Q S> basis (SymNo 1)."""
    cg = tg.clebsch
    f, spsm = _two_channel_tables()
    # TwoChQS_SetSingleSite (TwoChQS_SetSingleSite.cpp:5-124): 16 states in 10 blocks
    site = [(-2.0, 0.0, 0.0), (-1.0, 0.5, 0.5), (-1.0, 0.5, -0.5), (0.0, 0.0, 0.0), (0.0, 1.0, -1.0),
            (0.0, 1.0, 0.0), (0.0, 1.0, 1.0), (1.0, 0.5, 0.5), (1.0, 0.5, -0.5), (2.0, 0.0, 0.0)]
    sizes = [1, 2, 2, 3, 1, 1, 1, 2, 2, 1]
    offs = [sum(sizes[:b]) for b in range(len(sizes))]

    def block_of(t):
        for b in range(len(sizes)):
            if offs[b] <= t < offs[b] + sizes[b]:
                return b
        return -1

    def states(b):  # GetBlockLimit; a missing block (-1) is state 0 (NRGarrayClass.cpp:335)
        return range(0, 1) if b < 0 else range(offs[b], offs[b] + sizes[b])

    def dleq(a, b):
        return a < b or abs(a - b) < 1.0e-20

    def full(Si, typep, typ, ich, sigma):
        # FullMatEl of TwoChQS_HN_MatEl (TwoChQS_OpMatRules.cpp:843-957)
        bp, b = block_of(typep), block_of(typ)
        Stp, Sztp = site[bp][1], site[bp][2]
        Stt, Szt = site[b][1], site[b][2]
        Soldp, Sold = Si - Sztp, Si - Szt
        fermi = -1.0 if (_deq(Szt, 0.5) or _deq(Szt, -0.5)) else 1.0
        dS = 0.5 * sigma
        acc = 0.0
        Szold = Sold
        while Szold >= -Sold:
            Szoldp, Sz = Szold - dS, Si - Szold
            Szp = Sz + dS
            sbp = _find(site, (site[bp][0], site[bp][1], Szp))
            sb = _find(site, (site[b][0], site[b][1], Sz))
            if dleq(abs(Szp), Stp) and dleq(abs(Szold), Sold) and dleq(abs(Szoldp), Soldp):
                a0 = cg(Sold, Szold, Stt, Sz, Si, Si)
                a1 = cg(Soldp, Szoldp, Stp, Szp, Si, Si)
                a2 = cg(Soldp, Szoldp, 0.5, dS, Sold, Szold)
                for sp in states(sbp):
                    for s in states(sb):
                        x0, x1 = spsm[s][typ], spsm[sp][typep]
                        a3 = f(ich, sigma, sp, s)
                        acc += a0 * a1 * a2 * a3 * fermi * x0 * x1
            Szold -= 1.0
        return acc

    def hn_coef(S, ti, tj, ch, sg, dr):
        sigma = -1 if sg == 0 else 1
        return full(S, ti, tj, ch + 1, sigma) if dr == 0 else full(S, tj, ti, ch + 1, sigma)

    def op_factor(o, Si, Sj, ti, tj):
        # TwoChQS_fN_MatEl (TwoChQS_OpMatRules.cpp:1205-1352)
        ich = o + 1
        bi, bj = block_of(ti), block_of(tj)
        Scfi, Scfj = Si - site[bi][2], Sj - site[bj][2]
        c0, c1 = cg(Si, Si, 0.5, -0.5, Sj, Sj), cg(Si, Si, 0.5, 0.5, Sj, Sj)
        if not _deq(c0, 0.0):
            sigma, norm = -1, c0
        elif not _deq(c1, 0.0):
            sigma, norm = 1, c1
        else:
            return 0.0
        acc = 0.0
        Szcfj = Scfj
        while Szcfj >= -Scfj:
            Szi, Szj = Si - Szcfj, Sj - Szcfj
            bsi = _find(site, (site[bi][0], site[bi][1], Szi))
            bsj = _find(site, (site[bj][0], site[bj][1], Szj))
            a0 = cg(Scfi, Szcfj, site[bi][1], Szi, Si, Si)
            a1 = cg(Scfj, Szcfj, site[bj][1], Szj, Sj, Sj)
            for si in states(bsi):
                for sj in states(bsj):
                    acc += f(ich, sigma, sj, si) * a0 * a1 * spsm[si][ti] * spsm[sj][tj]
            Szcfj -= 1.0
        return acc / norm

    def op_check(o, qi, qj):
        if o < 2:  # TwoChQS_cd_check (TwoChQS_OpMatRules.cpp:16)
            return _deq(qj[0], qi[0] + 1.0) and (_deq(qj[1], qi[1] + 0.5) or _deq(qj[1], qi[1] - 0.5))
        return qi == qj

    # OneChQS_SetAnderson_Hm1, f_ch1 = f_ch2 = d (Main/Main_SetH0.cpp:1794-1969)
    scale = lam * 0.5 * (1.0 + 1.0 / lam)
    blocks = [(-1.0, 0.0), (0.0, 0.5), (1.0, 0.0)]
    n = [q + 1.0 for q, _ in blocks]
    fop = [(0, 1, np.array([[1.0]])), (1, 2, np.array([[-math.sqrt(2.0)]]))]
    return tg.ModelPlugin(
        total_spin=True, site_qn=site, site_bsize=sizes, hn_form=tg.HN_CHANNEL_SUM, onsite=False,
        hn_coef=hn_coef, op_class=[tg.OP_SITE, tg.OP_SITE] + [tg.OP_IMPURITY_DIAG] * 3,
        op_avg=[0, 0, 1, 1, 1], op_factor=op_factor, op_check=op_check,
        start_qn=blocks, start_bsize=[1, 1, 1],
        start_en=[0.5 * U / scale, (ed + 0.5 * U) / scale, (2.0 * ed + 1.5 * U) / scale],
        start_ops=[fop, fop, _start_ops_diag(3, n), _start_ops_diag(3, [x * x for x in n]),
                   _start_ops_diag(3, [S * (S + 1.0) for _, S in blocks])])


def one_channel_q(U, ed, lam):
    """One-channel Anderson model in the charge-only |Q> basis (SymNo 3): blocks
    carry (Q, 0); the site's Q = 0 block holds |up> and |dn>."""
    site = [(-1.0, 0.0), (0.0, 0.0), (1.0, 0.0)]  # CNRGCodeHandler::SetSingleSite, SymNo 3
    sizes = [1, 2, 1]
    qtype = [-1.0, 0.0, 0.0, 1.0]  # Q of the types |0>, |up>, |dn>, |up dn>

    def hn_coef(S, ti, tj, ch, sg, dr):
        # OneChQ_HN_MatEl (OpMatRules.cpp:1065-1147), OneChQSz_HN_MatEl's arithmetic
        sigma = 1 if sg == 0 else -1
        sign = lambda t: -1.0 if _deq(qtype[t], 0.0) else 1.0  # noqa: E731
        return sign(tj) * _fd(sigma, ti, tj) if dr == 0 else sign(ti) * _fd(sigma, tj, ti)

    def op_factor(o, Si, Sj, ti, tj):  # OneChQ_fN_MatEl (OpMatRules.cpp:1003-1033)
        return _fd(1 if o == 0 else -1, tj, ti)

    def op_check(o, qi, qj):
        if o < 2:  # OneChQ_cd_check (OpMatRules.cpp:92)
            return _deq(qj[0], qi[0] + 1.0)
        return qi == qj

    # OneChQ_SetAnderson_Hm1 (Main/Main_SetH0.cpp:217-352): the Q = 0 block two-fold
    scale = lam * 0.5 * (1.0 + 1.0 / lam)
    blocks = [(-1.0, 0.0), (0.0, 0.0), (1.0, 0.0)]
    return tg.ModelPlugin(
        total_spin=False, site_qn=site, site_bsize=sizes, hn_form=tg.HN_SPIN_SUM, onsite=True,
        hn_coef=hn_coef, op_class=[tg.OP_SITE, tg.OP_SITE, tg.OP_IMPURITY_DIAG, tg.OP_IMPURITY_DIAG],
        op_avg=[0, 0, 1, 1], op_factor=op_factor, op_check=op_check,
        start_qn=blocks, start_bsize=[1, 2, 1],
        start_en=[0.5 * U / scale, (ed + 0.5 * U) / scale, (ed + 0.5 * U) / scale, (2.0 * ed + 1.5 * U) / scale],
        start_ops=[[(0, 1, np.array([[1.0, 0.0]])), (1, 2, np.array([[0.0], [1.0]]))],
                   [(0, 1, np.array([[0.0, 1.0]])), (1, 2, np.array([[-1.0], [0.0]]))],
                   [(0, 0, np.array([[0.0]])), (1, 1, np.array([[0.5, 0.0], [0.0, -0.5]])), (2, 2, np.array([[0.0]]))],
                   [(0, 0, np.array([[0.0]])), (1, 1, np.array([[0.25, 0.0], [0.0, 0.25]])),
                    (2, 2, np.array([[0.0]]))]])
