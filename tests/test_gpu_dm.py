"""DM-NRG on the GPU (nrg_sweep_run_dm -> nrg_dm_backprop -> nrg_lehmann)
against the reference DM_NRG's own A(omega) (tests/golden/dm_*.npz, made by
tests/golden/make_dm_golden.py) and against the oracle on other temperatures
and frequency grids; the two-channel shells against the one-channel model
with Gamma1 + Gamma2 (an exact identity with every state kept) and against
the oracle's restatement.

Tolerance: spectra within 1e-8 relative (the block eigenvectors come from a
different eigensolver than LAPACK's, so agreement is at the eigenvector
round-off, amplified by near-degenerate levels), with an absolute floor of
1e-10 of the spectrum's maximum for the exponentially small tails."""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["dm_1chQS_n10_k60_T0", "dm_1chQS_n10_k60_M6", "dm_1chQS_n16_k150_M12"]


def _close(A, ref):
    np.testing.assert_allclose(A, ref, rtol=1e-8, atol=1e-10 * float(np.max(np.abs(ref))))


@pytest.mark.parametrize("name", CASES)
def test_dm_spectral_matches_reference(engine, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    ns, nc, U, G, ed, lam, b, nw, mtemp = g["config"]
    nsh = engine.sweep_dm(int(ns), int(nc), lam, U, ed, G)
    assert nsh == int(ns)
    prm = engine.dm_params(mtemp=int(mtemp), bbroad=b, nw=int(nw))
    tr = engine.dm_backprop(prm)
    assert np.all(np.isfinite(tr))
    om, A = engine.lehmann(prm)
    np.testing.assert_allclose(om, g["omega"], rtol=1e-14)
    _close(A, g["A"])


def test_dm_against_oracle_on_a_log_grid(engine):
    lam, ns = 2.5, 12
    temp = 0.7 * lam ** (-(8 - 1) / 2.0) / 0.727     # T = D_8 / betabar
    om = np.concatenate([-np.logspace(0, -5, 60), np.logspace(-5, 0, 60)])
    o_om, o_A, o_tr = orc.dm_spectral(ns, 80, lam, 0.4, -0.2, 0.015, temp, 0.6, omegas=om)
    engine.sweep_dm(ns, 80, lam, 0.4, -0.2, 0.015)
    prm = engine.dm_params(temp=temp, bbroad=0.6)
    tr = engine.dm_backprop(prm)
    np.testing.assert_allclose(tr, o_tr, rtol=1e-10)
    g_om, A = engine.lehmann(prm, omegas=om)
    np.testing.assert_array_equal(g_om, om)
    _close(A, o_A)
    t = engine.timing()
    assert t["lehmann_pairs"] > 0 and t["lehmann_evals"] > 0


def test_dm_call_order_and_model_errors(engine, tmp_path):
    cfg = tg.SweepConfig(tg.MODEL_1CH_QSZ, 3, 40, 2.5, 0.3, -0.15, 0.01, 0.0, 0.0, 0)
    import ctypes
    st = engine.L.nrg_sweep_run_dm(engine.h, ctypes.byref(cfg))
    assert st == 1  # DM shells exist for the |Q S> models only
    engine.sweep_dm(3, 40, 2.5, 0.3, -0.15, 0.01, model="2chQS", gamma2=0.01)
    with pytest.raises(tg.NRGError):  # the reference's DM_NRG reads one-channel shells only
        engine.dm_save_bin(str(tmp_path), "2chQSAnderson")
    engine.sweep_dm(6, 40, 2.5, 0.5, -0.25, 0.02)
    prm = engine.dm_params(nw=2)
    with pytest.raises(tg.NRGError) as e:  # Lehmann sums before the backward sweep
        engine.lehmann(prm)
    assert e.value.status == 8


def test_dm_shells_saved_in_reference_layout(engine, tmp_path):
    """nrg_dm_save_bin: the GPU sweep's shells as the reference's .bin files.
    Integers (blocks, iType, StCameFrom, Kept, MatBlockMap) equal the oracle's
    shells exactly; energies within 1e-12.  From shell 1 on, the product basis
    carries each implementation's own eigenvector signs (H_N agrees up to
    that gauge), so eigenvectors are checked by orthonormality (and against
    the oracle's in shell 0), and c_d by the Frobenius norm of each block
    pair, which the gauge leaves unchanged."""
    from oracle.binfiles import read_bin
    ns, nc = 8, 60
    engine.sweep_dm(ns, nc, 2.5, 0.5, -0.25, 0.02)
    engine.dm_save_bin(str(tmp_path), "1chQSAnderson")
    ref = orc.dm_shells(ns, nc, 2.5, 0.5, -0.25, 0.02)
    pars = open(tmp_path / "ThisCodePars.dat").read().split()
    assert float(pars[0]) == 2.5 and int(pars[2]) == ns and pars[4] == "1chQSAnderson"
    for N, s in enumerate(ref):
        ab = read_bin(str(tmp_path / f"Abasis_1chQSAnderson_N{N}.bin"), "basis")
        ac = read_bin(str(tmp_path / f"Acut_1chQSAnderson_N{N}.bin"), "basis")
        m = read_bin(str(tmp_path / f"Mat0_1chQSAnderson_N{N}.bin"), "matrix")
        np.testing.assert_array_equal(ab["QNumbers"], s["basis_qn"])
        np.testing.assert_array_equal(ab["BlockBegEnd"], s["basis_bbe"])
        np.testing.assert_array_equal(ab["iType"], s["basis_itype"])
        np.testing.assert_array_equal(ab["StCameFrom"], s["basis_stcf"])
        np.testing.assert_allclose(ab["dEn"], s["basis_en"], rtol=0, atol=1e-12 * max(1, np.abs(s["basis_en"]).max()))
        np.testing.assert_array_equal(ac["BlockBegEnd"], s["bbe"])
        np.testing.assert_array_equal(ac["Kept"], s["kept"])
        np.testing.assert_allclose(ac["dEn"], s["en"], rtol=0, atol=1e-12 * max(1, np.abs(s["en"]).max()))
        np.testing.assert_array_equal(m["MatBlockMap"], s["cd_map"])
        np.testing.assert_array_equal(m["MatBlockBegEnd"], s["cd_mbe"])
        bbe = s["bbe"]
        off = 0
        for b in range(len(bbe) // 2):
            n = int(bbe[2 * b + 1] - bbe[2 * b] + 1)
            Z = ac["dEigVec"][off:off + n * n].reshape(n, n)
            Zr = s["evec"][off:off + n * n].reshape(n, n)
            off += n * n
            assert np.abs(Z @ Z.T - np.eye(n)).max() < 1e-11
            if N == 0:
                np.testing.assert_allclose(np.abs(Z @ Zr.T), np.eye(n), atol=1e-9)
        for k in range(len(s["cd_map"]) // 2):
            lo, hi = s["cd_mbe"][2 * k], s["cd_mbe"][2 * k + 1] + 1
            a, r = m["MatEl"][lo:hi], s["cd_el"][lo:hi]
            assert abs(np.linalg.norm(a) - np.linalg.norm(r)) < 1e-10 * max(1.0, np.linalg.norm(r))


def test_two_channel_all_kept_is_one_channel_with_summed_gamma(engine):
    """The two-channel impurity couples to the even combination of the two
    identical chains only.  With every state kept (4 x 16^3 states in the
    last shell) A(omega) of 2chQS(Gamma1, Gamma2) equals 1chQS(Gamma1 +
    Gamma2) to round-off: the two-channel c_d rule, the 16-state site algebra
    and the last shell's Lehmann sum on the GPU against the one-channel path
    that is pinned to the reference DM_NRG."""
    om = np.concatenate([-np.logspace(0, -4, 40), np.logspace(-4, 0, 40)])
    T = 3e-3
    engine.sweep_dm(3, 100000, 2.5, 0.3, -0.15, 0.01, model="2chQS", gamma2=0.012)
    prm = engine.dm_params(temp=T, bbroad=0.6)
    assert prm.site_dim == 16.0
    tr2 = engine.dm_backprop(prm)
    _, A2 = engine.lehmann(prm, omegas=om)
    engine.sweep_dm(3, 100000, 2.5, 0.3, -0.15, 0.022)
    prm1 = engine.dm_params(temp=T, bbroad=0.6)
    tr1 = engine.dm_backprop(prm1)
    _, A1 = engine.lehmann(prm1, omegas=om)
    assert np.abs(A2 - A1).max() < 1e-10 * np.abs(A1).max()
    np.testing.assert_allclose(tr2, tr1, rtol=1e-10)


def test_two_channel_dm_against_oracle(engine):
    """Truncated two-channel shells (80 kept multiplets): the backward sweep
    through the 16-state site and the FDM sum against the oracle's
    restatement, at a temperature inside the chain."""
    lam, ns, nc = 2.5, 6, 80
    temp = 0.7 * lam ** (-(4 - 1) / 2.0) / 0.727
    om = np.concatenate([-np.logspace(0, -4, 30), np.logspace(-4, 0, 30)])
    o_om, o_A, o_tr = orc.dm_spectral(ns, nc, lam, 0.3, -0.15, 0.01, temp, 0.6, omegas=om, model="2chQS",
                                      gamma2=0.012, nthreads=min(8, os.cpu_count() or 1))
    engine.sweep_dm(ns, nc, lam, 0.3, -0.15, 0.01, model="2chQS", gamma2=0.012)
    prm = engine.dm_params(temp=temp, bbroad=0.6)
    tr = engine.dm_backprop(prm)
    np.testing.assert_allclose(tr, o_tr, rtol=1e-10)
    _, A = engine.lehmann(prm, omegas=om)
    _close(A, o_A)


def test_dm_on_an_uneven_grid(engine):
    """Frequencies not evenly spaced in ln|omega|: every tile takes the
    direct exponentials instead of the recurrence along the tile."""
    lam, ns = 2.5, 10
    temp = 0.7 * lam ** (-(6 - 1) / 2.0) / 0.727
    rng = np.random.default_rng(7)
    x = np.sort(10.0 ** rng.uniform(-5, 0, 70))
    om = np.concatenate([-x[::-1], x])
    _, o_A, _ = orc.dm_spectral(ns, 60, lam, 0.4, -0.2, 0.015, temp, 0.6, omegas=om)
    engine.sweep_dm(ns, 60, lam, 0.4, -0.2, 0.015)
    prm = engine.dm_params(temp=temp, bbroad=0.6)
    engine.dm_backprop(prm)
    _, A = engine.lehmann(prm, omegas=om)
    _close(A, o_A)


def _write_oracle_shells(d, nsites, ncut, lam, U, ed, G, name="1chQSAnderson"):
    shells = orc.dm_shells(nsites, ncut, lam, U, ed, G)
    for N, s in enumerate(shells):
        tg.write_dm_shell(str(d), name, N, s)
    tg.write_code_pars(str(d), lam, nsites, name)


def test_dm_from_snapshot_files(tmp_path):
    """The backward sweep and spectral function started from .bin snapshots in
    the reference's layout (as the reference's NRG_main writes them: the
    writer's files equal NRG_main's byte for byte, tests/test_binfile.py)
    instead of a GPU forward sweep, against the oracle's DM-NRG on the same
    shells."""
    lam, ns, nc, U, ed, G = 2.5, 12, 80, 0.4, -0.2, 0.015
    _write_oracle_shells(tmp_path, ns, nc, lam, U, ed, G)
    temp = 0.7 * lam ** (-(8 - 1) / 2.0) / 0.727
    om = np.concatenate([-np.logspace(0, -5, 60), np.logspace(-5, 0, 60)])
    _, o_A, o_tr = orc.dm_spectral(ns, nc, lam, U, ed, G, temp, 0.6, omegas=om)
    e = tg.Engine(0)
    try:
        assert e.dm_load_bin(str(tmp_path), "1chQSAnderson") == ns
        prm = e.dm_params(temp=temp, bbroad=0.6)
        np.testing.assert_allclose(e.dm_backprop(prm), o_tr, rtol=1e-10)
        _, A = e.lehmann(prm, omegas=om)
        _close(A, o_A)
    finally:
        e.close()


def test_dm_snapshot_round_trip(engine, tmp_path):
    """GPU forward sweep -> dm_save_bin -> dm_load_bin on a fresh context:
    the same spectral function."""
    engine.sweep_dm(10, 60, 2.5, 0.5, -0.25, 0.02)
    prm = engine.dm_params(mtemp=6, bbroad=0.6, nw=4)
    engine.dm_backprop(prm)
    om, A = engine.lehmann(prm)
    engine.dm_save_bin(str(tmp_path), "rt")
    e = tg.Engine(0)
    try:
        assert e.dm_load_bin(str(tmp_path), "rt") == 10
        p2 = e.dm_params(mtemp=6, bbroad=0.6, nw=4)
        e.dm_backprop(p2)
        om2, A2 = e.lehmann(p2)
        np.testing.assert_array_equal(om2, om)
        np.testing.assert_allclose(A2, A, rtol=1e-12, atol=1e-14 * float(np.abs(A).max()))
    finally:
        e.close()


def test_dm_snapshot_mismatch_is_rejected(engine, tmp_path):
    """A shell whose basis is not what BuildBasis makes of the previous
    shell's kept states (here: shell 2 of another kept count) is refused."""
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir(); b.mkdir()
    _write_oracle_shells(a, 4, 40, 2.5, 0.5, -0.25, 0.02)
    _write_oracle_shells(b, 4, 20, 2.5, 0.5, -0.25, 0.02)
    import shutil
    for k in ("Abasis", "Acut", "Mat0"):
        shutil.copy(b / f"{k}_1chQSAnderson_N2.bin", a / f"{k}_1chQSAnderson_N2.bin")
    with pytest.raises(tg.NRGError) as ei:
        engine.dm_load_bin(str(a), "1chQSAnderson")
    assert ei.value.status == 6  # NRG_ERR_SYNC
    with pytest.raises(tg.NRGError):
        engine.dm_load_bin(str(tmp_path / "missing"), "1chQSAnderson")
