"""Impurity thermodynamics with the free-chain subtraction on the GPU
(nrg_sweep_run_chain, nrg_thermo_run) against the reference NRG_main's own
chain and impurity files (tests/golden/thermo_*.npz, made by
tests/golden/make_thermo_golden.py) and against the oracle.

Tolerance: T chi and S within 1e-10 relative (1e-12 absolute): the block
eigenvalues come from a different eigensolver than LAPACK's and agree to a
few ulp of the largest level, which the Boltzmann sums carry over.  The
temperatures are the same arithmetic in both sweeps and must agree exactly."""
import os

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _close(a, ref):
    np.testing.assert_allclose(a, ref, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name,model", [("thermo_1chQS_n14_k150", "1chQS"),
                                        ("thermo_1chQSz_n12_k200", "1chQSz")])
def test_thermo_matches_reference_files(engine, name, model):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ns, nc, U, G, ed, lam, x = g["config"]
    r = engine.thermo(model, int(ns), int(nc), lam, U, ed, G, x, reuse_chain=False)
    assert not r.chain_reused and len(r.temp) == 4 * int(ns)
    s, e = g["imp_suscep"], g["imp_entropy"]
    np.testing.assert_array_equal(r.temp, s[:, 0])
    _close(r.suscep, s[:, 1]); _close(r.suscep_chain, s[:, 2]); _close(r.suscep_imp, s[:, 3])
    _close(r.entropy, e[:, 1]); _close(r.entropy_chain, e[:, 2]); _close(r.entropy_imp, e[:, 3])
    _close(r.suscep_chain, g["chain_suscep"][:, 1])
    _close(r.entropy_chain, g["chain_entropy"][:, 1])
    # the impurity sweep stays readable on the context
    it = engine.fetch().iters
    assert len(it) == int(ns)
    _close(np.array([i.thermo[:, 2] for i in it]).ravel(), s[:, 1])


def test_two_channel_chain_and_impurity(engine):
    g = np.load(os.path.join(GOLDEN, "thermo_2chQS_chain_n8_k300.npz"))
    ns, nc, U, G, ed, lam, x = g["config"]
    ch = engine.sweep_chain("2chQS", int(ns), int(nc), lam)
    th = np.array([i.thermo for i in ch.iters]).reshape(-1, 4)
    np.testing.assert_array_equal(th[:, 1], g["chain_suscep"][:, 0])
    _close(th[:, 2], g["chain_suscep"][:, 1])
    _close(th[:, 3], g["chain_entropy"][:, 1])
    h0 = ch.iters[0]  # the two-channel first site: 10 multiplets in 6 blocks at zero energy
    np.testing.assert_array_equal(h0.qn, [[-2, 0], [-1, 0.5], [0, 0], [0, 1], [1, 0.5], [2, 0]])
    np.testing.assert_array_equal(h0.bsize, [1, 2, 3, 1, 2, 1])
    assert not h0.en.any()
    # impurity minus chain against the oracle (no two-channel Anderson in NRG_main)
    r = engine.thermo("2chQS", 6, 200, 2.5, 0.3, -0.15, 0.01, 0.01)
    o_ch = np.array([i.thermo for i in orc.run("2chQS", 6, 200, 2.5, 0, 0, 0, chain=True).iters]).reshape(-1, 4)
    o_im = np.array([i.thermo for i in orc.run("2chQS", 6, 200, 2.5, 0.3, -0.15, 0.01, 0.01).iters]).reshape(-1, 4)
    np.testing.assert_array_equal(r.temp, o_im[:, 1])
    _close(r.suscep_imp, o_im[:, 2] - o_ch[:, 2])
    _close(r.entropy_imp, o_im[:, 3] - o_ch[:, 3])


def test_chain_reused_for_the_same_chain(engine):
    a = engine.thermo("1chQS", 8, 100, 2.5, 0.5, -0.25, 0.02, reuse_chain=False)
    b = engine.thermo("1chQS", 8, 100, 2.5, 0.3, -0.15, 0.01)
    assert b.chain_reused
    np.testing.assert_array_equal(a.suscep_chain, b.suscep_chain)
    np.testing.assert_array_equal(b.suscep_imp, b.suscep - b.suscep_chain)
    o = np.array([i.thermo for i in orc.run("1chQS", 8, 100, 2.5, 0.3, -0.15, 0.01).iters]).reshape(-1, 4)
    _close(b.suscep, o[:, 2])
    c = engine.thermo("1chQS", 8, 120, 2.5, 0.3, -0.15, 0.01)  # other Ncutoff: a new chain
    assert not c.chain_reused
    d = engine.thermo("1chQS", 8, 120, 2.5, 0.3, -0.15, 0.01, reuse_chain=False)
    assert not d.chain_reused
    np.testing.assert_array_equal(c.suscep_chain, d.suscep_chain)


def test_gpu_thermo_files(engine, tmp_path):
    g = np.load(os.path.join(GOLDEN, "thermo_1chQS_n14_k150.npz"))
    ns, nc, U, G, ed, lam, x = g["config"]
    r = engine.thermo("1chQS", int(ns), int(nc), lam, U, ed, G)
    names = sorted(os.path.basename(p) for p in r.save(str(tmp_path)))
    assert names == ["EntropyChain1Ch_QS_zEQ1.dat", "EntropyImp1ChQS_Anderson_zEQ1.dat",
                     "SuscepChain1Ch_QS_zEQ1.dat", "SuscepImp1ChQS_Anderson_zEQ1.dat"]
    for stem, key in (("SuscepImp1ChQS_Anderson", "imp_suscep"), ("EntropyImp1ChQS_Anderson", "imp_entropy"),
                      ("SuscepChain1Ch_QS", "chain_suscep"), ("EntropyChain1Ch_QS", "chain_entropy")):
        _close(np.loadtxt(str(tmp_path / f"{stem}_zEQ1.dat")), g[key])


def test_charge_only_symmetry_entropy(engine, tmp_path):
    """|Q> basis: entropy only (the reference's Sqnumber -1 takes no T chi);
    its chain run is the Anderson model with every parameter zeroed, minus
    the decoupled impurity's ln 4."""
    g = np.load(os.path.join(GOLDEN, "thermo_1chQ_n10_k150.npz"))
    ns, nc, U, G, ed, lam, x = g["config"]
    r = engine.thermo("1chQ", int(ns), int(nc), lam, U, ed, G)
    assert not r.suscep.any() and not r.suscep_chain.any()
    e = g["imp_entropy"]
    np.testing.assert_array_equal(r.temp, e[:, 0])
    _close(r.entropy, e[:, 1]); _close(r.entropy_chain, e[:, 2]); _close(r.entropy_imp, e[:, 3])
    _close(r.entropy_chain, g["chain_entropy"][:, 1])
    names = sorted(os.path.basename(p) for p in r.save(str(tmp_path)))
    assert names == ["EntropyChain1Ch_Q.dat", "EntropyImp1Ch_Anderson_Q.dat"]
    _close(np.loadtxt(str(tmp_path / "EntropyImp1Ch_Anderson_Q.dat")), e)
