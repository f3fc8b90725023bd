"""Thermodynamics with the free-chain subtraction, on the CPU: the oracle's
chain sweep (calcdens = 3) and impurity sweep (calcdens = 2) against the
reference NRG_main's own SuscepChain/EntropyChain and SuscepImp/EntropyImp
files (tests/golden/thermo_*.npz, made by tests/golden/make_thermo_golden.py),
and nrg_write_thermo's file layout against CNRGthermo::SaveNValue's."""
import os
import subprocess

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
NRG_MAIN = os.path.join(ROOT, "oracle", "_ref", "NRG_main")
CASES = [("thermo_1chQS_n14_k150", "1chQS"), ("thermo_1chQSz_n12_k200", "1chQSz"),
         ("thermo_2chQS_chain_n8_k300", "2chQS"), ("thermo_1chQ_n10_k150", "1chQ")]
# CNRGthermo::dImpValue subtracted in the chain run: 2 ln 2 for the |Q> entropy
# (its chain run is the Anderson model with all parameters zeroed), 0 otherwise
D_IMP = {"1chQ": 2.0 * np.log(2.0)}


@pytest.fixture(scope="module")
def lib_built():
    from twochnrg_gb300 import build
    build.build()


def _thermo(sweep):
    return np.array([it.thermo for it in sweep.iters]).reshape(-1, 4)


@pytest.mark.parametrize("name,model", CASES)
def test_oracle_chain_and_impurity_match_reference_files(name, model):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ns, nc, U, G, ed, lam, x = g["config"]
    ch = _thermo(orc.run(model, int(ns), int(nc), lam, 0.0, 0.0, 0.0, chain=True))
    ch[:, 3] -= D_IMP.get(model, 0.0)
    assert ch.shape[0] == 4 * int(ns)
    np.testing.assert_array_equal(ch[:, 1], g["chain_entropy"][:, 0])
    np.testing.assert_allclose(ch[:, 3], g["chain_entropy"][:, 1], rtol=1e-14, atol=0)
    assert not g["chain_entropy"][:, 2].any()  # chain files: third column 0
    if "chain_suscep" in g:
        np.testing.assert_allclose(ch[:, 2], g["chain_suscep"][:, 1], rtol=1e-14, atol=0)
    if "imp_entropy" not in g:
        return
    im = _thermo(orc.run(model, int(ns), int(nc), lam, U, ed, G, x))
    e = g["imp_entropy"]
    np.testing.assert_array_equal(im[:, 1], e[:, 0])
    np.testing.assert_allclose(im[:, 3], e[:, 1], rtol=1e-14, atol=0)
    np.testing.assert_allclose(ch[:, 3], e[:, 2], rtol=1e-14, atol=0)
    np.testing.assert_allclose(im[:, 3] - ch[:, 3], e[:, 3], rtol=1e-12, atol=1e-15)
    if "imp_suscep" in g:
        s = g["imp_suscep"]
        np.testing.assert_allclose(im[:, 2], s[:, 1], rtol=1e-14, atol=0)
        np.testing.assert_allclose(ch[:, 2], s[:, 2], rtol=1e-14, atol=0)
        np.testing.assert_allclose(im[:, 2] - ch[:, 2], s[:, 3], rtol=1e-12, atol=1e-15)


def test_chain_first_site_values():
    """H_0 of the chain: the free site's multiplets at zero energy, T chi =
    sum (2S+1) S(S+1)/3 / sum (2S+1) and S = ln(states)."""
    for model, states, tchi in (("1chQS", 4, 0.125), ("1chQSz", 4, 0.125), ("2chQS", 16, 0.25)):
        # (the |Q> chain starts with the decoupled impurity; not covered here)
        th = orc.run(model, 2, 100, 2.5, 0, 0, 0, chain=True).iters[0].thermo
        np.testing.assert_allclose(th[:, 2], tchi, rtol=1e-15)
        np.testing.assert_allclose(th[:, 3], np.log(states), rtol=1e-15)


def test_write_thermo_layout(lib_built, tmp_path):
    g = np.load(os.path.join(GOLDEN, "thermo_1chQS_n14_k150.npz"))
    s = g["imp_suscep"]
    p = str(tmp_path / "imp.dat")
    tg.write_thermo(p, s[:, 0], s[:, 1], s[:, 2])
    back = np.loadtxt(p)
    np.testing.assert_array_equal(back[:, :3], s[:, :3])
    np.testing.assert_array_equal(back[:, 3], s[:, 1] - s[:, 2])
    line = open(p).readline().split()
    assert len(line) == 4 and all(len(t.split("e")[0]) == 22 for t in line)  # d.dddddddddddddddddddd
    c = str(tmp_path / "chain.dat")
    tg.write_thermo(c, s[:, 0], s[:, 2])
    back = np.loadtxt(c)
    assert not back[:, 2].any()
    np.testing.assert_array_equal(back[:, 3], back[:, 1])
    with pytest.raises(tg.NRGError):
        tg.write_thermo(str(tmp_path / "bad.dat"), s[:3, 0], s[:2, 1])


@pytest.mark.skipif(not os.path.exists(NRG_MAIN), reason="reference binaries not built here")
def test_files_equal_the_reference_files(lib_built, tmp_path):
    """The four files written from the oracle's values equal, byte for byte,
    the ones the reference's NRG_main writes for the same two runs."""
    ref = tmp_path / "ref"
    ref.mkdir()
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    for calcdens in (3, 2):
        (ref / "input_nrg.dat").write_text(f"7\n80\n0.5\n0.02\n-0.25\n2.5\n0\n0\n0\n{calcdens}\n9999999\n")
        subprocess.run([NRG_MAIN, "-m", "Anderson"], cwd=str(ref), check=True, capture_output=True, env=env)
    ch = _thermo(orc.run("1chQS", 7, 80, 2.5, 0, 0, 0, chain=True))
    im = _thermo(orc.run("1chQS", 7, 80, 2.5, 0.5, -0.25, 0.02))
    res = tg.ThermoResult(im[:, 1], im[:, 2], ch[:, 2], im[:, 2] - ch[:, 2], im[:, 3], ch[:, 3],
                          im[:, 3] - ch[:, 3], False, 0.0, 0.0, 0.0, "1chQS")
    ours = tmp_path / "ours"
    ours.mkdir()
    for p in res.save(str(ours)):
        name = os.path.basename(p)
        assert open(p).read() == (ref / name).read_text(), name
