"""The reference's .bin snapshot layout (nrg_write_dm_shell, host code only):
a written shell reads back field by field; where the reference binaries are
built here (oracle/build_ref.sh), the files equal the ones the reference's own
NRG_main saves for the same sweep, and the reference's DM_NRG run on them gives
the reference's spectral function."""
import os
import subprocess

import numpy as np
import pytest

import twochnrg_gb300 as tg
from oracle import oracle as orc
from oracle.binfiles import read_bin

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NRG_MAIN = os.path.join(ROOT, "oracle", "_ref", "NRG_main")
DM_NRG = os.path.join(ROOT, "oracle", "_ref", "DM_NRG")
NAME = "1chQSAnderson"


@pytest.fixture(scope="module")
def lib_built():
    from twochnrg_gb300 import build
    build.build()


def _write(shells, d):
    for N, s in enumerate(shells):
        tg.write_dm_shell(str(d), NAME, N, s)


def test_written_shell_reads_back(lib_built, tmp_path):
    shells = orc.dm_shells(5, 40, 2.5, 0.5, -0.25, 0.02)
    _write(shells, tmp_path)
    for N, s in enumerate(shells):
        ab = read_bin(str(tmp_path / f"Abasis_{NAME}_N{N}.bin"), "basis")
        ac = read_bin(str(tmp_path / f"Acut_{NAME}_N{N}.bin"), "basis")
        m = read_bin(str(tmp_path / f"Mat0_{NAME}_N{N}.bin"), "matrix")
        for x in (ab, ac, m):
            assert x["trailing_bytes"] == 0 and x["Nshell"] == N and x["NQNumbers"] == 2
            assert x["totalS"] == 1 and list(x["Sqnumbers"]) == [1]
        np.testing.assert_array_equal(ab["QNumbers"], s["basis_qn"])
        np.testing.assert_array_equal(ab["BlockBegEnd"], s["basis_bbe"])
        np.testing.assert_array_equal(ab["iType"], s["basis_itype"])
        np.testing.assert_array_equal(ab["StCameFrom"], s["basis_stcf"])
        np.testing.assert_array_equal(ab["dEn"], s["basis_en"])
        np.testing.assert_array_equal(ac["dEn"], s["en"])
        np.testing.assert_array_equal(ac["dEigVec"], s["evec"])
        np.testing.assert_array_equal(ac["Kept"], s["kept"])
        np.testing.assert_array_equal(ac["BlockBegEndBC"], s["bbe"])
        np.testing.assert_array_equal(ac["StCameFrom"], np.arange(len(s["en"])))
        np.testing.assert_array_equal(m["MatEl"], s["cd_el"])
        np.testing.assert_array_equal(m["MatBlockMap"], s["cd_map"])
        np.testing.assert_array_equal(m["MatBlockBegEnd"], s["cd_mbe"])
        assert m["NeedOld"] == 1 and m["UpperTriangular"] == 0 and m["WignerEckartL"] == 0.5


def _reference_sweep(d):
    with open(os.path.join(d, "input_nrg.dat"), "w") as f:
        f.write("10\n60\n0.5\n0.02\n-0.25\n2.5\n0\n0\n1\n1\n9999999\n")
    subprocess.run([NRG_MAIN, "-m", "Anderson"], cwd=d, check=True, capture_output=True,
                   env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))


@pytest.mark.skipif(not os.path.exists(NRG_MAIN), reason="reference binaries not built here")
def test_files_equal_the_reference_snapshots(lib_built, tmp_path):
    ref = tmp_path / "ref"
    ours = tmp_path / "ours"
    ref.mkdir()
    ours.mkdir()
    _reference_sweep(str(ref))
    _write(orc.dm_shells(10, 60, 2.5, 0.5, -0.25, 0.02), ours)
    for N in range(10):
        for what, kind in (("Abasis", "basis"), ("Acut", "basis"), ("Mat0", "matrix")):
            r = read_bin(str(ref / f"{what}_{NAME}_N{N}.bin"), kind)
            o = read_bin(str(ours / f"{what}_{NAME}_N{N}.bin"), kind)
            for k, v in r.items():
                if k == "NQNumbers_stcf":  # never initialised by the reference
                    continue
                if isinstance(v, np.ndarray) and v.dtype.kind == "f":
                    np.testing.assert_allclose(o[k], v, rtol=1e-13, atol=1e-14, err_msg=f"{what} N{N} {k}")
                elif isinstance(v, np.ndarray):
                    np.testing.assert_array_equal(o[k], v, err_msg=f"{what} N{N} {k}")
                else:
                    assert o[k] == v, f"{what} N{N} {k}"


@pytest.mark.skipif(not os.path.exists(DM_NRG), reason="reference binaries not built here")
def test_reference_dm_nrg_reads_the_files(lib_built, tmp_path):
    g = np.load(os.path.join(ROOT, "tests", "golden", "dm_1chQS_n10_k60_T0.npz"))
    _write(orc.dm_shells(10, 60, 2.5, 0.5, -0.25, 0.02), tmp_path)
    tg.write_code_pars(str(tmp_path), 2.5, 10, NAME)
    subprocess.run([DM_NRG, "-F", "-e", "0.6", "-n", "4"], cwd=str(tmp_path), check=True, capture_output=True,
                   env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
    data = np.loadtxt(str(tmp_path / "rho_0_0_OmegaRhow.dat"))
    np.testing.assert_allclose(data[:, 0], g["omega"], rtol=1e-14)
    np.testing.assert_allclose(data[:, 1], g["A"], rtol=1e-12, atol=1e-300)
