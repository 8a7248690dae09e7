"""The reference's text interface on CPU: bse.in reading and the abslanc /
absspct / abs.gmres writers, byte for byte against the reference's own output
files (EXAMPLE/Cu_TwoPhoton/Results, fixtures in tests/golden/)."""
import os

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib(lib_built):
    return capi.load(lib_built)


def _read_lanc_text(path):
    with open(path) as f:
        lines = f.read().split("\n")
    n = int(lines[0].split()[0])
    kpref = float(lines[0].split()[1])
    ra, rb = np.zeros(n + 1), np.zeros(n + 1)
    ra[0] = float(lines[1])
    for i in range(1, n + 1):
        a, b = lines[1 + i].split()
        ra[i], rb[i] = float(a), float(b)
    eig = np.array([float(l.split()[2]) for l in lines[n + 2:] if len(l.split()) == 3])
    return n, kpref, ra, rb, eig


def test_abslanc_writer_is_byte_identical(lib, tmp_path):
    src = os.path.join(GOLD, "cu_abslanc_01.txt")
    n, kpref, ra, rb, eig = _read_lanc_text(src)
    out = str(tmp_path / "abslanc")
    capi.write_abslanc(out, n, kpref, ra, rb, eigs=eig)
    assert open(out, "rb").read() == open(src, "rb").read()


def test_absspct_writer_is_byte_identical(lib, tmp_path):
    src = os.path.join(GOLD, "cu_absspct_01_rows.txt")
    lines = open(src).read().split("\n")
    head = lines[0]
    it = int(head.split("iter=")[1].split()[0])
    gam = float(head.split("gam=")[1].split()[0])
    kpref = float(head.split("kpref=")[1].split("vol=")[0])
    vol = float(head.split("vol=")[1])
    rows = np.array([[float(v) for v in l.split()] for l in lines[2:] if l])
    out = str(tmp_path / "absspct")
    capi.write_absspct(out, it, gam, kpref, vol, rows)
    assert open(out, "rb").read() == open(src, "rb").read()


def test_absspct_from_the_coefficients_matches_the_reference_file(lib, tmp_path, oracle_lib):
    """The whole chain on CPU: the reference's Lanczos coefficients -> the
    oracle's write_core -> the writer, against the reference's file: every
    printed value within one unit of its 8th significant digit, and most
    records (59% measured) identical to the last character; the rest differ by
    one in the last digit of a column."""
    O = oracle_lib
    n, kpref, ra, rb, _ = _read_lanc_text(os.path.join(GOLD, "cu_abslanc_01.txt"))
    d = np.load(os.path.join(GOLD, "cu_twophoton_kat.npz"))
    vol = float(d["p1_vol"])
    el, eh, gam = -30.0 * WL.EV2HARTREE, 70.0 * WL.EV2HARTREE, 1.245 * WL.EV2HARTREE
    rows = O.write_core(ra, None, rb, n, kpref, el, eh, 5000, gam, 0.0, 0.0, vol)
    keep = d["p1_rows"]
    out = str(tmp_path / "absspct")
    capi.write_absspct(out, n, gam, kpref, vol, rows[keep])
    got = open(out).read().split("\n")
    ref = open(os.path.join(GOLD, "cu_absspct_01_rows.txt")).read().split("\n")
    assert got[:2] == ref[:2]
    gv = np.array([[float(v) for v in l.split()] for l in got[2:] if l])
    rv = np.array([[float(v) for v in l.split()] for l in ref[2:] if l])
    nz = rv != 0
    unit = 10.0 ** (np.floor(np.log10(np.abs(rv[nz]))) + 1 - 8)  # last printed digit of 0.dddddddd
    assert np.all(np.abs(gv[nz] - rv[nz]) <= 1.01 * unit)
    assert np.array_equal(gv[~nz], rv[~nz])
    same = sum(a == b for a, b in zip(got[2:], ref[2:]))
    assert same >= 0.5 * (len(ref) - 2), same


def test_voigt_header_and_columns(lib, tmp_path):
    rows = np.zeros((3, 9))
    rows[:, :5] = [[-1.5, 1e-3, 2e-3, -3e-3, 4e-3], [0.0, 0.0, 0.0, 0.0, 0.0], [12.25, 1e-120, -1e120, 5.0, 6.0]]
    out = str(tmp_path / "v")
    capi.write_absspct(out, 7, 0.0125, 2.5e-6, 0.0, rows, voigt=True)
    lines = open(out).read().split("\n")
    assert lines[0] == "#   iter=    7   gam= 0.12500000E-01   kpref= 0.25000000E-05"
    assert lines[1] == "     #   Energy           Spect        Spect(0)            SPKK         SPKK(0)"
    assert lines[2] == "-0.15000000E+01  0.10000000E-02  0.20000000E-02 -0.30000000E-02  0.40000000E-02"
    assert lines[3] == " 0.00000000E+00  0.00000000E+00  0.00000000E+00  0.00000000E+00  0.00000000E+00"
    # three-digit exponents drop the letter, as Ew.d does
    assert lines[4] == " 0.12250000E+02  0.10000000-119 -0.10000000+121  0.50000000E+01  0.60000000E+01"


def test_abs_gmres_rows(lib, tmp_path):
    out = str(tmp_path / "abs.gmres")
    capi.write_abs_gmres(out, [0.0, 2.0, -13.75], [1.0, 0.0417904142, -2.5e-12], [0.0205320995, 1e-3, 3.0],
                         [5.21248716e-08, 1.0e-7, 0.5], [43, 33, 9])
    lines = open(out).read().split("\n")
    assert lines[0] == " 0.00000000E+00  1.00000000E+00  2.05320995E-02  5.21248716E-08     43         43"
    assert lines[1] == " 2.00000000E+00  4.17904142E-02  1.00000000E-03  1.00000000E-07     33         76"
    assert lines[2] == "-1.37500000E+01 -2.50000000E-12  3.00000000E+00  5.00000000E-01      9         85"


def test_complex_abslanc_records(lib, tmp_path):
    out = str(tmp_path / "cl")
    ra, ia = np.array([1.0, 2.0]), np.array([0.5, -0.25])
    rb, ib = np.array([0.0, 3.0]), np.array([0.0, 0.125])
    capi.write_abslanc(out, 1, 2.0 ** -20, ra, rb, ia=ia, ib=ib)
    lines = open(out).read().split("\n")
    assert lines[0] == "       1  9.53674316406250000E-07"
    assert lines[1] == "   1.00000000000000000E+00   5.00000000000000000E-01"
    # '(2x,6ES24.17)': a negative value fills its field, no blank before it
    assert lines[2] == ("   2.00000000000000000E+00-2.50000000000000000E-01 3.00000000000000000E+00"
                        " 1.25000000000000000E-01 3.00000000000000000E+00 1.25000000000000000E-01")


def test_read_bse_in_haydock(lib, tmp_path):
    p = tmp_path / "bse.in"
    p.write_text("1\n0.0d0\nhay\n200 5000 -30.0 70.0 1.245d0 0.0\n")
    b = capi.read_bse_in(str(p))
    assert b["style"] == "hay" and b["niter"] == 200 and b["ne"] == 5000
    assert (b["el"], b["eh"], b["gam0"], b["ebase"]) == (-30.0, 70.0, 1.245, 0.0)


def test_read_bse_in_gmres_list_and_loop(lib, tmp_path):
    p = tmp_path / "bse.in"
    p.write_text("1\n0.0\n'inv'\n80, 0.5, 0.5, 1.0D-6\nlist\n3\n-5.0\n0.0\n 7.5d0\n")
    b = capi.read_bse_in(str(p))
    assert b["style"] == "inv" and b["inv_style"] == "list" and b["depth"] == 80
    assert b["convergence"] == 1e-6 and list(b["energies"]) == [-5.0, 0.0, 7.5]
    p.write_text("1\n0.0\ninv\n80 0.5 0.5 1e-6\nloop\n-10.0 10.0 0.1\n")
    b = capi.read_bse_in(str(p))
    # gmres_nsteps = 1 + ceiling((stop - start - step*1e-4) / step)  (OCEAN_gmres.f90:114)
    assert b["nomega"] == 201
    assert np.allclose(b["energies"], -10.0 + 0.1 * np.arange(201))
    p.write_text("1\n0.0\nfoo\n")
    with pytest.raises(capi.OcnError):
        capi.read_bse_in(str(p))


def test_output_filenames(lib):
    assert capi.output_filename("spct", "XAS", "Cu", 1, "1s", 1) == "absspct_Cu.0001_1s_01"
    assert capi.output_filename("lanc", "XAS", "C_", 1, "1s", 2) == "abslanc_C_.0001_1s_02"
    assert capi.output_filename("spct", "XES", "Ti", 12, "2p", 3) == "xesspct_Ti.0012_2p_03"
