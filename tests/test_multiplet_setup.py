"""nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181): the multiplet exchange
matrices from Slater radial integrals, restated on the host in the library
(closed-form Gaunt coefficients) and in the oracle (the reference's quadrature
of threey, CNBSE/zcmsnmult/zf90/newthreey.f90, with newgetylm's harmonics).

  * threey against sympy's Gaunt coefficients (exact, independent), 1e-13
  * library against oracle, every matrix element, 1e-13 relative to the largest
  * the matrix is Hermitian (real symmetric) for symmetric F^k, G^k, and obeys
    the selection rules (spin conserved in each pair, m balance)
  * the Slater-file reader
"""
import itertools
import math

import numpy as np
import pytest

from ocean_gb300 import capi


@pytest.fixture(scope="module")
def lib(lib_built):
    return capi.load(lib_built)


def test_threey_matches_sympy_gaunt(lib, oracle_lib):
    wig = pytest.importorskip("sympy.physics.wigner")
    O = oracle_lib
    rng = np.random.default_rng(0)
    cases = [c for c in itertools.product(range(4), range(7), range(4)) if (sum(c) % 2) == 0]
    for ll, lm, lr in [cases[i] for i in rng.choice(len(cases), 25, replace=False)]:
        for ml in range(-ll, ll + 1):
            for mm in range(-lm, lm + 1):
                mr = ml - mm
                if abs(mr) > lr:
                    continue
                want = (-1) ** (ml % 2) * float(wig.gaunt(ll, lm, lr, -ml, mm, mr))
                assert abs(capi.threey(ll, ml, lm, mm, lr, mr) - want) < 1e-13
                assert abs(O.threey(ll, ml, lm, mm, lr, mr) - want) < 1e-13
                # conj(Y_{lm,mm}) = (-1)^mm Y_{lm,-mm}
                mr2 = ml + mm
                if abs(mr2) <= lr:
                    want2 = (-1) ** ((ml + mm) % 2) * float(wig.gaunt(ll, lm, lr, -ml, -mm, mr2))
                    assert abs(capi.threey(ll, ml, lm, mm, lr, mr2, True) - want2) < 1e-13


def _slater(lc, lv, np_, seed):
    rng = np.random.default_rng(seed)

    def sym():
        a = rng.uniform(0.5, 8.0, size=(np_, np_))
        return 0.5 * (a + a.T)

    fk = {k: sym() for k in range(2, min(2 * lc, 2 * lv) + 1, 2)}
    gk = {k: sym() for k in range(abs(lc - lv), lc + lv + 1, 2)}
    sf = {k: 0.8 for k in fk}
    sg = {k: 0.8 for k in gk}
    return fk, gk, sf, sg


@pytest.mark.parametrize("lc,lv,np_", [(0, 0, 2), (0, 2, 3), (1, 0, 2), (1, 1, 2), (1, 2, 2), (1, 3, 3)])
def test_exchange_matrix_library_matches_oracle(lib, oracle_lib, lc, lv, np_):
    fk, gk, sf, sg = _slater(lc, lv, np_, 10 * lc + lv)
    mhr, mhi = capi.mult_exchange(lc, lv, fk, gk, sf, sg, scfac=0.9)
    ohr, ohi = oracle_lib.nbsemhsetup2(lc, lv, fk, gk, sf, sg, scfac=0.9)
    mham = 4 * (2 * lc + 1) * (2 * lv + 1) * np_
    assert mhr.size == mham * mham
    scale = np.max(np.abs(ohr))
    assert scale > 0.0
    assert np.max(np.abs(mhr - ohr)) < 1e-13 * scale
    assert np.max(np.abs(mhi)) == 0.0 and np.max(np.abs(ohi)) < 1e-13 * scale
    M = mhr.reshape(mham, mham, order="F")  # M[i1, i2] = mhr_l(i1, i2)
    assert np.max(np.abs(M - M.T)) < 1e-13 * scale


def test_exchange_matrix_selection_rules(lib):
    """Elements vanish unless core m minus valence m is the same on both sides
    (m1 + m2 = m3 + m4 of both terms) and the spins match as in the F term
    (core and valence spin each kept) or the G term (each side's core spin
    equal to its valence spin); a 1s core has no F^k (k >= 2) term."""
    lc, lv, np_ = 1, 2, 1
    fk, gk, sf, sg = _slater(lc, lv, np_, 3)
    mhr, _ = capi.mult_exchange(lc, lv, fk, gk)
    nb = 4 * (2 * lc + 1) * (2 * lv + 1) * np_
    M = mhr.reshape(nb, nb, order="F")
    basis = [(cs, cm, vs, vm) for cs in (-1, 1) for cm in range(-lc, lc + 1) for vs in (-1, 1)
             for vm in range(-lv, lv + 1)]
    for i1, (cs1, cm1, vs1, vm1) in enumerate(basis):
        for i2, (cs2, cm2, vs2, vm2) in enumerate(basis):
            f_spin = cs1 == cs2 and vs1 == vs2
            g_spin = cs1 == vs1 and cs2 == vs2
            if cm1 - vm1 != cm2 - vm2 or not (f_spin or g_spin):
                assert M[i1, i2] == 0.0
    fk0, gk0, _, _ = _slater(0, 2, 2, 4)
    assert fk0 == {}
    mhr0, _ = capi.mult_exchange(0, 2, {}, gk0)
    assert np.max(np.abs(mhr0)) > 0.0


def test_read_slater(lib, tmp_path):
    """fk<lc><lv><k><add10>: np*np values in column order, then the scale."""
    f = np.arange(1.0, 10.0).reshape(3, 3)
    vals = list(f.T.reshape(-1)) + [0.8]
    p = tmp_path / "fk132z026n02l01"
    p.write_text("\n".join(f"{v:.6e}" for v in vals[:5]) + "\n" + " ".join(f"{v}" for v in vals[5:]) + "\n")
    got, sc = capi.read_slater(str(p), 3)
    assert np.array_equal(got, f) and sc == 0.8
    p.write_text("1 2 3\n")
    with pytest.raises(capi.OcnError):
        capi.read_slater(str(p), 3)
