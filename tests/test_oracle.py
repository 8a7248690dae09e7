"""CPU tests of the oracle: pinned against the reference's golden vectors where
they exist (continued fraction, tridiagonal eigenvalues) and against
structural properties and numpy/scipy elsewhere."""
import os

import numpy as np
import pytest

from ocean_gb300 import workloads as WL

GOLD = os.path.join(os.path.dirname(__file__), "golden", "cu_twophoton_kat.npz")


@pytest.fixture(scope="module")
def kat():
    return np.load(GOLD)


@pytest.mark.parametrize("photon", range(1, 8))
def test_write_core_matches_reference_golden(oracle_lib, kat, photon):
    """write_core (OCEAN_haydock.f90:1801-1894) reproduces absspct_Cu.0001_1s_0P
    from abslanc_Cu.0001_1s_0P to the 8 significant digits the file holds."""
    O = oracle_lib
    p = f"p{photon}"
    n = int(kat[p + "_n"])
    ne = int(kat["ne"])
    out = O.write_core(kat[p + "_real_a"], None, kat[p + "_real_b"], n, float(kat[p + "_kpref"]),
                       float(kat["el_ev"]) * WL.EV2HARTREE, float(kat["eh_ev"]) * WL.EV2HARTREE, ne,
                       float(kat["gam0_ev"]) * WL.EV2HARTREE, 0.0, 0.0, float(kat[p + "_vol"]))
    assert out.shape[0] == int(kat[p + "_nrows"])
    got = out[kat[p + "_rows"]]
    ref = kat[p + "_spct"]
    # E15.8 keeps 8 significant digits: half a unit in the last place is <= 5e-8
    nz = ref != 0.0
    rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.max() < 6e-8, rel.max()
    assert np.abs(got[~nz]).max(initial=0.0) < 1e-12  # the 0 eV row: energy and sigma vanish


def test_single_precision_cmplx_is_needed(oracle_lib, kat):
    """The golden spectra carry the binary32 rounding of Fortran cmplx() without
    KIND; an all-FP64 recurrence misses them by far more than print precision."""
    ra, rb = kat["p1_real_a"], kat["p1_real_b"]
    n = int(kat["p1_n"])
    kp = float(kat["p1_kpref"])
    gam = float(kat["gam0_ev"]) * WL.EV2HARTREE
    rows = kat["p1_rows"][::7]
    ref = kat["p1_spct"][::7, 2]
    worst = 0.0
    for r, s in zip(rows, ref):
        e = -30.0 * WL.EV2HARTREE + 100.0 * WL.EV2HARTREE * (2 * r) / 10000.0
        ct = complex(e - ra[n - 1], gam)
        disc = np.sqrt(ct * ct - 4 * rb[n] ** 2)
        d = (ct + disc) / 2 if disc.imag > 0 else (ct - disc) / 2
        for j in range(n - 1, -1, -1):
            d = complex(e - ra[j], gam) - rb[j + 1] ** 2 / d
        val = kp * abs(d.imag) / abs(d) ** 2
        worst = max(worst, abs(val - s) / abs(s))
    assert worst > 1.5e-7


@pytest.mark.parametrize("photon", [1, 4, 7])
def test_redtrid_matches_reference_golden(oracle_lib, kat, photon):
    p = f"p{photon}"
    n = int(kat[p + "_n"])
    rc, w = oracle_lib.redtrid(n, kat[p + "_real_a"], kat[p + "_real_b"])
    assert rc == 0
    assert np.abs(w - kat[p + "_eig"]).max() < 6e-11  # printed with 10 decimals


@pytest.mark.parametrize("kmesh", [(2, 2, 2), (4, 4, 4), (3, 5, 2), (6, 1, 4), (5, 5, 5)])
@pytest.mark.parametrize("sign", [1, -1])
def test_fft_matches_numpy(oracle_lib, kmesh, sign):
    rng = np.random.default_rng(1)
    nk = int(np.prod(kmesh))
    x = rng.standard_normal(nk) + 1j * rng.standard_normal(nk)
    r, i = oracle_lib.fft3d(kmesh, x.real, x.imag, sign)
    a = x.reshape(kmesh)  # k3 fastest = C order of (k1, k2, k3)
    ref = (np.fft.ifftn(a) * nk) if sign > 0 else np.fft.fftn(a)
    assert np.allclose(r + 1j * i, ref.reshape(-1), rtol=0, atol=1e-12 * nk)


@pytest.mark.parametrize("n", [1, 2, 5, 17, 40])
def test_zhptrf_zhptrs_match_scipy(oracle_lib, n):
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h = a + a.conj().T  # Hermitian indefinite: exercises 2x2 pivots
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ap = np.array([h[i, j] for j in range(n) for i in range(j + 1)])
    info, ipiv, x = oracle_lib.zhptrf_solve(ap, b)
    assert info == 0
    assert np.allclose(h @ x, b, atol=1e-9 * np.abs(b).max() * max(1, np.linalg.cond(h)) ** 0.5)
    lu, piv, info2 = sl.lapack.zhetrf(h, lower=0)
    assert info2 == 0
    if n < 32:  # LAPACK's unblocked path: identical pivot choices
        assert list(ipiv) == list(piv)


@pytest.fixture(scope="module")
def tiny_problem(oracle_lib):
    w = WL.make("tiny", seed=1)
    return w, oracle_lib.OracleProblem(w)


def _dense(P, n):
    H = np.zeros((n, n), complex)
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        r, i = P.xact(e, np.zeros(n))
        H[:, j] = r + 1j * i
    return H


def test_action_is_hermitian(tiny_problem):
    w, P = tiny_problem
    H = _dense(P, w.npsi)
    assert np.abs(H - H.conj().T).max() < 1e-14 * np.abs(H).max()


def test_action_terms_recombine(tiny_problem):
    """E o psi + LR part: hflag off for LR leaves exactly E o psi."""
    w, P = tiny_problem
    r, i = P.xact(w.psi_r, w.psi_i, hflag=(0, 1, 1, 1, 1, 1))
    assert np.allclose(r + 1j * i, w.er * (w.psi_r + 1j * w.psi_i), atol=1e-15)


def test_multiplet_action_hermitian(oracle_lib):
    w = WL.make("c3small", seed=2)
    P = oracle_lib.OracleProblem(w)
    H = _dense(P, w.npsi)
    assert np.abs(H - H.conj().T).max() < 1e-13 * np.abs(H).max()
    # the multiplet + spin-orbit terms are active: switching them off changes H
    r, i = P.xact(w.psi_r, w.psi_i, hflag=(1, 1, 1, 1, 0, 0))
    r2, i2 = P.xact(w.psi_r, w.psi_i)
    assert np.abs((r - r2) + 1j * (i - i2)).max() > 1e-6


def test_lanczos_ritz_values_bracket_spectrum(tiny_problem):
    w, P = tiny_problem
    H = _dense(P, w.npsi)
    ev = np.linalg.eigvalsh(0.5 * (H + H.conj().T))
    rc, ra, ia, rb, done = P.haydock(w.npsi - 1)
    assert rc == 0 and done == w.npsi - 1
    psi = w.psi_r + 1j * w.psi_i
    assert abs(ra[0] - np.vdot(psi, H @ psi).real) < 1e-14
    T = np.diag(ra[:done]) + np.diag(rb[1:done], 1) + np.diag(rb[1:done], -1)
    rit = np.linalg.eigvalsh(T)
    assert rit[0] >= ev[0] - 1e-10 and rit[-1] <= ev[-1] + 1e-10
    assert abs(rit[0] - ev[0]) < 1e-3 and abs(rit[-1] - ev[-1]) < 1e-3


def test_haydock_nan_sets_ierr(tiny_problem):
    w, P = tiny_problem
    pr = w.psi_r.copy()
    pr[3] = np.nan
    rc, ra, ia, rb, done = P.haydock(5, pr, w.psi_i)
    assert rc == -1 and done == 1


def test_gmres_matches_direct_solve(tiny_problem):
    w, P = tiny_problem
    H = _dense(P, w.npsi)
    E = np.array([5.0, 5.1, 5.2, 9.0])
    rc, ore, oim, rel, its, tot = P.gmres(E, depth=20, ffff=1e-14)
    assert rc == 0
    rhs = w.allow * (w.psi_r + 1j * w.psi_i)
    for k, e in enumerate(E):
        z = e * WL.EV2HARTREE + 1j * w.gam0
        x = np.linalg.solve(z * np.eye(w.npsi) - H, rhs)
        ex = -np.vdot(rhs, x).imag * w.kpref
        assert abs(oim[k] - ex) < 1e-5 * abs(ex)
        assert its[k] >= 0


def test_pnorm_kpref():
    w = WL.make("tiny", seed=3)
    val = 1.0  # psi already normalised
    assert abs(np.sum(w.psi_r ** 2 + w.psi_i ** 2) - 1.0) < 1e-12
    assert w.kpref > 0 and val == 1.0


def test_spin_polarised_action_hermitian(oracle_lib):
    """nspn = 2 (valence spin alpha mod 2 picks the Bloch functions and the
    projector coefficients): the dense action stays Hermitian and differs from
    the action built from the spin-up functions alone."""
    w = WL.make("c3small", seed=5, nspn=2)
    P = oracle_lib.OracleProblem(w)
    H = _dense(P, w.npsi)
    assert np.abs(H - H.conj().T).max() < 1e-13 * np.abs(H).max()
    n = w.nb * w.nk * w.nx
    w1 = WL.make("c3small", seed=5, nspn=2)
    w1.ur[n:], w1.ui[n:] = w1.ur[:n], w1.ui[:n]
    r, i = oracle_lib.OracleProblem(w1).xact(w.psi_r, w.psi_i)
    r2, i2 = P.xact(w.psi_r, w.psi_i)
    assert np.abs((r - r2) + 1j * (i - i2)).max() > 1e-6


def _nonherm(w, seed=5):
    """The tiny workload with a core-hole lifetime Sigma'' on the band energies:
    H becomes non-Hermitian (complex diagonal)."""
    import dataclasses

    rng = np.random.default_rng(seed)
    return dataclasses.replace(w, ei=rng.uniform(0.005, 0.05, w.npsi))


def test_backwards_action_is_the_adjoint(oracle_lib):
    w = _nonherm(WL.make("tiny", seed=1))
    P = oracle_lib.OracleProblem(w)
    n = w.npsi
    H = _dense(P, n)
    Hb = np.zeros((n, n), complex)
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        r, i = P.xact(e, np.zeros(n), backwards=True)
        Hb[:, j] = r + 1j * i
    assert np.abs(H - H.conj().T).max() > 1e-4  # not Hermitian
    assert np.abs(Hb - H.conj().T).max() < 1e-14 * np.abs(H).max()


def test_two_sided_lanczos_reduces_to_lanczos_when_hermitian(tiny_problem, oracle_lib):
    w, P = tiny_problem
    rc, (ra, ia, rb, ib, rc_, ic), done = P.haydock_nonherm(30)
    assert rc == 0 and done == 30
    rh, ha, hia, hb, hdone = P.haydock(30)
    assert np.allclose(ra, ha, rtol=0, atol=1e-12 * np.abs(ha).max())
    assert np.allclose(rb * rc_ - ib * ic, hb * hb, rtol=1e-10)  # b c = b^2
    s1 = oracle_lib.write_core_bc(ra, ia, rb, ib, rc_, ic, 30, w.kpref, w.el, w.eh, 400, w.gam0)
    s0 = oracle_lib.write_core(ha, None, hb, 30, w.kpref, w.el, w.eh, 400, w.gam0)
    assert np.abs(s1[:, 2] - s0[:, 2]).max() < 1e-9 * np.abs(s0[:, 2]).max()


def test_two_sided_lanczos_moments(oracle_lib):
    """The tridiagonal T of the two-sided recurrence (A v_j = delta_{j+1} v_{j+1}
    + a_j v_j + beta_j v_{j-1}, stored as b = conj(beta), c = conj(delta))
    reproduces the moments w0^H A^k v0 of the non-Hermitian action for k < 2m."""
    w = _nonherm(WL.make("tiny", seed=1))
    P = oracle_lib.OracleProblem(w)
    n = w.npsi
    A = _dense(P, n)
    m = 8
    rc, (ra, ia, rb, ib, rc_, ic), done = P.haydock_nonherm(m)
    assert rc == 0 and done == m
    a = ra[:m] + 1j * ia[:m]
    b = rb[1:m] + 1j * ib[1:m]
    c = rc_[1:m] + 1j * ic[1:m]
    T = np.diag(a) + np.diag(np.conj(b), 1) + np.diag(np.conj(c), -1)
    v0 = w.allow * (w.psi_r + 1j * w.psi_i)
    for k in range(2 * m):
        exact = np.vdot(v0, np.linalg.matrix_power(A, k) @ v0)
        got = np.linalg.matrix_power(T, k)[0, 0]
        assert abs(got - exact) < 1e-9 * max(1.0, abs(exact)), (k, got, exact)


def test_two_sided_lanczos_spectrum_is_the_adjoint_resolvent(oracle_lib):
    """write_core on the stored coefficients (z - conj(a), b*c) gives
    kpref |Im <psi|(z - A^H)^-1|psi>| of the dense non-Hermitian action."""
    w = _nonherm(WL.make("tiny", seed=1))
    P = oracle_lib.OracleProblem(w)
    n = w.npsi
    A = _dense(P, n)
    m = 120
    rc, (ra, ia, rb, ib, rc_, ic), done = P.haydock_nonherm(m)
    assert rc == 0
    ne = 200
    s = oracle_lib.write_core_bc(ra, ia, rb, ib, rc_, ic, m, w.kpref, w.el, w.eh, ne, w.gam0)
    v0 = w.allow * (w.psi_r + 1j * w.psi_i)
    ex = np.zeros(ne + 1)
    for r in range(ne + 1):
        z = w.el + (w.eh - w.el) * r / ne + 1j * w.gam0
        ex[r] = w.kpref * abs(np.vdot(v0, np.linalg.solve(z * np.eye(n) - A.conj().T, v0)).imag)
    assert np.linalg.norm(s[:, 2] - ex) < 1e-5 * np.linalg.norm(ex)


@pytest.mark.parametrize("photon", [1, 4])
def test_calc_spect_core_is_write_core_on_the_midpoints(oracle_lib, kat, photon):
    """calc_spect_core (OCEAN_haydock.f90:1991-2027) evaluates write_core's
    fraction on the ne midpoints el + (eh - el)(2i+1)/(2ne): on the reference's
    own Lanczos coefficients it equals, bit for bit, the odd rows of write_core
    at 2 ne (which is pinned to the golden absspct files)."""
    O = oracle_lib
    p = f"p{photon}"
    n = int(kat[p + "_n"])
    kp = float(kat[p + "_kpref"])
    el, eh = float(kat["el_ev"]) * WL.EV2HARTREE, float(kat["eh_ev"]) * WL.EV2HARTREE
    gam = float(kat["gam0_ev"]) * WL.EV2HARTREE
    ne = 400
    ra, rb = kat[p + "_real_a"], kat[p + "_real_b"]
    ia = np.zeros_like(ra)
    sp = O.calc_spect_core(ra, ia, rb, n, kp, el, eh, ne, gam)
    wc = O.write_core(ra, ia, rb, n, kp, el, eh, 2 * ne, gam)
    assert np.array_equal(sp[:, 2], wc[1::2, 2])
    assert np.array_equal(sp[:, 1], wc[1::2, 4])
    assert np.array_equal(sp[:, 0], wc[1::2, 0])


def test_check_convergence_rel_area(oracle_lib, kat):
    """relArea = 2 sum|sp1 - sp2| / (sum|sp1| + sum|sp2|) over calc_spect_core's
    column 3, maxDiff its largest term (OCEAN_haydock.f90:1640-1652)."""
    O = oracle_lib
    n = int(kat["p1_n"])
    ra, rb = kat["p1_real_a"], kat["p1_real_b"]
    ia = np.zeros_like(ra)
    kp = float(kat["p1_kpref"])
    el, eh, gam = -1.0, 2.5, 0.05
    md, rel = O.check_convergence(ra, ia, rb, 150, 140, kp, el, eh, 300, gam)
    s1 = O.calc_spect_core(ra, ia, rb, 150, kp, el, eh, 300, gam)[:, 2]
    s2 = O.calc_spect_core(ra, ia, rb, 140, kp, el, eh, 300, gam)[:, 2]
    d, a1, a2 = 0.0, 0.0, 0.0
    for i in range(300):
        d += abs(s1[i] - s2[i])
        a1 += abs(s1[i])
        a2 += abs(s2[i])
    assert rel == 2.0 * d / (a1 + a2)
    assert md == np.max(np.abs(s1 - s2))
    assert n >= 150


def test_early_exit_two_in_a_row(oracle_lib):
    """The early exit stops at the first iteration whose relArea and the
    previous one's are both below the threshold (prevConv,
    OCEAN_haydock.f90:275-290); a single pass is not enough."""
    O = oracle_lib
    rel = np.array([0, 0, 0, 0.5, 0.01, 0.5, 0.01, 0.02, 0.001, 0.001])
    assert O.early_exit_iter(rel, 9, 2, 0.05) == 7
    assert O.early_exit_iter(rel, 9, 2, 0.005) == 9      # 8 and 9 pass
    assert O.early_exit_iter(rel, 9, 2, 0.0) == 9        # off
    assert O.early_exit_iter(rel, 6, 2, 0.05) == 6       # never twice in a row up to 6


def test_haydock_early_exit_matches_plain_run(tiny_problem, oracle_lib):
    """The early-exit run computes the same coefficients as the plain run up to
    its stopping iteration, which is the rule's answer on the relArea of each
    iteration recomputed from the plain run's coefficients."""
    O = oracle_lib
    w, P = tiny_problem
    niter, spacing, ne = 24, 3, 200
    rc, ra, ia, rb, done = P.haydock(niter)
    rels = np.zeros(niter + 1)
    for it in range(spacing + 1, niter + 1):
        rels[it] = O.check_convergence(ra, ia, rb, it, it - spacing, w.kpref, w.el, w.eh, ne, w.gam0)[1]
    thr = float(np.sort(rels[spacing + 1:])[niter // 2])  # some threshold that is met part-way
    stop = O.early_exit_iter(rels, niter, spacing, thr)
    assert spacing + 2 <= stop < niter
    rc2, ra2, ia2, rb2, done2, rel2 = P.haydock_conv(niter, thr, spacing, ne)
    assert rc2 == 0 and done2 == stop
    assert np.array_equal(ra2[:stop], ra[:stop]) and np.array_equal(rb2[:stop + 1], rb[:stop + 1])
    assert np.array_equal(rel2[spacing + 1:stop + 1], rels[spacing + 1:stop + 1])
