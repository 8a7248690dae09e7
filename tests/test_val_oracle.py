"""CPU tests of the valence BSE pieces that need no GPU.

* the library's host bubble builder (AI_bubble_populate with
  wall_search_old_way, OCEAN_bubble.f90:238-407) is bit-identical to the
  oracle's restatement, for even and odd meshes, zero and finite q;
* the oracle's valence action (OCEAN_action.f90:521-600) is Hermitian, term by
  term, on the synthetic inputs (the ladder satisfies ladder(-R,y,x) =
  ladder(R,x,y));
* the oracle's Haydock run over it reproduces the dense Hamiltonian's spectrum
  edges (Ritz values of the tridiagonal, redtrid);
* ocn_val_create rejects bad dimensions before touching a GPU.
"""
import ctypes as C

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL


@pytest.mark.parametrize("xmesh,qinb", [((4, 4, 4), (0, 0, 0)), ((3, 4, 5), (0, 0, 0)),
                                        ((6, 5, 4), (0.05, 0.0, 0.02)), ((10, 10, 10), (0, 0, 0))])
def test_bubble_matches_oracle_bit_for_bit(lib_built, oracle_lib, xmesh, qinb):
    capi.load(lib_built)
    O = oracle_lib
    a = 4.0 / WL.BOHR
    bvec = np.zeros(9)
    bvec[0], bvec[4], bvec[8] = 2 * np.pi / a, 2 * np.pi / (1.1 * a), 2 * np.pi / (0.9 * a)
    celvol = a ** 3 * 1.1 * 0.9
    b_lib, n_lib = capi.val_bubble(xmesh, bvec, qinb, celvol, 64)
    b_or, n_or = O.val_bubble(xmesh, bvec, qinb, celvol, 64)
    assert n_lib == n_or
    assert np.array_equal(b_lib, b_or)
    assert b_lib[0] == 0.0 and np.all(b_lib >= 0.0) and np.count_nonzero(b_lib) > 0


def test_bubble_is_inversion_symmetric_at_q0(lib_built):
    capi.load(lib_built)
    w = WL.make_val("vodd")
    b, _ = capi.val_bubble((5, 5, 5), w.bvec, (0, 0, 0), w.celvol, w.nk)
    B = b.reshape(5, 5, 5)
    assert np.array_equal(B, B[(-np.arange(5)) % 5][:, (-np.arange(5)) % 5][:, :, (-np.arange(5)) % 5])


@pytest.mark.parametrize("name", ["vtiny", "vodd", "vsmall"])
def test_oracle_action_is_hermitian(oracle_lib, name):
    O = oracle_lib
    w = WL.make_val(name, seed=3)
    P = O.OracleVal(w)
    rng = np.random.default_rng(5)
    n = w.npsi
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for flags in [(1, 1, 1), (0, 1, 0), (0, 0, 1)]:
        hx = P.act(x.real, x.imag, flags=flags)
        hy = P.act(y.real, y.imag, flags=flags)
        Hx, Hy = hx[0] + 1j * hx[1], hy[0] + 1j * hy[1]
        lhs, rhs = np.vdot(y, Hx), np.conj(np.vdot(x, Hy))
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs), flags


def test_oracle_haydock_brackets_the_dense_spectrum(oracle_lib):
    O = oracle_lib
    w = WL.make_val("vtiny", seed=4)
    P = O.OracleVal(w)
    n = w.npsi
    H = np.zeros((n, n), dtype=complex)
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        hr, hi = P.act(e, np.zeros(n))
        H[:, j] = hr + 1j * hi
    assert np.allclose(H, H.conj().T, atol=1e-13)
    ev = np.linalg.eigvalsh(H)
    niter = 40
    rc, ra, ia, rb, done = P.haydock(niter)
    assert rc == 0 and done == niter
    assert np.max(np.abs(ia[:niter])) < 1e-12 * np.max(np.abs(ra[:niter]))
    T = np.diag(ra[:niter]) + np.diag(rb[1:niter], 1) + np.diag(rb[1:niter], -1)
    ritz = np.linalg.eigvalsh(T)
    assert abs(ritz[0] - ev[0]) < 1e-8 and abs(ritz[-1] - ev[-1]) < 1e-8
    assert ritz[0] >= ev[0] - 1e-10 and ritz[-1] <= ev[-1] + 1e-10


def test_val_create_rejects_bad_dims_without_gpu(lib_built):
    lib = capi.load(lib_built)
    for change in [("nv", 0), ("nv", 33), ("nc", 0), ("precision", 5), ("nspn", 3), ("vspin", -1)]:
        d = capi.OcnValDims()
        d.nc, d.nv = 4, 2
        d.kmesh[:] = [2, 2, 2]
        d.xmesh[:] = [3, 3, 3]
        setattr(d, change[0], change[1])
        p = C.c_void_p()
        assert lib.ocn_val_create(C.byref(d), C.byref(p)) == capi.OCN_ERR_ARG
        assert not p.value
    d = capi.OcnValDims()
    d.nc, d.nv = 4, 2
    d.kmesh[:] = [2, 2, 40]
    d.xmesh[:] = [3, 3, 3]
    p = C.c_void_p()
    assert lib.ocn_val_create(C.byref(d), C.byref(p)) == capi.OCN_ERR_ARG
    assert "mesh" in capi.val_last_error()


# ---- write_val (the valence spectrum, file "opcons") against EXAMPLE/Si_valence

# EXAMPLE/Si_valence/opcons: 2000 rows, spect_range {2000 0 20} eV (Si.in); the
# fixture keeps every OPCONS_STRIDE-th row (tests/golden/make_opcons_fixture.py)
OPCONS_STRIDE = 5
OPCONS_NE = 2000


def _opcons_rows():
    import os

    from conftest import ROOT

    path = os.path.join(ROOT, "tests", "golden", "opcons_Si_valence_rows.txt")
    return [l.rstrip("\n") for l in open(path)]


def test_opcons_grid_and_optical_constants_match_the_reference(lib_built):
    capi.load(lib_built)
    lines = _opcons_rows()
    vals = np.array([[float(x) for x in l.split()] for l in lines[1:]])
    ne = OPCONS_NE
    rows = np.arange(0, ne, OPCONS_STRIDE)
    assert len(vals) == len(rows)
    el, eh = 0.0 * WL.EV2HARTREE, 20.0 * WL.EV2HARTREE
    omega = el + (eh - el) * (2 * rows + 1) / (2 * ne)
    out = capi.val_optical_constants(omega, vals[:, 1], vals[:, 2])
    # the energy grid (midpoints) and the columns that are pure functions of eps
    assert np.max(np.abs(out[:, 0] - vals[:, 0]) / vals[:, 0]) < 1e-13
    for j in (3, 4, 6, 7):
        ref = vals[:, j]
        err = np.abs(out[:, j] - ref) / np.maximum(np.abs(ref), 1e-300)
        assert np.max(err) < 1e-13, (j, np.max(err))
    # mu carries the physical constants, which the file's OCEAN version rounded
    # differently (5e-11 relative)
    nz = vals[:, 5] != 0
    assert np.max(np.abs(out[nz, 5] - vals[nz, 5]) / np.abs(vals[nz, 5])) < 1e-9


def test_opcons_writer_is_byte_identical(lib_built, tmp_path):
    capi.load(lib_built)
    lines = _opcons_rows()
    vals = np.array([[float(x) for x in l.split()] for l in lines[1:]])
    path = str(tmp_path / "opcons")
    capi.write_opcons(path, vals)
    assert open(path).read().splitlines() == lines


@pytest.mark.parametrize("semi_tda", [False, True])
def test_oracle_write_val_is_the_resolvent(oracle_lib, semi_tda):
    """With a vanishing last b the terminator drops out and eps is
    1 - fact [G(z) (+ G'(-z))] of the tridiagonal matrix (dense solve)."""
    O = oracle_lib
    rng = np.random.default_rng(8)
    n = 30
    ra = np.concatenate([rng.uniform(0.1, 0.9, n), [0.0]])
    rb = np.concatenate([[0.0], rng.uniform(0.02, 0.1, n - 1), [1e-12]])
    kpref, ucvol, gam0, ne = 0.7, 270.0, 0.01, 50
    el, eh = 0.05, 1.2
    out = O.write_val(ra, None, rb, n, kpref, ucvol, el, eh, ne, gam0, 1, semi_tda)
    T = np.diag(ra[:n]) + np.diag(rb[1:n], 1) + np.diag(rb[1:n], -1)
    fact = kpref * 2 * ucvol
    e1 = np.zeros(n)
    e1[0] = 1.0
    for r in range(ne):
        om = el + (eh - el) * (2 * r + 1) / (2 * ne)
        z = om + 1j * gam0
        eps = 1.0 - fact * np.linalg.solve(z * np.eye(n) - T, e1)[0]
        if semi_tda:
            eps -= fact * np.linalg.solve(-z * np.eye(n) - T, e1)[0]
        assert abs(out[r, 1] + 1j * out[r, 2] - eps) < 1e-9 * abs(eps), r


@pytest.mark.parametrize("nspn,vspin", [(1, 2), (2, 2), (2, 1)])
def test_oracle_spin_blocks_hermitian(oracle_lib, nspn, vspin):
    O = oracle_lib
    w = WL.make_val("vtiny", seed=6, nspn=nspn, vspin=vspin)
    assert w.npsi == w.nc * w.nv * w.nk * vspin * vspin
    P = O.OracleVal(w)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
    y = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
    hx, hy = P.act(x.real, x.imag), P.act(y.real, y.imag)
    lhs = np.vdot(y, hx[0] + 1j * hx[1])
    rhs = np.conj(np.vdot(x, hy[0] + 1j * hy[1]))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_oracle_singlet_reduces_to_one_spin_channel(oracle_lib):
    """valence_ham_spin = 2 with one DFT spin: a singlet psi (blocks up-up =
    down-down = z, spin-flip blocks 0) maps to a singlet whose up-up block is
    the one-channel action on z (exchange: two blocks at spin_prefac 1 = one
    block at 2), and the spin-flip blocks get nothing."""
    import dataclasses

    O = oracle_lib
    w2 = WL.make_val("vsmall", seed=7, nspn=1, vspin=2)
    nb1 = w2.npsi // 4
    w1 = dataclasses.replace(w2, vspin=1, er=w2.er[:nb1].copy(), ei=w2.ei[:nb1].copy(),
                             allow=w2.allow[:nb1].copy(), psi_r=w2.psi_r[:nb1].copy(), psi_i=w2.psi_i[:nb1].copy())
    rng = np.random.default_rng(4)
    z = rng.standard_normal(nb1) + 1j * rng.standard_normal(nb1)
    psi = np.zeros(w2.npsi, complex)
    psi[:nb1] = z
    psi[3 * nb1:] = z
    h2 = O.OracleVal(w2).act(psi.real, psi.imag)
    h1 = O.OracleVal(w1).act(z.real, z.imag)
    H2 = h2[0] + 1j * h2[1]
    H1 = h1[0] + 1j * h1[1]
    assert np.max(np.abs(H2[:nb1] - H1)) < 1e-13 * np.max(np.abs(H1))
    assert np.max(np.abs(H2[3 * nb1:] - H1)) < 1e-13 * np.max(np.abs(H1))
    assert np.max(np.abs(H2[nb1:3 * nb1])) == 0.0


def test_fxc_kernel_matches_oracle_bit_for_bit(lib_built, oracle_lib):
    """OCEAN_fxc_prep's ALDA kernel (five-point second derivative of n(ex + ec),
    Perdew-Zunger correlation): library host code against the oracle."""
    capi.load(lib_built)
    O = oracle_lib
    w = WL.make_val("vsmall", with_fxc=True)
    rho = np.concatenate([w.rho, [1e-9, 0.003, 0.5, 3.0]])  # both sides of rs = 1 and the cutoff
    a = capi.val_fxc_from_rho(rho[:-4].copy(), w.celvol, w.nk)
    b = O.val_fxc_from_rho(rho[:-4].copy(), w.celvol, w.nk)
    assert np.array_equal(a, b) and np.all(a < 0.0)
    a2 = capi.val_fxc_from_rho(rho, w.celvol, w.nk)
    b2 = O.val_fxc_from_rho(rho, w.celvol, w.nk)
    assert np.array_equal(a2, b2)


def test_oracle_fxc_term_is_hermitian(oracle_lib):
    O = oracle_lib
    w = WL.make_val("vodd", seed=2, with_fxc=True)
    P = O.OracleVal(w)
    rng = np.random.default_rng(6)
    x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
    y = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
    hx, hy = P.act(x.real, x.imag, flags=(0, 0, 0)), P.act(y.real, y.imag, flags=(0, 0, 0))
    lhs = np.vdot(y, hx[0] + 1j * hx[1])
    rhs = np.conj(np.vdot(x, hy[0] + 1j * hy[1]))
    assert abs(lhs) > 0 and abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_valence_host_entry_points_reject_bad_arguments(lib_built, tmp_path):
    """Host-side valence entry points return OCN_ERR_ARG instead of aborting."""
    import ctypes as C

    lib = capi.load(lib_built)
    out = np.zeros(64)
    bvec = (C.c_double * 9)(*([1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0]))
    q = (C.c_double * 3)(0, 0, 0)
    assert lib.ocn_val_bubble_populate((C.c_int * 3)(4, 4, 4), bvec, q, C.c_double(-1.0), 8, capi._dp(out),
                                       None) == capi.OCN_ERR_ARG
    assert lib.ocn_val_bubble_populate((C.c_int * 3)(4, 0, 4), bvec, q, C.c_double(1.0), 8, capi._dp(out),
                                       None) == capi.OCN_ERR_ARG
    with pytest.raises(capi.OcnError):
        capi.val_pair_energies(2, 2, 1, 1, 1, np.zeros(3), 3, 3, np.zeros(3), 3, 1)  # conduction window past the file
    with pytest.raises(capi.OcnError):
        capi.val_fxc_from_rho(np.ones(4), -1.0, 8)
    with pytest.raises(capi.OcnError):
        capi.read_val_u2(str(tmp_path / "missing"), (2, 2, 2), 1, 1, 1, 2, 1, 2)
    assert lib.ocn_val_optical_constants(-1, None, None, None, None) == capi.OCN_ERR_ARG
    assert lib.ocn_write_opcons(str(tmp_path / "x").encode(), 1, None) == capi.OCN_ERR_ARG


def test_valence_gmres_matches_dense_solve(oracle_lib):
    """GMRES over the valence action (OCEAN_gmres.f90:508-908, have_val) solves
    ((w + i G) - H) x = allow o psi0 at tight tolerance: <b|x> against a dense
    solve of the same action, and the outputs scaled by fact = kpref 2 celvol."""
    O = oracle_lib
    w = WL.make_val("vtiny", seed=31)
    P = O.OracleVal(w)
    n = w.npsi
    H = np.zeros((n, n), complex)
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        hr, hi = P.act(e, np.zeros(n))
        H[:, j] = hr + 1j * hi
    E = np.array([5.0, 5.2, 9.0])
    rc, ore, oim, rel, its, tot = P.gmres(E, depth=12, ffff=1e-22, max_restarts=400)
    assert rc == 0
    b = w.allow * (w.psi_r + 1j * w.psi_i)
    fact = w.kpref * 2.0 * w.celvol
    for i, ev in enumerate(E):
        z = ev * WL.EV2HARTREE + 1j * w.gam0
        x = np.linalg.solve(z * np.eye(n) - H, b)
        f = np.vdot(b, x)
        assert abs((1.0 - f.real * fact) - ore[i]) < 1e-9 * abs(ore[i])
        assert abs(-f.imag * fact - oim[i]) < 1e-9 * abs(oim[i])
