"""Valence BSE action and Haydock on the GPU against the oracle.

Tolerances
  * FP64 H psi vs oracle (each term alone and all together): relative 2-norm < 1e-12
  * mixed H psi vs oracle: relative 2-norm < 1e-6 (the FP32 interaction terms
    are a small fraction of H psi on these inputs; each term alone: < 1e-5)
  * FP64 Haydock: first 10 a_n relative < 1e-12, b_n < 1e-12
  * mixed Haydock: spectrum (Spect(0) column) relative < 1e-4
  * benchmark size (v2, states and ladder built on the device): Hermiticity
    |<y|Hx> - conj(<x|Hy>)| / |<y|Hx>| < 1e-12 (FP64), < 1e-6 (mixed), and
    linearity H(x + 2y) = Hx + 2Hy to 1e-12 (FP64)
"""
import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    import torch  # noqa: F401

    return capi.load(lib_built), oracle_lib


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", ["vtiny", "vsmall", "vodd"])
@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_apply_matches_oracle(built, name, prec):
    _, O = built
    w = WL.make_val(name, seed=11)
    P = O.OracleVal(w)
    ctx = capi.ValContext(w, precision=prec)
    try:
        rng = np.random.default_rng(2)
        x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        for flags in [(1, 1, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1)]:
            for back in (False, True):
                gr, gi = ctx.apply_H(x.real, x.imag, flags=flags, backwards=back)
                orr, oi = P.act(x.real, x.imag, backwards=back, flags=flags)
                assert np.linalg.norm(orr + 1j * oi) > 0.0, (name, flags)
                err = _rel(gr + 1j * gi, orr + 1j * oi)
                if prec == capi.OCN_PREC_FP64:
                    tol = 1e-12
                else:  # FP32 interaction terms: each alone to 1e-5, with the energies to 1e-6
                    tol = 1e-5 if flags in ((0, 1, 0), (0, 0, 1)) else 1e-6
                assert err < tol, (name, flags, back, err)
    finally:
        ctx.close()


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_haydock_matches_oracle(built, prec):
    _, O = built
    w = WL.make_val("vsmall", seed=12)
    P = O.OracleVal(w)
    ctx = capi.ValContext(w, precision=prec)
    try:
        niter = 30
        ra, ia, rb, done = ctx.haydock(niter)
        rc, ora, oia, orb, odone = P.haydock(niter)
        assert rc == 0 and done == niter == odone
        if prec == capi.OCN_PREC_FP64:
            assert np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
            assert np.max(np.abs(rb[1:11] - orb[1:11]) / np.abs(orb[1:11])) < 1e-12
        s = capi.spectrum_cf(ra, ia, rb, niter, w.kpref, w.el, w.eh, 400, w.gam0)
        so = O.write_core(ora, oia, orb, niter, w.kpref, w.el, w.eh, 400, w.gam0)
        assert _rel(s[:, 2], so[:, 2]) < (1e-10 if prec == capi.OCN_PREC_FP64 else 1e-4)
    finally:
        ctx.close()


def test_device_entry_points_equal_host_ones(built):
    import torch

    w = WL.make_val("vodd", seed=13)
    ctx = capi.ValContext(w, precision=capi.OCN_PREC_MIXED)
    try:
        hr, hi = ctx.apply_H(w.psi_r, w.psi_i)
        d_in = torch.tensor(np.concatenate([w.psi_r, w.psi_i]), device="cuda:0")
        d_out = torch.empty_like(d_in)
        torch.cuda.synchronize()
        ctx.apply_H_dev(d_in.data_ptr(), d_out.data_ptr())
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        assert np.array_equal(out[:w.npsi], hr) and np.array_equal(out[w.npsi:], hi)
        a1 = ctx.haydock(12)
        a2 = ctx.haydock_dev(12, d_in.data_ptr())
        assert np.array_equal(a1[0], a2[0]) and np.array_equal(a1[2], a2[2])
    finally:
        ctx.close()


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_benchmark_size_is_hermitian_and_linear(built, prec):
    import torch

    w = WL.make_val("v2", seed=14, device="cuda:0")
    ctx = capi.ValContext(w, precision=prec)
    try:
        g = torch.Generator(device="cuda:0")
        g.manual_seed(7)
        n = w.npsi
        x = torch.randn(2 * n, generator=g, device="cuda:0", dtype=torch.float64)
        y = torch.randn(2 * n, generator=g, device="cuda:0", dtype=torch.float64)
        hx, hy, hz = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
        torch.cuda.synchronize()
        ctx.apply_H_dev(x.data_ptr(), hx.data_ptr())
        ctx.apply_H_dev(y.data_ptr(), hy.data_ptr())
        z = x + 2.0 * y
        torch.cuda.synchronize()
        ctx.apply_H_dev(z.data_ptr(), hz.data_ptr())
        torch.cuda.synchronize()
        c = lambda v: torch.complex(v[:n], v[n:])  # noqa: E731
        lhs = torch.vdot(c(y), c(hx)).item()
        rhs = torch.vdot(c(x), c(hy)).conj().item()
        tol = 1e-12 if prec == capi.OCN_PREC_FP64 else 1e-6
        assert abs(lhs - rhs) / abs(lhs) < tol
        lin = (torch.linalg.norm(c(hz) - c(hx) - 2.0 * c(hy)) / torch.linalg.norm(c(hz))).item()
        assert lin < (1e-12 if prec == capi.OCN_PREC_FP64 else 1e-6)
        assert torch.isfinite(hz).all()
    finally:
        ctx.close()


@pytest.mark.parametrize("semi_tda,backf,cplx", [(False, False, False), (True, False, False), (True, True, False),
                                                 (False, False, True)])
def test_val_spectrum_matches_oracle(built, semi_tda, backf, cplx):
    """write_val on the GPU against the oracle: 1e-13 relative per column."""
    _, O = built
    rng = np.random.default_rng(21)
    n = 60
    ra = rng.uniform(0.1, 0.9, n + 1)
    rb = np.concatenate([[0.0], rng.uniform(0.02, 0.2, n)])
    ia = ib = rc = ic = None
    if cplx:
        ia = rng.uniform(-0.01, 0.01, n + 1)
        ib = rng.uniform(-0.02, 0.02, n + 1)
        rc = rb * rng.uniform(0.9, 1.1, n + 1)
        ic = rng.uniform(-0.02, 0.02, n + 1)
    args = (n, 0.7, 270.0, 0.0, 1.3, 500, 0.01)
    g = capi.val_spectrum(ra, ia, rb, *args, val_ham_spin=1, semi_tda=semi_tda, backf=backf, ib=ib, rc=rc, ic=ic)
    o = O.write_val(ra, ia, rb, *args, 1, semi_tda, backf, ib=ib, rc=rc, ic=ic)
    for j in range(8):
        err = np.abs(g[:, j] - o[:, j]) / np.maximum(np.abs(o[:, j]), 1e-300)
        assert np.max(err) < 1e-13, (j, np.max(err))


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_valence_haydock_spectrum_end_to_end(built, prec):
    """Haydock over the valence action, then write_val: GPU against the oracle's
    whole run (eps2 column, relative 2-norm 1e-10 FP64, 1e-4 mixed)."""
    _, O = built
    w = WL.make_val("vsmall", seed=23)
    ctx = capi.ValContext(w, precision=prec)
    try:
        niter = 30
        ra, ia, rb, done = ctx.haydock(niter)
    finally:
        ctx.close()
    P = O.OracleVal(w)
    rc, ora, oia, orb, _ = P.haydock(niter)
    assert rc == 0 and done == niter
    args = (niter, w.kpref, w.celvol, w.el, w.eh, 400, w.gam0)
    g = capi.val_spectrum(ra, ia, rb, *args, semi_tda=True)
    o = O.write_val(ora, oia, orb, *args, 1, True)
    err = np.linalg.norm(g[:, 2] - o[:, 2]) / np.linalg.norm(o[:, 2])
    assert err < (1e-10 if prec == capi.OCN_PREC_FP64 else 1e-4), err


@pytest.mark.parametrize("nspn,vspin", [(1, 2), (2, 2), (2, 1)])
@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_spin_blocks_match_oracle(built, nspn, vspin, prec):
    _, O = built
    w = WL.make_val("vsmall", seed=31, nspn=nspn, vspin=vspin)
    P = O.OracleVal(w)
    ctx = capi.ValContext(w, precision=prec)
    try:
        rng = np.random.default_rng(3)
        x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        for flags in [(1, 1, 1), (0, 1, 0), (0, 0, 1)]:
            gr, gi = ctx.apply_H(x.real, x.imag, flags=flags)
            orr, oi = P.act(x.real, x.imag, flags=flags)
            err = _rel(gr + 1j * gi, orr + 1j * oi)
            tol = 1e-12 if prec == capi.OCN_PREC_FP64 else (1e-6 if flags == (1, 1, 1) else 1e-5)
            assert err < tol, (flags, err)
        ra, ia, rb, done = ctx.haydock(20)
        rc, ora, oia, orb, _ = P.haydock(20)
        if prec == capi.OCN_PREC_FP64:
            assert np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
    finally:
        ctx.close()


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_fxc_term_matches_oracle(built, prec):
    _, O = built
    w = WL.make_val("vsmall", seed=41, with_fxc=True)
    P = O.OracleVal(w)
    ctx = capi.ValContext(w, precision=prec)
    try:
        rng = np.random.default_rng(4)
        x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        for flags in [(0, 0, 0), (0, 1, 0), (1, 1, 1)]:
            gr, gi = ctx.apply_H(x.real, x.imag, flags=flags)
            orr, oi = P.act(x.real, x.imag, flags=flags)
            err = _rel(gr + 1j * gi, orr + 1j * oi)
            tol = 1e-12 if prec == capi.OCN_PREC_FP64 else (1e-6 if flags == (1, 1, 1) else 1e-5)
            assert err < tol, (flags, err)
        import ctypes as C

        ctx._chk(ctx.lib.ocn_val_set_fxc(ctx.ptr, None))  # off again: the exchange alone
        gr, gi = ctx.apply_H(x.real, x.imag, flags=(0, 1, 0))
        P0 = O.OracleVal(__import__("dataclasses").replace(w, rho=None))
        orr, oi = P0.act(x.real, x.imag, flags=(0, 1, 0))
        assert _rel(gr + 1j * gi, orr + 1j * oi) < (1e-12 if prec == capi.OCN_PREC_FP64 else 1e-5)
    finally:
        ctx.close()


def test_fxc_refuses_two_spins(built):
    w = WL.make_val("vtiny", seed=1, vspin=2)
    ctx = capi.ValContext(w)
    try:
        with pytest.raises(capi.OcnError) as e:
            ctx._chk(ctx.lib.ocn_val_set_fxc(ctx.ptr, capi._dp(np.ones(w.nx))))
        assert e.value.code == 9962
    finally:
        ctx.close()


def test_state_and_argument_errors(built):
    """Missing operator data and bad arguments return status codes (no abort)."""
    import ctypes as C

    lib, _ = built
    w = WL.make_val("vtiny", seed=2)
    d = capi.OcnValDims()
    d.nc, d.nv = w.nc, w.nv
    d.kmesh[:] = list(w.kmesh)
    d.xmesh[:] = list(w.xmesh)
    p = C.c_void_p()
    assert lib.ocn_val_create(C.byref(d), C.byref(p)) == 0
    try:
        n = w.npsi
        a = np.zeros(n)
        flags = (C.c_int * 3)(1, 1, 1)
        rc = lib.ocn_val_apply_H(p, capi._dp(a), capi._dp(a), capi._dp(a), capi._dp(a), flags, 0)
        assert rc == capi.OCN_ERR_STATE and "not set" in capi.val_last_error(p)
        assert lib.ocn_val_set_energies(p, None, None) == capi.OCN_ERR_ARG
        assert lib.ocn_val_set_allow(p, capi._dp(np.ones(n))) == 0
        only_e = (C.c_int * 3)(1, 0, 0)
        rc = lib.ocn_val_apply_H(p, capi._dp(a), capi._dp(a), capi._dp(a), capi._dp(a), only_e, 0)
        assert rc == capi.OCN_ERR_STATE  # energies still missing
        ra, ia, rb = np.zeros(5), np.zeros(5), np.zeros(5)
        done = C.c_int(0)
        rc = lib.ocn_val_haydock(p, capi._dp(a), capi._dp(a), 0, flags, capi._dp(ra), capi._dp(ia), capi._dp(rb),
                                 C.byref(done))
        assert rc == capi.OCN_ERR_ARG
    finally:
        lib.ocn_val_destroy(p)


def test_many_valence_bands_on_a_cubic_mesh(built):
    """Nv = 16 on the 8^3 k-mesh: more (line, v) pairs than the cubic kernel
    keeps in registers, so the generic direct-term kernel runs (A and B sums of
    one x-point in shared memory, 131 KB in FP32) -- same results; in FP64 that
    is 262 KB: OCN_ERR_UNSUPPORTED at creation."""
    _, O = built
    w = WL.make_val("vtiny", seed=51, nc=4, nv=16, kmesh=(8, 8, 8), xmesh=(4, 3, 2))
    P = O.OracleVal(w)
    ctx = capi.ValContext(w, precision=capi.OCN_PREC_MIXED)
    try:
        rng = np.random.default_rng(8)
        x = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        gr, gi = ctx.apply_H(x.real, x.imag, flags=(0, 0, 1))
        orr, oi = P.act(x.real, x.imag, flags=(0, 0, 1))
        assert _rel(gr + 1j * gi, orr + 1j * oi) < 1e-5
    finally:
        ctx.close()
    with pytest.raises(capi.OcnError) as e:
        capi.ValContext(w, precision=capi.OCN_PREC_FP64)
    assert e.value.code == 9962 and "shared memory" in str(e.value)


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_smaller_context_keeps_larger_one_working(built, prec):
    """Kernel shared-memory limits are process-wide: a small context created
    while a large one is alive must not shrink them under the large one."""
    _, O = built
    big = WL.make_val("vsmall", seed=21, nv=4, kmesh=(8, 8, 8))
    small = WL.make_val("vtiny", seed=22)
    cb = capi.ValContext(big, precision=prec)
    try:
        r1 = cb.apply_H(big.psi_r, big.psi_i)
        cs = capi.ValContext(small, precision=prec)
        try:
            cs.apply_H(small.psi_r, small.psi_i)
            r2 = cb.apply_H(big.psi_r, big.psi_i)
        finally:
            cs.close()
        assert np.array_equal(r1[0], r2[0]) and np.array_equal(r1[1], r2[1])
        orr, oi = O.OracleVal(big).act(big.psi_r, big.psi_i)
        assert _rel(r2[0] + 1j * r2[1], orr + 1j * oi) < (1e-12 if prec == capi.OCN_PREC_FP64 else 1e-6)
    finally:
        cb.close()


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_valence_gmres_matches_oracle(built, prec):
    """GMRES over the valence action (ocn_val_gmres; OCEAN_gmres.f90:508-908 with
    the have_val branches) against the oracle's sweep: FP64 within 1e-8 at a
    tight tolerance (the same iteration counts within one), mixed within 1e-4
    at a tolerance above its precision floor."""
    _, O = built
    w = WL.make_val("vsmall", seed=32)
    P = O.OracleVal(w)
    E = np.array([6.0, 6.2, 6.4, 11.0])
    tol = 1e-20 if prec == capi.OCN_PREC_FP64 else 1e-10
    ctx = capi.ValContext(w, precision=prec)
    try:
        ore, oim, rel, its = ctx.gmres(E, depth=16, tol=tol, max_restarts=500)
    finally:
        ctx.close()
    rc, ore2, oim2, rel2, its2, tot = P.gmres(E, depth=16, ffff=1e-20, max_restarts=500)
    assert rc == 0
    bar = 1e-8 if prec == capi.OCN_PREC_FP64 else 1e-4
    assert np.max(np.abs(oim - oim2) / np.abs(oim2)) < bar
    assert np.max(np.abs(ore - ore2) / np.abs(ore2)) < bar
    if prec == capi.OCN_PREC_FP64:
        assert np.max(np.abs(its - its2)) <= 1
