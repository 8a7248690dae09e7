"""GPU parity tests: libocean_gpu.so (through its C ABI) against the CPU oracle
on the same seeded inputs.

Tolerances
  * index bookkeeping (xshift, W, phased u2): bit-exact
  * FP64 action H*psi:      ||dH|| / ||H psi|| < 1e-12
  * FP64 Lanczos:           first 10 a_n, b_n relative < 1e-12
  * continued fraction:     GPU vs oracle < 1e-12 relative; vs golden file 6e-8
  * GMRES (FP64):           eps2 within 1e-8 relative of the oracle's
"""
import os

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    return capi.load(lib_built), oracle_lib


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


PROBLEMS = {}


def problem(name, O, seed=0, **kw):
    key = (name, seed, tuple(sorted(kw.items())))
    if key not in PROBLEMS:
        w = WL.make(name, seed=seed, **kw)
        PROBLEMS[key] = (w, O.OracleProblem(w))
    return PROBLEMS[key]


@pytest.mark.parametrize("name", ["tiny", "c1"])
def test_bloch_phase_and_W_bit_exact(built, name):
    _, O = built
    w, P = problem(name, O)
    ctx = capi.Context(w)
    try:
        ur, ui = ctx.get_bloch()
        W, xs, tau = ctx.get_W()
    finally:
        ctx.close()
    assert xs == P.xshift and tau == P.tau_shifted
    assert np.array_equal(W, P.W)
    assert np.array_equal(ur, P.ur) and np.array_equal(ui, P.ui)


@pytest.mark.parametrize("name", ["tiny", "small", "c1", "c3small"])
def test_apply_H_fp64_matches_oracle(built, name):
    _, O = built
    w, P = problem(name, O, seed=4)
    ctx = capi.Context(w)
    try:
        rng = np.random.default_rng(11)
        for trial in range(2):
            pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
            hr, hi = ctx.apply_H(pr, pi)
            orr, oi = P.xact(pr, pi)
            assert _rel(hr + 1j * hi, orr + 1j * oi) < 1e-12
        assert ctx.launches > 0
    finally:
        ctx.close()


@pytest.mark.parametrize("hflag", [(0, 1, 1, 1, 1, 1), (1, 1, 1, 1, 0, 1), (1, 1, 1, 1, 1, 0),
                                   (0, 1, 1, 1, 0, 0)])
@pytest.mark.parametrize("backwards", [False, True])
def test_apply_H_term_switches(built, hflag, backwards):
    _, O = built
    w = WL.make("c3small", seed=5)
    w.ei = np.linspace(0.0, 0.01, w.npsi)  # complex energies exercise the backwards conjugate
    P = O.OracleProblem(w)
    ctx = capi.Context(w)
    try:
        hr, hi = ctx.apply_H(w.psi_r, w.psi_i, hflag=hflag, backwards=backwards)
        orr, oi = P.xact(w.psi_r, w.psi_i, hflag=hflag, backwards=backwards)
        assert _rel(hr + 1j * hi, orr + 1j * oi) < 1e-12
    finally:
        ctx.close()


def test_apply_H_hermitian_on_gpu(built):
    _, O = built
    w, _ = problem("c3small", O, seed=6)
    ctx = capi.Context(w)
    try:
        rng = np.random.default_rng(2)
        a = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        b = rng.standard_normal(w.npsi) + 1j * rng.standard_normal(w.npsi)
        ha = np.array(ctx.apply_H(a.real.copy(), a.imag.copy()))
        hb = np.array(ctx.apply_H(b.real.copy(), b.imag.copy()))
        ha = ha[0] + 1j * ha[1]
        hb = hb[0] + 1j * hb[1]
        assert abs(np.vdot(b, ha) - np.vdot(hb, a)) < 1e-12 * abs(np.vdot(b, ha))
    finally:
        ctx.close()


@pytest.mark.parametrize("name,niter", [("small", 30), ("c1", 60), ("c3small", 30)])
def test_haydock_fp64_matches_oracle(built, name, niter):
    _, O = built
    w, P = problem(name, O, seed=7)
    ctx = capi.Context(w)
    try:
        ra, ia, rb, done = ctx.haydock(niter)
    finally:
        ctx.close()
    rc, ora, oia, orb, odone = P.haydock(niter)
    assert rc == 0 and done == odone == niter
    assert np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
    assert np.max(np.abs(rb[1:11] - orb[1:11]) / np.abs(orb[1:11])) < 1e-12
    assert np.max(np.abs(ia[:niter])) < 1e-12
    # spectra from both coefficient sets
    sg = capi.spectrum_cf(ra, ia, rb, niter, w.kpref, w.el, w.eh, 400, w.gam0)
    so = O.write_core(ora, oia, orb, niter, w.kpref, w.el, w.eh, 400, w.gam0)
    assert _rel(sg[:, 2], so[:, 2]) < 1e-9


def test_haydock_nan_returns_reference_ierr(built):
    _, O = built
    w, _ = problem("tiny", O, seed=8)
    ctx = capi.Context(w)
    try:
        pr = w.psi_r.copy()
        pr[0] = np.nan
        with pytest.raises(capi.OcnError) as ei:
            ctx.haydock(4, pr, w.psi_i)
        assert ei.value.code == -1
        # the context stays usable after the error
        ra, ia, rb, done = ctx.haydock(4)
        assert done == 4 and np.all(np.isfinite(ra[:4]))
    finally:
        ctx.close()


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_haydock_graph_replay_deterministic(built, prec):
    """The captured 3-iteration graph plus the remainder iterations give the same
    coefficients on every call (deterministic reductions), for counts that are and
    are not multiples of three, and match the oracle's first coefficients."""
    _, O = built
    w, P = problem("small", O, seed=12)
    ctx = capi.Context(w, precision=prec)
    try:
        r1 = ctx.haydock(31)
        ctx.timing(True)  # graph re-captured with event-record nodes
        r2 = ctx.haydock(31)
        kt = ctx.timing_read()
        ctx.timing(False)
        r3 = ctx.haydock(30)
        r4 = ctx.haydock(2)
        # no stale CUDA error leaks into the next library call
        capi.spectrum_cf(r2[0], r2[1], r2[2], 31, w.kpref, w.el, w.eh, 50, w.gam0)
    finally:
        ctx.close()
    assert kt["combine_lanczos"][0] >= 3 and kt["lr_band_to_x"][1] > 0.0
    assert all(np.array_equal(a, b) for a, b in zip(r1[:3], r2[:3]))
    assert np.array_equal(r1[0][:30], r3[0][:30]) and np.array_equal(r1[2][:31], r3[2][:31])
    assert np.array_equal(r1[0][:2], r4[0][:2])
    _, ora, oia, orb, _ = P.haydock(31)
    tol = 1e-12 if prec == capi.OCN_PREC_FP64 else 1e-4
    assert np.max(np.abs(r1[0][:10] - ora[:10]) / np.abs(ora[:10])) < tol


@pytest.mark.parametrize("photon", [1, 5])
def test_spectrum_cf_reproduces_reference_golden(built, photon):
    _, O = built
    d = np.load(os.path.join(ROOT, "tests", "golden", "cu_twophoton_kat.npz"))
    p = f"p{photon}"
    n = int(d[p + "_n"])
    args = (d[p + "_real_a"], None, d[p + "_real_b"], n, float(d[p + "_kpref"]),
            -30.0 * WL.EV2HARTREE, 70.0 * WL.EV2HARTREE, 5000, 1.245 * WL.EV2HARTREE)
    g = capi.spectrum_cf(*args, ucvol=float(d[p + "_vol"]))
    o = O.write_core(*args, 0.0, 0.0, float(d[p + "_vol"]))
    assert np.max(np.abs(g - o) / np.maximum(np.abs(o), 1e-300)) < 1e-12
    ref = d[p + "_spct"]
    got = g[d[p + "_rows"]]
    nz = ref != 0
    assert np.max(np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])) < 6e-8


def test_spectrum_voigt_matches_oracle(built):
    _, O = built
    d = np.load(os.path.join(ROOT, "tests", "golden", "cu_twophoton_kat.npz"))
    n = int(d["p3_n"])
    args = (d["p3_real_a"], None, d["p3_real_b"], n, float(d["p3_kpref"]),
            -30.0 * WL.EV2HARTREE, 70.0 * WL.EV2HARTREE, 500, 1.245 * WL.EV2HARTREE)
    gg = 0.8 * WL.EV2HARTREE
    g = capi.spectrum_cf(*args, gam_gauss=gg, nval=0.05, eps=4.0)
    o = O.write_core(*args, 0.0, gg, 1.0, 0, 0.05, 4.0)
    assert np.max(np.abs(g[:, :5] - o[:, :5]) / np.maximum(np.abs(o[:, :5]), 1e-300)) < 1e-9


@pytest.mark.parametrize("lanes", [1, 3])
@pytest.mark.parametrize("name", ["tiny", "small"])
def test_gmres_fp64_matches_oracle(built, name, lanes):
    """Recycled GMRES (one projection per recycled energy, and energy lanes)
    against the oracle's restatement of the reference's sequential updates."""
    _, O = built
    w, P = problem(name, O, seed=9)
    E = np.array([4.0, 4.1, 4.2, 4.3, 8.0, 8.05])
    ctx = capi.Context(w)
    try:
        ctx.set_gmres_lanes(lanes)
        ore, oim, rel, its = ctx.gmres(E, depth=16, tol=1e-20, max_restarts=500)
    finally:
        ctx.close()
    rc, ore2, oim2, rel2, its2, tot = P.gmres(E, depth=16, ffff=1e-20, max_restarts=500)
    assert rc == 0
    assert np.max(np.abs(oim - oim2) / np.abs(oim2)) < 1e-8
    assert np.max(np.abs(ore - ore2) / np.abs(ore2)) < 1e-8
    if lanes == 1:  # the same sweep: the same iteration counts (the threshold is near the FP64 floor)
        assert np.max(np.abs(its - its2)) <= 1


def test_gmres_restart_and_recycle_paths(built):
    """A shallow basis forces restarts at the depth and preconditioner resets
    between energies; the result still matches the oracle."""
    _, O = built
    w, P = problem("small", O, seed=10)
    E = np.array([2.0, 2.2, 2.4, 6.0, 6.1, 14.0])
    ctx = capi.Context(w)
    try:
        ore, oim, rel, its = ctx.gmres(E, depth=5, tol=1e-20, max_restarts=2000)
    finally:
        ctx.close()
    rc, ore2, oim2, rel2, its2, tot = P.gmres(E, depth=5, ffff=1e-20, max_restarts=2000)
    assert rc == 0
    assert np.max(np.abs(oim - oim2) / np.abs(oim2)) < 1e-8
    assert np.max(np.abs(ore - ore2) / np.abs(ore2)) < 1e-8


# ------------------------------------------------------------- mixed precision
# Split-BF16 tensor-core contractions keep ~16 significant bits per product and
# accumulate in FP32: H*psi is expected within 1e-4 relative of the FP64 oracle,
# and Haydock spectra within the 1e-4 relative spectral error the path targets.

@pytest.mark.parametrize("name", ["tiny", "small", "c1", "c3small"])
def test_apply_H_mixed_matches_oracle(built, name):
    _, O = built
    w, P = problem(name, O, seed=4)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        rng = np.random.default_rng(13)
        pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
        hr, hi = ctx.apply_H(pr, pi)
        orr, oi = P.xact(pr, pi)
        assert _rel(hr + 1j * hi, orr + 1j * oi) < 1e-4
        # the long-range part alone (E and multiplet off) still agrees
        hf = (1, 1, 1, 1, 0, 0)
        r1, i1 = ctx.apply_H(pr, pi, hflag=hf)
        r0, i0 = ctx.apply_H(pr, pi, hflag=(0, 1, 1, 1, 0, 0))
        o1r, o1i = P.xact(pr, pi, hflag=hf)
        o0r, o0i = P.xact(pr, pi, hflag=(0, 1, 1, 1, 0, 0))
        lr_gpu = (r1 - r0) + 1j * (i1 - i0)
        lr_ref = (o1r - o0r) + 1j * (o1i - o0i)
        assert _rel(lr_gpu, lr_ref) < 2e-4
    finally:
        ctx.close()


def test_haydock_mixed_spectrum_error(built):
    _, O = built
    w, P = problem("c1", O, seed=7)
    niter = 200
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        ra, ia, rb, done = ctx.haydock(niter)
    finally:
        ctx.close()
    rc, ora, oia, orb, _ = P.haydock(niter)
    assert done == niter and rc == 0
    assert np.max(np.abs(ra[:5] - ora[:5]) / np.abs(ora[:5])) < 1e-4
    sg = capi.spectrum_cf(ra, ia, rb, niter, w.kpref, w.el, w.eh, 2000, w.gam0)
    so = O.write_core(ora, oia, orb, niter, w.kpref, w.el, w.eh, 2000, w.gam0)
    assert _rel(sg[:, 2], so[:, 2]) < 1e-4


@pytest.mark.parametrize("lanes", [1, 2])
def test_gmres_mixed_matches_oracle(built, lanes):
    """Mixed precision (split-BF16 action, double-float Gram dots) against the
    FP64 oracle: every energy within 1e-4 relative."""
    _, O = built
    w, P = problem("small", O, seed=9)
    E = np.array([4.0, 4.1, 4.2, 8.0])
    # |g|^2 threshold above the floor set by the split-BF16 action (~1e-11 here)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=2)
    try:
        ctx.set_gmres_lanes(lanes)
        ore, oim, rel, its = ctx.gmres(E, depth=16, tol=1e-9, max_restarts=200)
    finally:
        ctx.close()
    rc, ore2, oim2, rel2, its2, tot = P.gmres(E, depth=16, ffff=1e-14, max_restarts=200)
    assert rc == 0
    assert np.max(np.abs(oim - oim2) / np.abs(oim2)) < 1e-4
    assert np.max(np.abs(ore - ore2) / np.abs(ore2)) < 1e-4


@pytest.mark.parametrize("name", ["c3small"])
def test_multiplet_mixed_tensor_core_term(built, name):
    """The multiplet term alone (long range off): split-BF16 tcgen05 projector
    contractions with the FP64 direct/exchange matrices, against the oracle."""
    _, O = built
    w, P = problem(name, O, seed=6)
    rng = np.random.default_rng(17)
    pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        m1 = (0, 1, 1, 1, 1, 0)
        m0 = (0, 1, 1, 1, 0, 0)
        r1, i1 = ctx.apply_H(pr, pi, hflag=m1)
        r0, i0 = ctx.apply_H(pr, pi, hflag=m0)
        o1r, o1i = P.xact(pr, pi, hflag=m1)
        o0r, o0i = P.xact(pr, pi, hflag=m0)
        got = (r1 - r0) + 1j * (i1 - i0)
        ref = (o1r - o0r) + 1j * (o1i - o0i)
        assert np.linalg.norm(ref) > 0
        assert _rel(got, ref) < 2e-4
    finally:
        ctx.close()


@pytest.mark.parametrize("name", ["tiny", "small", "c3small"])
def test_spin_polarised_fp64_matches_oracle(built, name):
    """nspn = 2: every term picks the Bloch functions / projectors of the
    valence spin alpha mod 2 (long_range.f90:788-801, OCEAN_multiplet.f90)."""
    _, O = built
    w, P = problem(name, O, seed=11, nspn=2)
    rng = np.random.default_rng(3)
    pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
    ctx = capi.Context(w)
    try:
        hr, hi = ctx.apply_H(pr, pi)
        ra, ia, rb, done = ctx.haydock(20)
    finally:
        ctx.close()
    orr, oi = P.xact(pr, pi)
    assert _rel(hr + 1j * hi, orr + 1j * oi) < 1e-12
    rc, ora, oia, orb, _ = P.haydock(20)
    assert rc == 0 and done == 20
    assert np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10])) < 1e-12


@pytest.mark.parametrize("name", ["small", "c3small"])
def test_spin_polarised_mixed_matches_oracle(built, name):
    """nspn = 2 on the tensor cores: one contraction per valence spin, each
    writing the channels of its spin, for the long-range and multiplet terms."""
    _, O = built
    w, P = problem(name, O, seed=11, nspn=2)
    rng = np.random.default_rng(4)
    pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        hr, hi = ctx.apply_H(pr, pi)
        ra, ia, rb, done = ctx.haydock(30)
    finally:
        ctx.close()
    orr, oi = P.xact(pr, pi)
    assert _rel(hr + 1j * hi, orr + 1j * oi) < 1e-4
    rc, ora, oia, orb, _ = P.haydock(30)
    sg = capi.spectrum_cf(ra, ia, rb, 30, w.kpref, w.el, w.eh, 500, w.gam0)
    so = O.write_core(ora, oia, orb, 30, w.kpref, w.el, w.eh, 500, w.gam0)
    assert _rel(sg[:, 2], so[:, 2]) < 1e-4
