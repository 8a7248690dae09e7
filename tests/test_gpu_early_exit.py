"""Haydock early exit (haydockconv.ipt; OCEAN_haydock.f90:268-292 with
check_convergence :1608-1661 and calc_spect_core :1991-2027) on the GPU
against the oracle's restatement.

  * FP64: the run stops at the same iteration as the oracle's early-exit run,
    with first-10 coefficients within 1e-12 and the spectra of the stopped runs
    within 1e-10; the threshold is taken between two of the oracle's relArea
    values so that the stop is not decided by rounding
  * mixed: the stopping iteration within +-2 of the oracle's (relArea moves by
    ~1e-7 with the split-BF16 action), spectra within 1e-4
  * off (threshold 0) runs all iterations
"""
import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

NITER, SPACING, NE = 150, 5, 400


@pytest.fixture(scope="module")
def case(lib_built, oracle_lib):
    capi.load(lib_built)
    O = oracle_lib
    w = WL.make("c1", seed=21)
    P = O.OracleProblem(w)
    # the oracle's relArea of every step, from a plain run, picks a threshold met part-way
    rc, ra, ia, rb, done = P.haydock(NITER)
    rels = np.zeros(NITER + 1)
    for it in range(SPACING + 1, NITER + 1):
        rels[it] = O.check_convergence(ra, ia, rb, it, it - SPACING, w.kpref, w.el, w.eh, NE, w.gam0)[1]
    srt = np.sort(rels[SPACING + 1:])
    thr = None
    for q in (0.3, 0.4, 0.5, 0.6):  # midway between two sorted values, far from either
        i = int(q * len(srt))
        cand = 0.5 * (srt[i] + srt[i + 1])
        stop = O.early_exit_iter(rels, NITER, SPACING, cand)
        if SPACING + 10 < stop < NITER - 10 and min(np.abs(rels[SPACING + 1:] - cand)) > 1e-6 * cand:
            thr = cand
            break
    assert thr is not None
    rc, ora, oia, orb, odone, orel = P.haydock_conv(NITER, thr, SPACING, NE)
    assert rc == 0 and odone == stop
    return w, O, thr, (ora, oia, orb, odone)


@pytest.mark.parametrize("prec", [capi.OCN_PREC_FP64, capi.OCN_PREC_MIXED])
def test_early_exit_matches_oracle(case, prec):
    w, O, thr, (ora, oia, orb, odone) = case
    ctx = capi.Context(w, precision=prec)
    try:
        ctx.set_haydock_conv(thr, SPACING, NE)
        ra, ia, rb, done = ctx.haydock(NITER)
        # the same context with the test off runs every step
        ctx.set_haydock_conv(0.0)
        _, _, _, done_off = ctx.haydock(NITER)
    finally:
        ctx.close()
    assert done_off == NITER
    if prec == capi.OCN_PREC_FP64:
        assert done == odone
        assert np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
    else:
        assert abs(done - odone) <= 2
    assert np.all(ra[done:] == 0.0) and np.all(rb[done + 1:] == 0.0)
    n = min(done, odone)
    sg = capi.spectrum_cf(ra, ia, rb, n, w.kpref, w.el, w.eh, 2000, w.gam0)
    so = O.write_core(ora, oia, orb, n, w.kpref, w.el, w.eh, 2000, w.gam0)
    err = np.linalg.norm(sg[:, 2] - so[:, 2]) / np.linalg.norm(so[:, 2])
    assert err < (1e-10 if prec == capi.OCN_PREC_FP64 else 1e-4)
