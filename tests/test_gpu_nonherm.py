"""Non-Hermitian Haydock (ocn_haydock_nonherm, the two-sided Lanczos of
OCEAN_haydock_nonHerm_do) against the oracle's restatement, and its spectrum.

H is made non-Hermitian by a lifetime Sigma'' on the band energies.

Tolerances
  * FP64 coefficients vs oracle: first 10 a, b, c relative < 1e-11
  * GPU continued fraction (complex b, c) vs oracle write_core: 1e-12 relative
  * Hermitian problem: two-sided spectrum vs the Haydock spectrum: 1e-9
  * mixed precision vs FP64 spectra (Spect(0)): 1e-4 relative
"""
import dataclasses

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    return capi.load(lib_built), oracle_lib


def _nonherm(name, seed=5):
    w = WL.make(name, seed=1)
    rng = np.random.default_rng(seed)
    return dataclasses.replace(w, ei=rng.uniform(0.005, 0.05, w.npsi))


def _spec(co, n, w, ne=400):
    return capi.spectrum_cf_bc(*co, n, w.kpref, w.el, w.eh, ne, w.gam0)


@pytest.mark.parametrize("name", ["tiny", "c3small"])
def test_fp64_coefficients_match_oracle(built, name):
    _, O = built
    w = _nonherm(name)
    ctx = capi.Context(w, precision=capi.OCN_PREC_FP64)
    try:
        co, done = ctx.haydock_nonherm(24)
    finally:
        ctx.close()
    assert done == 24
    rc, oc, odone = O.OracleProblem(w).haydock_nonherm(24)
    assert rc == 0
    a = co[0][:10] + 1j * co[1][:10]
    oa = oc[0][:10] + 1j * oc[1][:10]
    assert np.max(np.abs(a - oa) / np.abs(oa)) < 1e-11
    for k in (2, 4):  # b, c
        g = co[k][1:11] + 1j * co[k + 1][1:11]
        o = oc[k][1:11] + 1j * oc[k + 1][1:11]
        assert np.max(np.abs(g - o) / np.abs(o)) < 1e-11
    s_gpu = _spec(co, 24, w)
    s_or = O.write_core_bc(*oc, 24, w.kpref, w.el, w.eh, 400, w.gam0)
    s_same = _spec(oc, 24, w)  # the GPU continued fraction on the oracle's coefficients
    assert np.max(np.abs(s_same[:, 2] - s_or[:, 2])) < 1e-12 * np.abs(s_or[:, 2]).max()
    assert np.linalg.norm(s_gpu[:, 2] - s_or[:, 2]) < 1e-9 * np.linalg.norm(s_or[:, 2])


def test_hermitian_problem_gives_the_haydock_spectrum(built):
    w = WL.make("c1", seed=3)
    ctx = capi.Context(w, precision=capi.OCN_PREC_FP64)
    try:
        co, done = ctx.haydock_nonherm(40)
        ra, ia, rb, hdone = ctx.haydock(40)
    finally:
        ctx.close()
    s2 = _spec(co, 40, w)
    s1 = capi.spectrum_cf(ra, ia, rb, 40, w.kpref, w.el, w.eh, 400, w.gam0)
    assert np.linalg.norm(s2[:, 2] - s1[:, 2]) < 1e-9 * np.linalg.norm(s1[:, 2])


@pytest.mark.parametrize("name", ["c1", "c3small"])
def test_mixed_precision_spectrum(built, name):
    """Mixed precision against FP64; with nvec = 2 the mixed path applies H and
    H^dagger as one block (one read of the operator data)."""
    w = _nonherm(name)
    out = {}
    for key, prec, nvec in (("fp64", capi.OCN_PREC_FP64, 1), ("mixed", capi.OCN_PREC_MIXED, 1),
                            ("pair", capi.OCN_PREC_MIXED, 2)):
        ctx = capi.Context(w, precision=prec, nvec=nvec)
        try:
            co, done = ctx.haydock_nonherm(60)
        finally:
            ctx.close()
        assert done == 60
        out[key] = _spec(co, 60, w)[:, 2]
    ref = out["fp64"]
    assert np.linalg.norm(out["mixed"] - ref) < 1e-4 * np.linalg.norm(ref)
    assert np.linalg.norm(out["pair"] - ref) < 1e-4 * np.linalg.norm(ref)
    assert np.linalg.norm(out["pair"] - out["mixed"]) < 1e-5 * np.linalg.norm(ref)
