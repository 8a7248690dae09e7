"""ocn_spectrum_cf_noalloc (static device scratch, no allocation) against
ocn_spectrum_cf on the same inputs, through the C ABI.

Both run the same write_core kernel on the same coefficients, so the spectra
agree to 1e-14 relative (in practice bit for bit).  Calls come in pairs so that
the second call of a pair reads the scratch left behind by the first.
This file is collected last so that it also runs after every other GPU test.
"""
import os

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-14
MAX_ITER, MAX_NE = 4096, 8192  # OCN_CF_NOALLOC_MAX_ITER, OCN_CF_NOALLOC_MAX_NE


def _close(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def _kat(photon):
    d = np.load(os.path.join(ROOT, "tests", "golden", "cu_twophoton_kat.npz"))
    p = f"p{photon}"
    return (d[p + "_real_a"], d[p + "_real_b"], int(d[p + "_n"]), float(d[p + "_kpref"]),
            float(d[p + "_vol"]))


def test_noalloc_matches_spectrum_cf_twice_in_a_row(lib_built):
    capi.load(lib_built)
    el, eh, gam0 = -30.0 * WL.EV2HARTREE, 70.0 * WL.EV2HARTREE, 1.245 * WL.EV2HARTREE
    for photon in (1, 2):
        ra, rb, n, kpref, vol = _kat(photon)
        ref = capi.spectrum_cf(ra, None, rb, n, kpref, el, eh, 5000, gam0, ucvol=vol)
        first = capi.spectrum_cf_noalloc(ra, None, rb, n, kpref, el, eh, 5000, gam0, ucvol=vol)
        second = capi.spectrum_cf_noalloc(ra, None, rb, n, kpref, el, eh, 5000, gam0, ucvol=vol)
        assert _close(first, ref) < TOL
        assert _close(second, ref) < TOL
    # a shorter fraction after a longer one, with imaginary a and the gamfcn column
    ra, rb, n, kpref, vol = _kat(3)
    ia = np.linspace(0.0, 1e-3, n + 1)
    for it in (n, 40):
        kw = dict(ucvol=vol, old_broaden=1, nval=0.2, eps=5.0, ebase=8979.0)
        ref = capi.spectrum_cf(ra, ia, rb, it, kpref, el, eh, 1000, gam0, **kw)
        got = capi.spectrum_cf_noalloc(ra, ia, rb, it, kpref, el, eh, 1000, gam0, **kw)
        assert _close(got, ref) < TOL


def test_noalloc_at_its_size_limits(lib_built):
    capi.load(lib_built)
    rng = np.random.default_rng(5)
    ra = rng.uniform(-0.5, 0.5, MAX_ITER + 1)
    rb = rng.uniform(0.05, 0.4, MAX_ITER + 1)
    rb[0] = 0.0
    args = (ra, None, rb, MAX_ITER, 1.3, -0.8, 1.6, MAX_NE, 0.02)
    ref = capi.spectrum_cf(*args)
    for _ in range(2):
        assert _close(capi.spectrum_cf_noalloc(*args), ref) < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch(lib_built):
    capi.load(lib_built)
    ra = np.zeros(MAX_ITER + 2)
    rb = np.full(MAX_ITER + 2, 0.1)
    with pytest.raises(capi.OcnError) as e:
        capi.spectrum_cf_noalloc(ra, None, rb, MAX_ITER + 1, 1.0, -1.0, 1.0, 100, 0.02)
    assert e.value.code == capi.OCN_ERR_ARG and "scratch limit" in str(e.value)
    with pytest.raises(capi.OcnError) as e:
        capi.spectrum_cf_noalloc(ra, None, rb, 10, 1.0, -1.0, 1.0, MAX_NE + 1, 0.02)
    assert e.value.code == capi.OCN_ERR_ARG and "scratch limit" in str(e.value)
    # still usable after the rejected calls
    ref = capi.spectrum_cf(ra, None, rb, 10, 1.0, -1.0, 1.0, 100, 0.02)
    assert _close(capi.spectrum_cf_noalloc(ra, None, rb, 10, 1.0, -1.0, 1.0, 100, 0.02), ref) < TOL
