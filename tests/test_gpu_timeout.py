"""The bounded waits of the tensor-core contractions, made to run out on purpose.

With the test hook on, the contraction kernels' load warp issues no loads: the
MMA warp's wait on the first full stage (bounded at about one second) is never
satisfied, so the kernel records the expiry, issues nothing further, frees its
tensor memory and returns.  Nothing is in flight when the CTAs exit.  The call
must report OCN_ERR_TIMEOUT, and the same context must then give the correct
action (against the oracle, relative 2-norm < 1e-4) and the same bits as before.
"""
import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

OCN_ERR_TIMEOUT = 5


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    return capi.load(lib_built), oracle_lib


def test_starved_contraction_reports_timeout_and_context_recovers(built):
    _, O = built
    w = WL.make("tiny", seed=3)
    P = O.OracleProblem(w)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        rng = np.random.default_rng(5)
        pr, pi = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
        before = ctx.apply_H(pr, pi)
        ctx.starve_tc(True)
        with pytest.raises(capi.OcnError) as exc:
            ctx.apply_H(pr, pi)
        assert exc.value.code == OCN_ERR_TIMEOUT
        ctx.starve_tc(False)
        after = ctx.apply_H(pr, pi)
        assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
        orr, oi = P.xact(pr, pi)
        rel = np.linalg.norm((after[0] - orr) + 1j * (after[1] - oi)) / np.linalg.norm(orr + 1j * oi)
        assert rel < 1e-4
        # a Haydock run on the same context still works
        ra, ia, rb, done = ctx.haydock(8)
        assert done == 8 and np.all(np.isfinite(ra[:8]))
    finally:
        ctx.close()
