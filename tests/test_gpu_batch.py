"""Batched Haydock over independent, unevenly sized problems (ocn_haydock_batch).

All contexts stay alive together (different k-meshes, band counts, edges and
precisions), their three-iteration graphs run as branches of one graph, and each
context must produce exactly what it produces on its own (bit for bit: the same
kernels in the same order per context), which in turn matches the oracle.

Tolerances
  * batch vs the same context run alone: bit-identical
  * FP64 chains vs oracle: first 10 a_n relative < 1e-12
  * mixed chains vs oracle: spectra (Spect(0)) relative < 1e-4
"""
import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

SHAPES = [  # (nb, kmesh n, xmesh m, core_l, precision, chains)
    (12, 2, 4, 0, capi.OCN_PREC_MIXED, 2),
    (16, 3, 4, 1, capi.OCN_PREC_MIXED, 3),
    (20, 4, 5, 0, capi.OCN_PREC_MIXED, 3),
    (10, 5, 4, 0, capi.OCN_PREC_FP64, 1),
]


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    import torch  # noqa: F401

    return capi.load(lib_built), oracle_lib


def _starts(w, nv, seed):
    rng = np.random.default_rng(seed)
    pr, pi = np.zeros((nv, w.npsi)), np.zeros((nv, w.npsi))
    pr[0], pi[0] = w.psi_r, w.psi_i
    for v in range(1, nv):
        r, i = rng.standard_normal(w.npsi), rng.standard_normal(w.npsi)
        s = np.sqrt(np.sum(r * r + i * i))
        pr[v], pi[v] = r / s, i / s
    return pr, pi


@pytest.mark.parametrize("niter", [31, 12])
def test_batch_equals_each_context_alone_and_the_oracle(built, niter):
    import torch

    _, O = built
    ws, ctxs, bufs, starts = [], [], [], []
    try:
        for i, (nb, n, m, lc, prec, nv) in enumerate(SHAPES):
            w = WL.make("batch", seed=40 + i, nb=nb, kmesh=(n, n, n), xmesh=(m, m, m), core_l=lc)
            ctx = capi.Context(w, precision=prec, nvec=nv)
            pr, pi = _starts(w, nv, 70 + i)
            d = torch.empty(2 * w.npsi * nv, dtype=torch.float64, device="cuda:0")
            for v in range(nv):
                d[2 * v * w.npsi:(2 * v + 1) * w.npsi].copy_(torch.from_numpy(pr[v]))
                d[(2 * v + 1) * w.npsi:(2 * v + 2) * w.npsi].copy_(torch.from_numpy(pi[v]))
            ws.append(w)
            ctxs.append(ctx)
            bufs.append(d)
            starts.append((pr, pi))
        torch.cuda.synchronize()
        res = capi.haydock_batch(ctxs, [d.data_ptr() for d in bufs], [s[5] for s in SHAPES], niter)
        for i, (w, ctx, d) in enumerate(zip(ws, ctxs, bufs)):
            nv = SHAPES[i][5]
            ra, ia, rb, done = res[i]
            assert list(done) == [niter] * nv
            sra, sia, srb, sdone = ctx.haydock_block_dev(niter, nv, d.data_ptr())
            assert np.array_equal(ra, sra) and np.array_equal(rb, srb), i
            P = O.OracleProblem(w)
            for v in range(nv):
                rc, ora, oia, orb, _ = P.haydock(niter, starts[i][0][v], starts[i][1][v])
                assert rc == 0
                if SHAPES[i][4] == capi.OCN_PREC_FP64:
                    assert np.max(np.abs(ra[v, :10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
                else:
                    sg = capi.spectrum_cf(ra[v], ia[v], rb[v], niter, w.kpref, w.el, w.eh, 500, w.gam0)
                    so = O.write_core(ora, oia, orb, niter, w.kpref, w.el, w.eh, 500, w.gam0)
                    err = np.linalg.norm(sg[:, 2] - so[:, 2]) / np.linalg.norm(so[:, 2])
                    assert err < 1e-4, (i, v, err)
    finally:
        for c in ctxs:
            c.close()


def test_batch_rejects_a_context_listed_twice(built):
    import torch

    w = WL.make("tiny", seed=2)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED)
    try:
        d = torch.zeros(2 * w.npsi, dtype=torch.float64, device="cuda:0")
        with pytest.raises(capi.OcnError) as e:
            capi.haydock_batch([ctx, ctx], [d.data_ptr(), d.data_ptr()], [1, 1], 6)
        assert e.value.code == capi.OCN_ERR_ARG
    finally:
        ctx.close()
