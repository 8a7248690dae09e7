"""Block (multi-vector) paths against the oracle and the single-vector paths.

A block of nv psi vectors shares one H: ocn_apply_H_block acts on all of them,
ocn_haydock_block runs nv independent Lanczos chains in lockstep.  Each chain
must be the reference's single-chain Haydock on its own psi0.

Tolerances
  * FP64 block chains vs single FP64 chains: bit-identical (same kernels per chain)
  * FP64 block chains vs oracle: first 10 a_n, b_n relative < 1e-12
  * mixed block H*psi vs oracle: < 1e-4 relative per vector
  * mixed block H*psi vs mixed single-vector H*psi: < 1e-6 relative
  * mixed block Haydock spectra vs oracle chains: < 1e-4 relative
"""
import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    return capi.load(lib_built), oracle_lib


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _start_vectors(w, nv, seed):
    """psi0 of chain 0 is the workload's; the others are normalised complex Gaussians."""
    rng = np.random.default_rng(seed)
    pr = np.zeros((nv, w.npsi))
    pi = np.zeros((nv, w.npsi))
    pr[0], pi[0] = w.psi_r, w.psi_i
    for v in range(1, nv):
        r, i = rng.standard_normal(w.npsi) * w.allow, rng.standard_normal(w.npsi) * w.allow
        nrm = np.sqrt(np.sum(r * r + i * i))
        pr[v], pi[v] = r / nrm, i / nrm
    return pr, pi


@pytest.mark.parametrize("name,nv", [("small", 3), ("c3small", 2)])
def test_apply_H_block_mixed(built, name, nv):
    _, O = built
    w = WL.make(name, seed=5)
    P = O.OracleProblem(w)
    rng = np.random.default_rng(21)
    pr, pi = rng.standard_normal((nv, w.npsi)), rng.standard_normal((nv, w.npsi))
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=nv)
    try:
        br, bi = ctx.apply_H_block(pr, pi)
        for v in range(nv):
            orr, oi = P.xact(pr[v], pi[v])
            assert _rel(br[v] + 1j * bi[v], orr + 1j * oi) < 1e-4
            sr, si = ctx.apply_H(pr[v], pi[v])
            assert _rel(br[v] + 1j * bi[v], sr + 1j * si) < 1e-6
        # a smaller block on the same context
        b2r, b2i = ctx.apply_H_block(pr[:1], pi[:1])
        assert _rel(b2r[0] + 1j * b2i[0], br[0] + 1j * bi[0]) < 1e-6
    finally:
        ctx.close()


def test_apply_H_block_fp64_exact(built):
    _, O = built
    w = WL.make("small", seed=6)
    P = O.OracleProblem(w)
    rng = np.random.default_rng(22)
    pr, pi = rng.standard_normal((2, w.npsi)), rng.standard_normal((2, w.npsi))
    ctx = capi.Context(w, nvec=2)
    try:
        br, bi = ctx.apply_H_block(pr, pi)
        for v in range(2):
            orr, oi = P.xact(pr[v], pi[v])
            assert _rel(br[v] + 1j * bi[v], orr + 1j * oi) < 1e-12
    finally:
        ctx.close()


@pytest.mark.parametrize("niter", [31, 60])
def test_haydock_block_fp64_equals_single_chains(built, niter):
    _, O = built
    w = WL.make("c1", seed=8)
    P = O.OracleProblem(w)
    nv = 3
    pr, pi = _start_vectors(w, nv, 31)
    ctx = capi.Context(w, nvec=nv)
    try:
        ra, ia, rb, done = ctx.haydock_block(niter, pr, pi)
        assert list(done) == [niter] * nv
        for v in range(nv):
            sra, sia, srb, sdone = ctx.haydock(niter, pr[v], pi[v])
            assert np.array_equal(ra[v], sra) and np.array_equal(rb[v], srb)
            rc, ora, oia, orb, _ = P.haydock(niter, pr[v], pi[v])
            assert rc == 0
            assert np.max(np.abs(ra[v, :10] - ora[:10]) / np.abs(ora[:10])) < 1e-12
            assert np.max(np.abs(rb[v, 1:11] - orb[1:11]) / np.abs(orb[1:11])) < 1e-12
    finally:
        ctx.close()


@pytest.mark.parametrize("name,nv,niter", [("c1", 3, 121), ("c3small", 2, 40)])
def test_haydock_block_mixed_matches_oracle_chains(built, name, nv, niter):
    _, O = built
    w = WL.make(name, seed=9)
    P = O.OracleProblem(w)
    pr, pi = _start_vectors(w, nv, 41)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=nv)
    try:
        ra, ia, rb, done = ctx.haydock_block(niter, pr, pi)
        ra2, ia2, rb2, done2 = ctx.haydock_block(niter, pr, pi)  # graph replay
        single = [ctx.haydock(niter, pr[v], pi[v]) for v in range(nv)]
    finally:
        ctx.close()
    assert list(done) == [niter] * nv
    assert np.array_equal(ra, ra2) and np.array_equal(rb, rb2)
    for v in range(nv):
        rc, ora, oia, orb, _ = P.haydock(niter, pr[v], pi[v])
        assert rc == 0
        assert np.max(np.abs(ra[v, :5] - ora[:5]) / np.abs(ora[:5])) < 1e-4
        sg = capi.spectrum_cf(ra[v], ia[v], rb[v], niter, w.kpref, w.el, w.eh, 1000, w.gam0)
        so = O.write_core(ora, oia, orb, niter, w.kpref, w.el, w.eh, 1000, w.gam0)
        assert _rel(sg[:, 2], so[:, 2]) < 1e-4
        # the lockstep chain and the single mixed chain agree to FP32 round-off
        sra = single[v][0]
        assert np.max(np.abs(ra[v, :5] - sra[:5]) / np.abs(sra[:5])) < 1e-6


def test_block_size_checked(built):
    w = WL.make("tiny", seed=1)
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=2)
    try:
        pr = np.zeros((3, w.npsi))
        with pytest.raises(capi.OcnError) as ei:
            ctx.haydock_block(6, pr, pr)
        assert ei.value.code == capi.OCN_ERR_ARG
        with pytest.raises(capi.OcnError) as ei:
            ctx.apply_H_block(pr, pr)
        assert ei.value.code == capi.OCN_ERR_ARG
        # the context still works after the rejected calls
        pr2, pi2 = _start_vectors(w, 2, 3)
        ra, ia, rb, done = ctx.haydock_block(6, pr2, pi2)
        assert list(done) == [6, 6]
    finally:
        ctx.close()


def test_output_staging_is_bit_identical(built):
    """The band->x contraction's outputs stored through shared memory (tile
    parameter 6) are the same values as stored directly."""
    for name, nv in (("c1", 2), ("c3small", 2), ("tiny", 1)):
        w = WL.make(name, seed=17)
        rng = np.random.default_rng(8)
        pr, pi = rng.standard_normal((nv, w.npsi)), rng.standard_normal((nv, w.npsi))
        ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=nv)
        try:
            t = list(ctx.tiles())
            out = []
            for stg in (0, 1):
                t[6] = stg
                ctx.set_tiles(tuple(t))
                out.append(ctx.apply_H_block(pr, pi))
        finally:
            ctx.close()
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]), name


def test_autotune_and_tilings_keep_the_action(built):
    """Every tiling of the contractions gives the same H*psi to FP32 round-off,
    and the autotuner leaves a working, reported configuration."""
    _, O = built
    w = WL.make("c1", seed=12)
    P = O.OracleProblem(w)
    rng = np.random.default_rng(5)
    pr, pi = rng.standard_normal((2, w.npsi)), rng.standard_normal((2, w.npsi))
    ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, nvec=2)
    try:
        default = ctx.tiles()
        base_r, base_i = ctx.apply_H_block(pr, pi)
        for tiles in [(2, 1, 152, 152, 0, 0, 0), (3, 4, 76, 76, 4, 256, 1), (default[0], 8, 152, 76, 0, 512, 1)]:
            ctx.set_tiles(tiles)
            assert ctx.tiles() == tiles
            r, i = ctx.apply_H_block(pr, pi)
            assert _rel(r + 1j * i, base_r + 1j * base_i) < 1e-6
        ms, best = ctx.autotune(nv=2, reps=2)
        assert ms > 0 and ctx.tiles() == best
        r, i = ctx.apply_H_block(pr, pi)
        for v in range(2):
            orr, oi = P.xact(pr[v], pi[v])
            assert _rel(r[v] + 1j * i[v], orr + 1j * oi) < 1e-4
        with pytest.raises(capi.OcnError) as e:
            ctx.set_tiles((0, 1, 1, 1, 0, 0, 0))
        assert e.value.code == capi.OCN_ERR_ARG
        # the Haydock graph is rebuilt for the new tiling
        ra, ia, rb, done = ctx.haydock_block(9, pr / np.linalg.norm(pr[0] + 1j * pi[0]),
                                             pi / np.linalg.norm(pr[0] + 1j * pi[0]))
        assert list(done) == [9, 9]
    finally:
        ctx.close()
