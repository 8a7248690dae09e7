"""Adjoint GMRES gradients (ocn_gmres_vjp + ocn_w2_vjp through GmresSpectrum)
against central finite differences, of this library and of the oracle's GMRES.

The loss is L = sum_w c_w out_im(w) + d_w out_re(w) with fixed random c, d.
Parameters: interactionScale (W scale), the 64-sample W(r) table (checked
along a random direction), Gamma and a scissor shift.  Central differences
use a step of 1e-4 relative to the parameter; the scissor, an energy like
Gamma, takes the step 1e-4 Gamma (an absolute 1e-4 Hartree would be ~1% of
Gamma and leave ~1e-4 truncation error).  GMRES runs converge to
|g|^2 < 1e-20, so the difference quotient carries O(h^2) ~ 1e-8 truncation
and ~1e-7 solver noise.

Tolerances
  * FP64 adjoint vs FD of this library:   2e-5 relative
  * FP64 adjoint vs FD of the oracle:     2e-5 relative
  * mixed-precision adjoint vs FP64 adjoint: 2e-3 relative
"""
import dataclasses

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

pytestmark = pytest.mark.gpu

TOL_G2 = 1e-20
GAMMA = 0.3 * WL.EV2HARTREE


@pytest.fixture(scope="module")
def built(lib_built, oracle_lib):
    import torch  # noqa: F401

    return capi.load(lib_built), oracle_lib


def _setup(name, nomega, seed=3):
    w = WL.make(name, seed=seed)
    E = np.linspace(w.el + 0.1 * (w.eh - w.el), w.eh - 0.3 * (w.eh - w.el), nomega) * WL.HARTREE2EV
    rng = np.random.default_rng(seed + 100)
    c, d = rng.standard_normal(nomega), rng.standard_normal(nomega)
    v = rng.standard_normal(len(w.ptab))
    v *= 1e-4 * np.max(np.abs(w.ptab)) / np.max(np.abs(v))
    return w, E, c, d, v


def _loss(ore, oim, c, d):
    return float(np.dot(c, oim) + np.dot(d, ore))


def _autograd(prob, w, c, d):
    import torch

    from ocean_gb300 import adjoint

    scale = torch.tensor(w.interaction_scale, dtype=torch.float64, requires_grad=True)
    ptab = torch.tensor(w.ptab, dtype=torch.float64, requires_grad=True)
    gamma = torch.tensor(GAMMA, dtype=torch.float64, requires_grad=True)
    sc = torch.tensor(0.0, dtype=torch.float64, requires_grad=True)
    ore, oim = adjoint.gmres_spectrum(prob, scale, ptab, gamma, sc)
    L = (torch.from_numpy(c) * oim).sum() + (torch.from_numpy(d) * ore).sum()
    L.backward()
    return float(L.detach()), {"scale": float(scale.grad), "ptab": ptab.grad.numpy().copy(), "gamma": float(gamma.grad),
                      "scissor": float(sc.grad)}


def _eval_lib(prob, w, E, c, d, scale, ptab, gamma, scissor):
    prob.set_parameters(scale, ptab, scissor)
    ore, oim, rel, its = prob.ctx.gmres_dev(prob.d_hay.data_ptr(), E, resolution=gamma, **prob.kw)
    return _loss(ore, oim, c, d)


def _eval_oracle(O, w, E, c, d, scale, ptab, gamma, scissor):
    wv = dataclasses.replace(w, ptab=np.ascontiguousarray(ptab), interaction_scale=scale, er=w.er + scissor)
    P = O.OracleProblem(wv)
    rc, ore, oim, rel, its, tot = P.gmres(E, depth=40, gres=gamma, ffff=TOL_G2, max_restarts=400)
    assert rc == 0
    return _loss(ore, oim, c, d)


def _fd(f, w, v):
    """central differences of f(scale, ptab, gamma, scissor) at the base point"""
    s0, p0 = w.interaction_scale, np.asarray(w.ptab, dtype=np.float64)
    hs, hg, hc = 1e-4 * s0, 1e-4 * GAMMA, 1e-4 * GAMMA
    return {
        "scale": (f(s0 + hs, p0, GAMMA, 0.0) - f(s0 - hs, p0, GAMMA, 0.0)) / (2 * hs),
        "ptab_dir": (f(s0, p0 + v, GAMMA, 0.0) - f(s0, p0 - v, GAMMA, 0.0)) / 2.0,
        "gamma": (f(s0, p0, GAMMA + hg, 0.0) - f(s0, p0, GAMMA - hg, 0.0)) / (2 * hg),
        "scissor": (f(s0, p0, GAMMA, hc) - f(s0, p0, GAMMA, -hc)) / (2 * hc),
    }


def _compare(g, fd, v, tol):
    got = {"scale": g["scale"], "ptab_dir": float(np.dot(g["ptab"], v)), "gamma": g["gamma"],
           "scissor": g["scissor"]}
    errs = {k: abs(got[k] - fd[k]) / max(abs(fd[k]), 1e-300) for k in fd}
    assert all(e < tol for e in errs.values()), (errs, got, fd)


def test_adjoint_matches_library_finite_differences(built):
    from ocean_gb300 import adjoint

    w, E, c, d, v = _setup("c1", 4)
    prob = adjoint.GmresProblem(w, E, depth=40, tol=TOL_G2, max_restarts=400)
    try:
        L, g = _autograd(prob, w, c, d)
        fd = _fd(lambda s, p, gm, sc: _eval_lib(prob, w, E, c, d, s, p, gm, sc), w, v)
        L0 = _eval_lib(prob, w, E, c, d, w.interaction_scale, w.ptab, GAMMA, 0.0)
    finally:
        prob.close()
    assert abs(L - L0) <= 1e-12 * abs(L0)
    _compare(g, fd, v, 2e-5)


def test_adjoint_matches_oracle_finite_differences(built):
    _, O = built
    from ocean_gb300 import adjoint

    w, E, c, d, v = _setup("tiny", 3, seed=5)
    prob = adjoint.GmresProblem(w, E, depth=40, tol=TOL_G2, max_restarts=400)
    try:
        _, g = _autograd(prob, w, c, d)
    finally:
        prob.close()
    fd = _fd(lambda s, p, gm, sc: _eval_oracle(O, w, E, c, d, s, p, gm, sc), w, v)
    _compare(g, fd, v, 2e-5)


def test_adjoint_mixed_agrees_with_fp64(built):
    from ocean_gb300 import adjoint

    w, E, c, d, v = _setup("c1", 3, seed=8)
    grads = []
    for prec, tol in ((capi.OCN_PREC_FP64, 1e-16), (capi.OCN_PREC_MIXED, 1e-10)):
        prob = adjoint.GmresProblem(w, E, precision=prec, depth=40, tol=tol, max_restarts=400)
        try:
            grads.append(_autograd(prob, w, c, d)[1])
        finally:
            prob.close()
    g64, gmx = grads
    for k in ("scale", "gamma", "scissor"):
        assert abs(gmx[k] - g64[k]) < 2e-3 * abs(g64[k]), (k, gmx[k], g64[k])
    assert np.linalg.norm(gmx["ptab"] - g64["ptab"]) < 2e-3 * np.linalg.norm(g64["ptab"])


def test_vjp_rejects_unsupported_terms(built):
    import torch

    w = WL.make("c3small", seed=1)
    ctx = capi.Context(w)
    try:
        n = w.npsi
        d = torch.zeros(2 * n * 2, dtype=torch.float64, device="cuda:0")
        gW = torch.zeros(w.nk * w.nx, dtype=torch.float64, device="cuda:0")
        with pytest.raises(capi.OcnError) as e:
            ctx.gmres_vjp(d.data_ptr(), [5.0], d.data_ptr(), gW.data_ptr(), grad_im=[1.0])
        assert e.value.code == 9962
    finally:
        ctx.close()


def test_windowed_recomputation_gives_the_stored_gradient(built):
    """With a memory cap below the solutions' size the energies are taken in
    windows, forward keeps nothing and backward solves each window again: the
    spectrum and every gradient equal, bit for bit, those of the same windows
    with the solutions stored."""
    from ocean_gb300 import adjoint

    w, E, c, d, v = _setup("tiny", 7, seed=8)
    per_x = 2 * w.npsi * 8
    kw = dict(depth=24, tol=TOL_G2, max_restarts=400)
    stored = adjoint.GmresProblem(w, E, window=3, **kw)
    recomp = adjoint.GmresProblem(w, E, max_stored_bytes=3.5 * per_x, **kw)
    try:
        assert (stored.recompute, stored.window) == (False, 3)
        assert (recomp.recompute, recomp.window) == (True, 3)
        L1, g1 = _autograd(stored, w, c, d)
        L2, g2 = _autograd(recomp, w, c, d)
    finally:
        stored.close()
        recomp.close()
    assert L1 == L2
    assert g1["scale"] == g2["scale"] and g1["gamma"] == g2["gamma"] and g1["scissor"] == g2["scissor"]
    assert np.array_equal(g1["ptab"], g2["ptab"])
    # and the windowed gradient is the gradient: central differences of the library
    prob = adjoint.GmresProblem(w, E, **kw)
    try:
        fd = _fd(lambda *a: _eval_lib(prob, w, E, c, d, *a), w, v)
    finally:
        prob.close()
    _compare(g2, fd, v, 2e-5)
