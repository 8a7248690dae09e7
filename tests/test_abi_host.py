"""CPU tests of the C-ABI library: it builds for sm_103a, loads, exports every
entry point declared in include/ocean_gpu.h, validates arguments, and its
host-side index bookkeeping (xshift, W table, core-hole phase) is bit-identical
to the oracle's restatement of OCEAN_bloch_lrLOAD and lr_populate_W2."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from ocean_gb300 import capi
from ocean_gb300 import workloads as WL

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ocean_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|double|const char\*|long long|void\*)\s+(ocn_\w+)\(", txt,
                                 re.M)))


def test_library_exports_every_declared_symbol(lib_built):
    lib = capi.load(lib_built)
    syms = header_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(capi.EXPORTS) == syms
    assert b"sm_103a" in lib.ocn_version()


def test_product_never_touches_the_oracle():
    for dirpath, _, files in os.walk(os.path.join(ROOT, "ocean_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "liboracle" not in txt and "import oracle" not in txt, f


def test_create_rejects_bad_dims_without_gpu(lib_built):
    lib = capi.load(lib_built)
    w = WL.make("tiny")
    for field, val in [("nalpha", 5), ("num_bands", 0), ("nspn", 3), ("core_l", 2), ("precision", 7)]:
        d = capi._dims(w)
        setattr(d, field, val)
        ptr = C.c_void_p()
        rc = lib.ocn_ctx_create(C.byref(d), C.byref(ptr))
        assert rc == 1 and not ptr.value, field
        assert capi.last_error()
    d = capi._dims(w)
    d.kmesh[0] = 40
    ptr = C.c_void_p()
    assert lib.ocn_ctx_create(C.byref(d), C.byref(ptr)) == 1
    assert lib.ocn_ctx_create(None, C.byref(ptr)) == 1


def _oracle_w(O, w):
    P_d = O.dims_of(w)
    tau = (C.c_double * 3)(*list(w.tau))
    xs = (C.c_int * 3)()
    O.lib().or_lrload(C.byref(P_d), tau, (C.c_int * 3)(1, 1, 1), xs, None, None)
    lr = O.lr_in_of(w)
    W = np.zeros(w.nk * w.nx)
    O.lib().or_populate_w2(C.byref(P_d), C.byref(lr), tau, xs, O.dptr(W))
    return W, tuple(xs), tuple(tau)


@pytest.mark.parametrize("case", [
    dict(name="tiny", tau=(0.0, 0.0, 0.0)),
    dict(name="c1", tau=(0.0, 0.0, 0.0)),
    dict(name="tiny", kmesh=(3, 4, 5), xmesh=(5, 4, 3), tau=(0.31, 0.77, 0.05)),
    dict(name="tiny", kmesh=(1, 2, 3), xmesh=(6, 6, 2), tau=(0.9, 0.5, 0.49)),
])
def test_w2_and_xshift_bit_exact(lib_built, oracle_lib, case):
    kw = {k: v for k, v in case.items() if k in ("kmesh", "xmesh")}
    w = WL.make(case["name"], seed=0, **kw)
    w.tau = np.array(case["tau"], dtype=float)
    W, xs, tau = capi.w2_host(w)
    Wo, xso, tauo = _oracle_w(oracle_lib, w)
    assert xs == xso and tau == tauo
    assert np.array_equal(W, Wo)
    assert np.all(np.isfinite(W)) and W.min() > 0


def test_w2_isolated_and_eps3d_bit_exact(lib_built, oracle_lib):
    w = WL.make("tiny", seed=0, kmesh=(4, 3, 2), xmesh=(4, 4, 4))
    w.tau = np.array([0.2, 0.6, 0.1])
    p, keep = capi._lr_params(w)
    p.isolated, p.iso_cut = 1, 9.0
    p.have_eps3d = 1
    p.epsilon3d[:] = [3.0, 4.5, 6.0]
    p.pbc[:] = [1, 0, 1]
    d = capi._dims(w)
    W = np.zeros(w.nk * w.nx)
    xs = (C.c_int * 3)()
    tau = (C.c_double * 3)()
    capi.check(capi.load().ocn_w2_host(C.byref(d), C.byref(p), capi._dp(W), xs, tau))
    O = oracle_lib
    lr = O.lr_in_of(w)
    lr.isolated, lr.iso_cut, lr.have_eps3d = 1, 9.0, 1
    lr.epsilon3d[:] = [3.0, 4.5, 6.0]
    lr.pbc[:] = [1, 0, 1]
    Wo = np.zeros_like(W)
    O.lib().or_populate_w2(C.byref(O.dims_of(w)), C.byref(lr), tau, xs, O.dptr(Wo))
    assert np.array_equal(W, Wo)
    assert (W == 0).any()  # isolated cut and pbc prefactor both zero some entries


@pytest.mark.parametrize("kmesh,xmesh,tau", [((4, 4, 4), (8, 8, 8), (0.0, 0.0, 0.0)),
                                             ((3, 2, 5), (4, 6, 3), (0.4, 0.1, 0.8))])
def test_phase_table_bit_exact(lib_built, oracle_lib, kmesh, xmesh, tau):
    w = WL.make("tiny", seed=0, kmesh=kmesh, xmesh=xmesh)
    w.tau = np.array(tau)
    _, xs, _ = capi.w2_host(w)
    c, s = capi.phase_table_host(w, xs)
    # oracle: phase applied to u = 1 + 0i reproduces cos/sin exactly
    O = oracle_lib
    n = w.nb * w.nk * w.nx
    ur, ui = np.ones(n), np.zeros(n)
    t = (C.c_double * 3)(*tau)
    xo = (C.c_int * 3)()
    O.lib().or_lrload(C.byref(O.dims_of(w)), t, (C.c_int * 3)(1, 1, 1), xo, O.dptr(ur), O.dptr(ui))
    assert tuple(xo) == xs
    # u(n,k,x): band fastest; the table is per (x,k)
    assert np.array_equal(ur.reshape(w.nx, w.nk, w.nb)[:, :, 0].reshape(-1), c)
    assert np.array_equal(ui.reshape(w.nx, w.nk, w.nb)[:, :, 0].reshape(-1), s)


def test_redtrid_matches_golden(lib_built):
    d = np.load(os.path.join(ROOT, "tests", "golden", "cu_twophoton_kat.npz"))
    n = int(d["p2_n"])
    w = capi.redtrid(n, d["p2_real_a"], d["p2_real_b"])
    assert np.abs(w - d["p2_eig"]).max() < 6e-11


def test_pnorm_matches_reference_formula(lib_built):
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(100), rng.standard_normal(100)
    r, i, kp = capi.pnorm(a, b, 64, 432.0)
    r2, i2, kp2 = WL.pnorm(a, b, 64, 432.0)
    assert np.allclose(r, r2, rtol=1e-15) and abs(kp - kp2) < 1e-15 * kp


def test_w2_vjp_is_the_exact_chain_rule_of_w2(lib_built):
    """ocn_w2_vjp against finite differences of ocn_w2_host: W is linear in the
    W(r) table and in interactionScale, so central differences are exact up to
    rounding."""
    import dataclasses

    from ocean_gb300 import capi
    from ocean_gb300 import workloads as WL

    capi.load(lib_built)
    w = WL.make("c1", seed=2)
    rng = np.random.default_rng(7)
    G = rng.standard_normal(w.nk * w.nx)
    gp, gs = capi.w2_vjp(w, G)

    def L(ptab, scale):
        W, _, _ = capi.w2_host(dataclasses.replace(w, ptab=np.ascontiguousarray(ptab), interaction_scale=scale))
        return float(np.dot(G, W))

    p0 = np.asarray(w.ptab, dtype=np.float64)
    for m in (0, 1, 17, len(p0) - 1):
        e = np.zeros_like(p0)
        e[m] = 1e-3
        fd = (L(p0 + e, 1.0) - L(p0 - e, 1.0)) / 2e-3
        assert abs(gp[m] - fd) <= 1e-9 * max(1.0, abs(fd)), (m, gp[m], fd)
    fd_s = (L(p0, 1.0 + 1e-3) - L(p0, 1.0 - 1e-3)) / 2e-3
    assert abs(gs - fd_s) <= 1e-9 * abs(fd_s)
    # entries beyond the table (the 1/(eps r) tail) do not depend on it
    assert np.count_nonzero(gp) <= len(p0)
