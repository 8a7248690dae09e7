"""ctypes bindings of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py as the checker and the CPU baseline.
The product package (ocean_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)


class OrDims(C.Structure):
    _fields_ = [("nb", C.c_int), ("kmesh", C.c_int * 3), ("xmesh", C.c_int * 3), ("na", C.c_int),
                ("nspn", C.c_int), ("core_l", C.c_int)]


class OrOps(C.Structure):
    _fields_ = [("er", DP), ("ei", DP), ("allow", DP), ("ur", DP), ("ui", DP), ("W", DP),
                ("somelr", DP), ("someli", DP), ("lmin", C.c_int), ("lmax", C.c_int),
                ("npmax", C.c_int), ("nproj", IP), ("mpcr", DP), ("mpci", DP), ("mpm", DP),
                ("mhr", DP), ("mhi", DP), ("celvol", C.c_double),
                ("interaction_scale", C.c_double), ("e0", C.c_int), ("long_range", C.c_int),
                ("mult", C.c_int), ("nhflag", C.c_int * 6), ("nthreads", C.c_int)]


class OrLrIn(C.Structure):
    _fields_ = [("avec", C.c_double * 9), ("tau", C.c_double * 3), ("epsilon0", C.c_double),
                ("interaction_scale", C.c_double), ("nptab", C.c_int), ("rtab", DP), ("ptab", DP),
                ("isolated", C.c_int), ("iso_cut", C.c_double), ("pbc", C.c_int * 3),
                ("have_eps3d", C.c_int), ("epsilon3d", C.c_double * 3),
                ("xshift_override", C.c_int * 3)]


def build(force: bool = False) -> str:
    path = os.path.join(_HERE, "liboracle.so")
    srcs = [os.path.join(_HERE, f) for f in ("ocean_oracle.cpp", "ocean_oracle_val.cpp", "ocean_oracle.h")]
    if force or not os.path.exists(path) or os.path.getmtime(path) < max(os.path.getmtime(f) for f in srcs):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return path


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        L = _LIB
        L.or_intval.restype = C.c_double
        L.or_pnorm.restype = C.c_double
        L.or_gamfcn.restype = C.c_double
        L.or_threey.restype = C.c_double
        L.or_val_wall_length.restype = C.c_double
    return _LIB


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(DP)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(IP)


def dims_of(w) -> OrDims:
    d = OrDims()
    d.nb = w.nb
    d.kmesh[:] = list(w.kmesh)
    d.xmesh[:] = list(w.xmesh)
    d.na = w.na
    d.nspn = w.nspn
    d.core_l = w.core_l
    return d


def lr_in_of(w) -> OrLrIn:
    p = OrLrIn()
    p.avec[:] = list(w.avec)
    p.tau[:] = list(w.tau)
    p.epsilon0 = w.epsilon0
    p.interaction_scale = w.interaction_scale
    p.nptab = len(w.rtab)
    p.rtab = dptr(w.rtab)
    p.ptab = dptr(w.ptab)
    p.isolated = 0
    p.iso_cut = 0.0
    p.pbc[:] = [0, 0, 0]
    p.have_eps3d = 0
    p.epsilon3d[:] = [1.0, 1.0, 1.0]
    p.xshift_override[:] = [1, 1, 1]
    return p


class OracleProblem:
    """Operator data of one workload, set up by the oracle's own lrLOAD + W2."""

    def __init__(self, w, nthreads: int = 0, hflag=(1, 1, 1, 1, 1, 1)):
        L = lib()
        self.w = w
        # keep every array whose address is handed to the C side alive
        self._refs = [w.er, w.ei, w.allow, w.rtab, w.ptab]
        if w.mult is not None:
            self._refs += list(w.mult.values())
        self.d = dims_of(w)
        self.ur = w.ur.copy()
        self.ui = w.ui.copy()
        tau = (C.c_double * 3)(*list(w.tau))
        ovr = (C.c_int * 3)(1, 1, 1)
        xs = (C.c_int * 3)()
        L.or_lrload(C.byref(self.d), tau, ovr, xs, dptr(self.ur), dptr(self.ui))
        self.xshift = tuple(xs)
        self.tau_shifted = tuple(tau)
        self.lr = lr_in_of(w)
        self.W = np.zeros(w.nk * w.nx)
        L.or_populate_w2(C.byref(self.d), C.byref(self.lr), tau, xs, dptr(self.W))
        o = OrOps()
        o.er = dptr(w.er)
        o.ei = dptr(w.ei)
        o.allow = dptr(w.allow)
        o.ur = dptr(self.ur)
        o.ui = dptr(self.ui)
        o.W = dptr(self.W)
        o.celvol = w.celvol
        o.interaction_scale = w.interaction_scale
        o.e0 = 1
        o.long_range = 1
        o.mult = 1 if w.mult is not None else 0
        o.nhflag[:] = list(hflag)
        o.nthreads = nthreads
        self._keep = []
        if w.mult is not None:
            m = w.mult
            o.lmin, o.lmax, o.npmax = m["lmin"], m["lmax"], m["npmax"]
            o.nproj = iptr(m["nproj"])
            o.mpcr, o.mpci = dptr(m["mpcr"]), dptr(m["mpci"])
            o.mpm, o.mhr, o.mhi = dptr(m["mpm"]), dptr(m["mhr"]), dptr(m["mhi"])
            self.somelr = np.zeros(w.na * w.na)
            self.someli = np.zeros(w.na * w.na)
            L.or_soprep(w.core_l, C.c_double(w.so_xi), dptr(self.somelr), dptr(self.someli))
            o.somelr, o.someli = dptr(self.somelr), dptr(self.someli)
        self.o = o

    def xact(self, pr, pi, hflag=None, backwards=False):
        out_r = np.zeros(self.w.npsi)
        out_i = np.zeros(self.w.npsi)
        hf = None if hflag is None else (C.c_int * 6)(*hflag)
        lib().or_xact(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(pr)),
                      dptr(np.ascontiguousarray(pi)), dptr(out_r), dptr(out_i), hf,
                      int(bool(backwards)))
        return out_r, out_i

    def haydock(self, niter, pr=None, pi=None):
        w = self.w
        pr = w.psi_r if pr is None else pr
        pi = w.psi_i if pi is None else pi
        ra = np.zeros(niter + 1)
        ia = np.zeros(niter + 1)
        rb = np.zeros(niter + 1)
        done = C.c_int(0)
        rc = lib().or_haydock(C.byref(self.d), C.byref(self.o), dptr(pr), dptr(pi), niter,
                              dptr(ra), dptr(ia), dptr(rb), C.byref(done))
        return rc, ra, ia, rb, done.value

    def haydock_conv(self, niter, threshold, spacing, ne, el=None, eh=None, gam0=None, pr=None, pi=None):
        """Haydock with the haydockconv.ipt early exit (OCEAN_haydock.f90:268-292,
        check_convergence :1608-1661): returns rc, a, ia, b, niter_actual and the
        relArea of each checked iteration."""
        w = self.w
        pr = w.psi_r if pr is None else pr
        pi = w.psi_i if pi is None else pi
        el = w.el if el is None else el
        eh = w.eh if eh is None else eh
        gam0 = w.gam0 if gam0 is None else gam0
        ra, ia, rb, rel = (np.zeros(niter + 1) for _ in range(4))
        done = C.c_int(0)
        rc = lib().or_haydock_conv(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(pr)),
                                   dptr(np.ascontiguousarray(pi)), niter, C.c_double(threshold), int(spacing),
                                   C.c_double(w.kpref), C.c_double(el), C.c_double(eh), int(ne), C.c_double(gam0),
                                   dptr(ra), dptr(ia), dptr(rb), dptr(rel), C.byref(done))
        return rc, ra, ia, rb, done.value, rel

    def haydock_nonherm(self, niter, pr=None, pi=None):
        """Two-sided Lanczos (OCEAN_haydock.f90:53-164,1250-1433): complex a, b, c."""
        w = self.w
        pr = w.psi_r if pr is None else pr
        pi = w.psi_i if pi is None else pi
        co = [np.zeros(niter + 1) for _ in range(6)]
        done = C.c_int(0)
        rc = lib().or_haydock_nonherm(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(pr)),
                                      dptr(np.ascontiguousarray(pi)), niter, *[dptr(x) for x in co],
                                      C.byref(done))
        return rc, co, done.value

    def gmres(self, energies_ev, depth=80, gres=None, gprc=None, ffff=1e-6, max_restarts=50):
        w = self.w
        e = np.ascontiguousarray(energies_ev, dtype=np.float64)
        n = len(e)
        gres = w.gam0 if gres is None else gres
        gprc = w.gmres_gprc if gprc is None else gprc
        ore, oim, rel = np.zeros(n), np.zeros(n), np.zeros(n)
        its = np.zeros(n, dtype=np.int32)
        tot = C.c_int(0)
        rc = lib().or_gmres(C.byref(self.d), C.byref(self.o), dptr(w.psi_r), dptr(w.psi_i),
                            C.c_double(w.kpref), dptr(e), n, depth, C.c_double(gres),
                            C.c_double(gprc), C.c_double(ffff), max_restarts, dptr(ore), dptr(oim),
                            dptr(rel), iptr(its), C.byref(tot))
        return rc, ore, oim, rel, its, tot.value


def calc_spect_core(ra, ia, rb, it, kpref, el, eh, ne, gam0, ebase=0.0):
    """calc_spect_core (OCEAN_haydock.f90:1991-2027): ne x 3 (energy, Re, Im part columns)."""
    out = np.zeros(ne * 3)
    lib().or_calc_spect_core(dptr(np.ascontiguousarray(ra, dtype=np.float64)),
                             dptr(np.ascontiguousarray(ia, dtype=np.float64)),
                             dptr(np.ascontiguousarray(rb, dtype=np.float64)), it, C.c_double(kpref),
                             C.c_double(el), C.c_double(eh), ne, C.c_double(gam0), C.c_double(ebase), dptr(out))
    return out.reshape(ne, 3)


def check_convergence(ra, ia, rb, iter1, iter2, kpref, el, eh, ne, gam0):
    """check_convergence (OCEAN_haydock.f90:1608-1661): (maxDiff, relArea)."""
    md, rel = C.c_double(0.0), C.c_double(0.0)
    lib().or_check_convergence(dptr(np.ascontiguousarray(ra, dtype=np.float64)),
                               dptr(np.ascontiguousarray(ia, dtype=np.float64)),
                               dptr(np.ascontiguousarray(rb, dtype=np.float64)), iter1, iter2, C.c_double(kpref),
                               C.c_double(el), C.c_double(eh), ne, C.c_double(gam0), C.byref(md), C.byref(rel))
    return md.value, rel.value


def early_exit_iter(rel, niter, spacing, threshold):
    """The stopping iteration of the early exit for per-iteration relArea values."""
    return int(lib().or_early_exit_iter(dptr(np.ascontiguousarray(rel, dtype=np.float64)), niter, int(spacing),
                                        C.c_double(threshold)))


def nbsemhsetup2(lc, lv, fk, gk, scfk=None, scgk=None, scfac=1.0, npt=16):
    """The exchange matrix of valence l = lv (OCEAN_multiplet.f90:2007-2181),
    threey by npt-point Gauss-Legendre quadrature: (mhr, mhi) flat, (mham,
    mham) with i1 fastest, Hartree.  fk / gk: {k: (np, np) array} in eV."""
    npr = None
    for d in (fk, gk):
        for a in d.values():
            npr = np.asarray(a).shape[0]

    def stack(d, sc):
        ks = sorted(d)
        if not ks:
            return None, None, 0, -1
        arr = np.concatenate([np.asarray(d[k], dtype=np.float64).T.reshape(-1) for k in ks])
        scl = np.array([1.0 if sc is None else sc.get(k, 1.0) for k in ks])
        return arr, scl, ks[0], ks[-1]

    fa, fs, kfl, kfh = stack(fk, scfk)
    ga, gs, kgl, kgh = stack(gk, scgk)
    mham = 4 * (2 * lc + 1) * (2 * lv + 1) * npr
    mhr, mhi = np.zeros(mham * mham), np.zeros(mham * mham)
    lib().or_nbsemhsetup2(lc, lv, npr, kfl, kfh, None if fa is None else dptr(fa), None if fs is None else dptr(fs),
                          kgl, kgh, None if ga is None else dptr(ga), None if gs is None else dptr(gs),
                          C.c_double(scfac), npt, dptr(mhr), dptr(mhi))
    return mhr, mhi


def threey(ll, ml, lm, mm, lr, mr, conjug=False, npt=16):
    return float(lib().or_threey(ll, ml, lm, mm, lr, mr, int(bool(conjug)), npt))


def write_core(ra, ia, rb, it, kpref, el, eh, ne, gam0, ebase=0.0, gam_gauss=0.0, ucvol=1.0,
               old_broaden=0, nval=0.0, eps=1.0):
    out = np.zeros((ne + 1) * 9)
    ia_p = None if ia is None else dptr(np.ascontiguousarray(ia, dtype=np.float64))
    lib().or_write_core(dptr(np.ascontiguousarray(ra, dtype=np.float64)), ia_p,
                        dptr(np.ascontiguousarray(rb, dtype=np.float64)), it, C.c_double(kpref),
                        C.c_double(el), C.c_double(eh), ne, C.c_double(gam0), C.c_double(ebase),
                        C.c_double(gam_gauss), C.c_double(ucvol), old_broaden, C.c_double(nval),
                        C.c_double(eps), dptr(out))
    return out.reshape(ne + 1, 9)


def write_core_bc(ra, ia, rb, ib, rc, ic, it, kpref, el, eh, ne, gam0, ebase=0.0, ucvol=1.0):
    """write_core rows for complex b and c (non-Hermitian runs)."""
    out = np.zeros((ne + 1) * 9)
    arrs = [dptr(np.ascontiguousarray(x, dtype=np.float64)) for x in (ra, ia, rb, ib, rc, ic)]
    lib().or_write_core_bc(*arrs, it, C.c_double(kpref), C.c_double(el), C.c_double(eh), ne, C.c_double(gam0),
                           C.c_double(ebase), C.c_double(ucvol), dptr(out))
    return out.reshape(ne + 1, 9)


def write_val(ra, ia, rb, it, kpref, ucvol, el, eh, ne, gam0, val_ham_spin=1, semi_tda=False, backf=False,
              ib=None, rc=None, ic=None):
    """write_val rows (ne x 8) of a valence run."""
    out = np.zeros(ne * 8)
    arr = [None if x is None else dptr(np.ascontiguousarray(x, dtype=np.float64)) for x in (ia, ib, rc, ic)]
    rc_ = lib().or_write_val(dptr(np.ascontiguousarray(ra, dtype=np.float64)), arr[0],
                             dptr(np.ascontiguousarray(rb, dtype=np.float64)), arr[1], arr[2], arr[3], it,
                             C.c_double(kpref), C.c_double(ucvol), val_ham_spin, int(bool(semi_tda)),
                             int(bool(backf)), C.c_double(el), C.c_double(eh), ne, C.c_double(gam0), dptr(out))
    assert rc_ == 0
    return out.reshape(ne, 8)


def redtrid(n, ra, rb):
    w = np.zeros(n + 1)
    rc = lib().or_redtrid(n, dptr(np.ascontiguousarray(ra, dtype=np.float64)),
                          dptr(np.ascontiguousarray(rb, dtype=np.float64)), dptr(w))
    return rc, w


def fft3d(kmesh, re, im, sign):
    re = np.ascontiguousarray(re, dtype=np.float64).copy()
    im = np.ascontiguousarray(im, dtype=np.float64).copy()
    km = (C.c_int * 3)(*kmesh)
    lib().or_fft3d(km, dptr(re), dptr(im), sign)
    return re, im


def zhptrf_solve(ap: np.ndarray, b: np.ndarray):
    """Factor packed-upper Hermitian ap (complex, n(n+1)/2) and solve for b."""
    n = len(b)
    apc = np.ascontiguousarray(ap, dtype=np.complex128).copy()
    ipiv = np.zeros(n, dtype=np.int32)
    info = lib().or_zhptrf_u(n, apc.view(np.float64).ctypes.data_as(DP), iptr(ipiv))
    x = np.ascontiguousarray(b, dtype=np.complex128).copy()
    if info == 0:
        lib().or_zhptrs_u(n, apc.view(np.float64).ctypes.data_as(DP), iptr(ipiv),
                          x.view(np.float64).ctypes.data_as(DP))
    return info, ipiv, x


# ---------------------------------------------------------------- valence BSE

class OrValDims(C.Structure):
    _fields_ = [("nc", C.c_int), ("nv", C.c_int), ("kmesh", C.c_int * 3), ("xmesh", C.c_int * 3),
                ("nspn", C.c_int), ("vspin", C.c_int)]


class OrValOps(C.Structure):
    _fields_ = [("er", DP), ("ei", DP), ("allow", DP), ("conr", DP), ("coni", DP), ("valr", DP),
                ("vali", DP), ("bubble", DP), ("ladder", DP), ("bande", C.c_int), ("bflag", C.c_int),
                ("lflag", C.c_int), ("fxc", DP)]


def val_fxc_from_rho(rho, celvol, nkpts):
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    out = np.zeros(len(rho))
    lib().or_val_fxc_from_rho(len(rho), dptr(rho), C.c_double(celvol), int(nkpts), dptr(out))
    return out


def val_wall_length(xmesh, bvec) -> float:
    return lib().or_val_wall_length((C.c_int * 3)(*xmesh), (C.c_double * 9)(*list(bvec)))


def val_bubble(xmesh, bvec, qinb, celvol, nkpts):
    """AI_bubble_populate with wall_search_old_way; returns (bubble, ngvec)."""
    n = int(np.prod(xmesh))
    out = np.zeros(n)
    length = val_wall_length(xmesh, bvec)
    ng = lib().or_val_bubble_populate((C.c_int * 3)(*xmesh), (C.c_double * 9)(*list(bvec)),
                                      (C.c_double * 3)(*list(qinb)), C.c_double(celvol), nkpts,
                                      C.c_double(length), dptr(out))
    return out, ng


class OracleVal:
    """Operator data of one valence workload (ValWorkload with host arrays; the
    ladder may be None when only slabs are timed)."""

    def __init__(self, w, bflag=1, lflag=1, bande=1):
        self.w = w
        if w.ladder is None:
            w = __import__("dataclasses").replace(w, ladder=np.zeros(1))
        self.bubble, self.ngvec = val_bubble(w.xmesh, w.bvec, w.qinb, w.celvol, w.nk)
        self._refs = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (w.er, w.ei, w.allow, w.conr, w.coni, w.valr, w.vali, self.bubble, w.ladder)]
        d = OrValDims()
        d.nc, d.nv = w.nc, w.nv
        d.kmesh[:] = list(w.kmesh)
        d.xmesh[:] = list(w.xmesh)
        d.nspn = getattr(w, "nspn", 1)
        d.vspin = getattr(w, "vspin", 1)
        self.d = d
        o = OrValOps()
        (o.er, o.ei, o.allow, o.conr, o.coni, o.valr, o.vali, o.bubble, o.ladder) = [dptr(a) for a in self._refs]
        o.bande, o.bflag, o.lflag = bande, bflag, lflag
        self.fxc = None
        if getattr(w, "rho", None) is not None:
            self.fxc = val_fxc_from_rho(w.rho, w.celvol, w.nk)
            o.fxc = dptr(self.fxc)
        self.o = o

    def act(self, pr, pi, backwards=False, flags=None):
        """H psi; flags = (bande, bflag, lflag) for this call only (default: the
        flags the problem was built with)."""
        saved = (self.o.bande, self.o.bflag, self.o.lflag)
        if flags is not None:
            self.o.bande, self.o.bflag, self.o.lflag = flags
        hr, hi = np.zeros(self.w.npsi), np.zeros(self.w.npsi)
        try:
            lib().or_val_act(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(pr, dtype=np.float64)),
                             dptr(np.ascontiguousarray(pi, dtype=np.float64)), dptr(hr), dptr(hi),
                             int(bool(backwards)))
        finally:
            self.o.bande, self.o.bflag, self.o.lflag = saved
        return hr, hi

    def haydock(self, niter, pr=None, pi=None):
        w = self.w
        pr = np.ascontiguousarray(w.psi_r if pr is None else pr, dtype=np.float64)
        pi = np.ascontiguousarray(w.psi_i if pi is None else pi, dtype=np.float64)
        ra, ia, rb = np.zeros(niter + 1), np.zeros(niter + 1), np.zeros(niter + 1)
        done = C.c_int(0)
        rc = lib().or_val_haydock(C.byref(self.d), C.byref(self.o), dptr(pr), dptr(pi), niter, dptr(ra), dptr(ia),
                                  dptr(rb), C.byref(done))
        return rc, ra, ia, rb, done.value

    def gmres(self, energies_ev, depth=80, gres=None, gprc=0.5, ffff=1e-6, max_restarts=50):
        """GMRES over the valence action (OCEAN_gmres.f90:508-908, have_val)."""
        w = self.w
        e = np.ascontiguousarray(energies_ev, dtype=np.float64)
        n = len(e)
        gres = w.gam0 if gres is None else gres
        ore, oim, rel = np.zeros(n), np.zeros(n), np.zeros(n)
        its = np.zeros(n, dtype=np.int32)
        tot = C.c_int(0)
        rc = lib().or_val_gmres(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(w.psi_r)),
                                dptr(np.ascontiguousarray(w.psi_i)), C.c_double(w.kpref), C.c_double(w.celvol),
                                dptr(e), n, depth, C.c_double(gres), C.c_double(gprc), C.c_double(ffff),
                                max_restarts, dptr(ore), dptr(oim), dptr(rel), iptr(its), C.byref(tot))
        return rc, ore, oim, rel, its, tot.value

    def ladder_slab(self, pr, pi, y0, y1, lad_slab):
        """Direct-term contribution of y in [y0, y1) (lad_slab: ladder rows of those y)."""
        hr, hi = np.zeros(self.w.npsi), np.zeros(self.w.npsi)
        lib().or_val_ladder_slab(C.byref(self.d), C.byref(self.o), dptr(np.ascontiguousarray(pr, dtype=np.float64)),
                                 dptr(np.ascontiguousarray(pi, dtype=np.float64)), int(y0), int(y1),
                                 dptr(np.ascontiguousarray(lad_slab, dtype=np.float64)), dptr(hr), dptr(hi))
        return hr, hi
