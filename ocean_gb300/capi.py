"""ctypes bindings of libocean_gpu.so and a thin host-side mirror of the
reference's call surface (OCEAN_xact / OCEAN_haydock_do / OCEAN_gmres_do_recycle).

The library is the product: this module only marshals numpy arrays across the
C ABI declared in include/ocean_gpu.h.  It raises if the library is missing;
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libocean_gpu.so")

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)

OCN_PREC_FP64 = 0
OCN_PREC_MIXED = 1
OCN_OK, OCN_ERR_NAN, OCN_ERR_ARG, OCN_ERR_STATE = 0, -1, 1, 4

STATUS = {0: "OK", -1: "NaN in Lanczos a", 1: "bad argument", 2: "CUDA error", 3: "allocation failed",
          4: "operator data not set", 5: "device wait timed out", 6: "GMRES did not converge",
          7: "Gram matrix factorisation failed", 9962: "unsupported"}


class OcnDims(C.Structure):
    _fields_ = [("num_bands", C.c_int), ("kmesh", C.c_int * 3), ("xmesh", C.c_int * 3),
                ("nalpha", C.c_int), ("nspn", C.c_int), ("core_l", C.c_int),
                ("precision", C.c_int), ("device", C.c_int), ("nvec", C.c_int)]


class OcnSystem(C.Structure):
    _fields_ = [("celvol", C.c_double), ("interaction_scale", C.c_double), ("e0", C.c_int),
                ("long_range", C.c_int), ("mult", C.c_int), ("nhflag", C.c_int * 6)]


class OcnLrParams(C.Structure):
    _fields_ = [("avec", C.c_double * 9), ("tau", C.c_double * 3), ("epsilon0", C.c_double),
                ("interaction_scale", C.c_double), ("nptab", C.c_int), ("rtab", DP),
                ("ptab", DP), ("isolated", C.c_int), ("iso_cut", C.c_double),
                ("pbc", C.c_int * 3), ("have_eps3d", C.c_int), ("epsilon3d", C.c_double * 3),
                ("xshift_override", C.c_int * 3)]


class OcnMultData(C.Structure):
    _fields_ = [("lmin", C.c_int), ("lmax", C.c_int), ("nproj", IP), ("mpcr", DP), ("mpci", DP),
                ("mpm", DP), ("mhr", DP), ("mhi", DP)]


class OcnCfParams(C.Structure):
    _fields_ = [("el", C.c_double), ("eh", C.c_double), ("gam0", C.c_double),
                ("ebase", C.c_double), ("gam_gauss", C.c_double), ("ne", C.c_int),
                ("ucvol", C.c_double), ("old_broaden", C.c_int), ("nval", C.c_double),
                ("eps", C.c_double)]


class OcnGmresParams(C.Structure):
    _fields_ = [("depth", C.c_int), ("resolution", C.c_double), ("preconditioner", C.c_double),
                ("convergence", C.c_double), ("max_restarts", C.c_int)]


class OcnHaydockConv(C.Structure):
    _fields_ = [("threshold", C.c_double), ("spacing", C.c_int), ("ne", C.c_int), ("el", C.c_double),
                ("eh", C.c_double), ("gam0", C.c_double), ("kpref", C.c_double)]


class OcnBseIn(C.Structure):
    _fields_ = [("dumi", C.c_int), ("dumf", C.c_double), ("style", C.c_char * 8), ("niter", C.c_int),
                ("ne", C.c_int), ("el", C.c_double), ("eh", C.c_double), ("gam0", C.c_double),
                ("ebase", C.c_double), ("depth", C.c_int), ("resolution", C.c_double),
                ("preconditioner", C.c_double), ("convergence", C.c_double), ("inv_style", C.c_char * 8),
                ("nomega", C.c_int)]


# every entry point declared in include/ocean_gpu.h
EXPORTS = [
    "ocn_ctx_create", "ocn_ctx_destroy", "ocn_last_error", "ocn_version", "ocn_set_system",
    "ocn_set_energies", "ocn_set_allow", "ocn_set_bloch", "ocn_lr_init", "ocn_set_W", "ocn_get_W",
    "ocn_get_bloch", "ocn_set_mult", "ocn_set_spin_orbit", "ocn_soprep", "ocn_apply_H",
    "ocn_apply_H_dev", "ocn_haydock", "ocn_haydock_dev", "ocn_psi_pnorm", "ocn_spectrum_cf",
    "ocn_redtrid", "ocn_gmres", "ocn_kernel_launches", "ocn_w2_host", "ocn_phase_table_host",
    "ocn_timing_enable", "ocn_timing_reset", "ocn_timing_read", "ocn_stream", "ocn_apply_H_block",
    "ocn_haydock_block", "ocn_haydock_block_dev", "ocn_spectrum_cf_noalloc", "ocn_gmres_dev",
    "ocn_gmres_vjp", "ocn_w2_vjp", "ocn_haydock_batch", "ocn_autotune", "ocn_set_tiles", "ocn_get_tiles",
    "ocn_read_bse_in", "ocn_write_abslanc", "ocn_write_absspct", "ocn_write_abs_gmres", "ocn_output_filename",
    "ocn_read_u2dat", "ocn_read_rpottrim", "ocn_read_energies", "ocn_read_cks", "ocn_cks_to_mpc", "ocn_read_cmel",
    "ocn_input_filename", "ocn_haydock_nonherm", "ocn_spectrum_cf_bc",
    "ocn_val_create", "ocn_val_destroy", "ocn_val_last_error", "ocn_val_kernel_launches", "ocn_val_stream",
    "ocn_val_set_energies", "ocn_val_set_allow", "ocn_val_set_states", "ocn_val_set_states_dev",
    "ocn_val_set_bubble", "ocn_val_set_ladder", "ocn_val_set_ladder_dev", "ocn_val_bubble_populate",
    "ocn_val_apply_H", "ocn_val_apply_H_dev", "ocn_val_haydock", "ocn_val_haydock_dev",
    "ocn_val_spectrum", "ocn_val_optical_constants", "ocn_write_opcons", "ocn_val_set_fxc",
    "ocn_val_fxc_from_rho", "ocn_read_val_u2", "ocn_val_pair_energies", "ocn_test_starve_tc",
    "ocn_gmres_set_lanes", "ocn_set_haydock_conv", "ocn_read_haydockconv",
    "ocn_read_u2par", "ocn_read_con_u2", "ocn_read_obf_control",
    "ocn_mult_exchange", "ocn_threey", "ocn_read_slater", "ocn_val_gmres",
]

TIMED_CLASSES = ["lr_band_to_x", "lr_kmesh_transform", "lr_x_to_band", "lr_prep", "multiplet",
                 "combine_lanczos"]


def _lr_params(w):
    p = OcnLrParams()
    p.avec[:] = list(w.avec)
    p.tau[:] = list(w.tau)
    p.epsilon0 = w.epsilon0
    p.interaction_scale = w.interaction_scale
    rtab, ptab = _f64(w.rtab), _f64(w.ptab)
    p.nptab = len(rtab)
    p.rtab = _dp(rtab)
    p.ptab = _dp(ptab)
    p.pbc[:] = [0, 0, 0]
    p.epsilon3d[:] = [1.0, 1.0, 1.0]
    p.xshift_override[:] = [1, 1, 1]
    return p, (rtab, ptab)


def _dims(w, precision=0, device=0, nvec=1):
    d = OcnDims()
    d.num_bands = w.nb
    d.kmesh[:] = list(w.kmesh)
    d.xmesh[:] = list(w.xmesh)
    d.nalpha = w.na
    d.nspn = w.nspn
    d.core_l = w.core_l
    d.precision = precision
    d.device = device
    d.nvec = nvec
    return d


def w2_host(w):
    """W(Nk,Nx), xshift and shifted tau computed by the library's host code."""
    d = _dims(w)
    p, keep = _lr_params(w)
    W = np.zeros(w.nk * w.nx)
    xs = (C.c_int * 3)()
    tau = (C.c_double * 3)()
    check(load().ocn_w2_host(C.byref(d), C.byref(p), _dp(W), xs, tau))
    return W, tuple(xs), tuple(tau)


def haydock_batch(contexts, d_psi0, nvs, niter: int):
    """ocn_haydock_batch: context i runs nvs[i] chains from device address
    d_psi0[i] (vector v at + 2*v*npsi doubles).  Returns per context arrays
    (ra, ia, rb) of shape (nv, niter+1) and the iteration counts."""
    lib = load()
    k = len(contexts)
    outs = [tuple(np.zeros((nv, niter + 1)) for _ in range(3)) for nv in nvs]
    dones = [np.zeros(nv, dtype=np.int32) for nv in nvs]
    ctxs = (C.c_void_p * k)(*[c.ptr.value for c in contexts])
    nvarr = (C.c_int * k)(*nvs)
    psi = (C.c_void_p * k)(*d_psi0)
    ra = (DP * k)(*[_dp(o[0]) for o in outs])
    ia = (DP * k)(*[_dp(o[1]) for o in outs])
    rb = (DP * k)(*[_dp(o[2]) for o in outs])
    nd = (IP * k)(*[d.ctypes.data_as(IP) for d in dones])
    rc = lib.ocn_haydock_batch(ctxs, k, nvarr, psi, niter, ra, ia, rb, nd)
    if rc:
        bad = next((c for c in contexts if last_error(c.ptr)), None)
        raise OcnError(rc, last_error(bad.ptr) if bad else "")
    return [(o[0], o[1], o[2], d) for o, d in zip(outs, dones)]


def w2_vjp(w, G):
    """dL/dptab and dL/d(interaction_scale) from dL/dW (Nk*Nx, [x*Nk + k])."""
    d = _dims(w)
    p, keep = _lr_params(w)
    gp = np.zeros(len(keep[1]))
    gs = C.c_double(0.0)
    check(load().ocn_w2_vjp(C.byref(d), C.byref(p), _dp(_f64(G)), _dp(gp), C.byref(gs)))
    return gp, gs.value


def phase_table_host(w, xshift):
    d = _dims(w)
    c, s = np.zeros(w.nk * w.nx), np.zeros(w.nk * w.nx)
    xs = (C.c_int * 3)(*xshift)
    check(load().ocn_phase_table_host(C.byref(d), xs, _dp(c), _dp(s)))
    return c, s

_LIB = None


def load(path: str = LIB_PATH):
    """Load libocean_gpu.so; raises (no fallback) if it is absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: run ocean_gb300.build.build() first")
        lib = C.CDLL(path)
        lib.ocn_version.restype = C.c_char_p
        lib.ocn_kernel_launches.restype = C.c_longlong
        lib.ocn_stream.restype = C.c_void_p
        lib.ocn_val_kernel_launches.restype = C.c_longlong
        lib.ocn_val_stream.restype = C.c_void_p
        _LIB = lib
    return _LIB


class OcnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ocean_gpu error {code} ({STATUS.get(code, '?')}): {msg}")
        self.code = code


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 contiguous array required"
    return a.ctypes.data_as(DP)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def last_error(ctx=None) -> str:
    buf = C.create_string_buffer(1024)
    load().ocn_last_error(ctx, buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int, ctx=None):
    if rc != 0:
        raise OcnError(rc, last_error(ctx))


class Context:
    """One problem on one GPU: mirrors the module state the reference loads in
    ocean_load_data (OCEAN_load_data.f90:8-173) and the operators that use it."""

    def __init__(self, w, precision: int = OCN_PREC_FP64, device: int = 0,
                 hflag=(1, 1, 1, 1, 1, 1), set_mult: bool = True, nvec: int = 1):
        lib = load()
        self.w = w
        self.lib = lib
        d = _dims(w, precision, device, nvec)
        self.nvec = max(1, nvec)
        self.dims = d
        self.ptr = C.c_void_p()
        check(lib.ocn_ctx_create(C.byref(d), C.byref(self.ptr)))
        try:
            s = OcnSystem()
            s.celvol = w.celvol
            s.interaction_scale = w.interaction_scale
            s.e0 = 1
            s.long_range = 1
            s.mult = 1 if (w.mult is not None and set_mult) else 0
            s.nhflag[:] = list(hflag)
            self._chk(lib.ocn_set_system(self.ptr, C.byref(s)))
            self._chk(lib.ocn_set_energies(self.ptr, _dp(_f64(w.er)), _dp(_f64(w.ei))))
            self._chk(lib.ocn_set_allow(self.ptr, _dp(_f64(w.allow))))
            self._chk(lib.ocn_set_bloch(self.ptr, _dp(_f64(w.ur)), _dp(_f64(w.ui))))
            p = OcnLrParams()
            p.avec[:] = list(w.avec)
            p.tau[:] = list(w.tau)
            p.epsilon0 = w.epsilon0
            p.interaction_scale = w.interaction_scale
            self._rtab = _f64(w.rtab)
            self._ptab = _f64(w.ptab)
            p.nptab = len(self._rtab)
            p.rtab = _dp(self._rtab)
            p.ptab = _dp(self._ptab)
            p.pbc[:] = [0, 0, 0]
            p.epsilon3d[:] = [1.0, 1.0, 1.0]
            p.xshift_override[:] = [1, 1, 1]
            self._chk(lib.ocn_lr_init(self.ptr, C.byref(p)))
            if w.mult is not None and set_mult:
                m = w.mult
                md = OcnMultData()
                md.lmin, md.lmax = m["lmin"], m["lmax"]
                self._nproj = np.ascontiguousarray(m["nproj"], dtype=np.int32)
                md.nproj = self._nproj.ctypes.data_as(IP)
                md.mpcr, md.mpci = _dp(m["mpcr"]), _dp(m["mpci"])
                md.mpm, md.mhr, md.mhi = _dp(m["mpm"]), _dp(m["mhr"]), _dp(m["mhi"])
                self._chk(lib.ocn_set_mult(self.ptr, C.byref(md)))
                self._chk(lib.ocn_soprep(self.ptr, C.c_double(w.so_xi)))
        except Exception:
            self.close()
            raise

    def _chk(self, rc):
        check(rc, self.ptr)

    def close(self):
        if self.ptr:
            self.lib.ocn_ctx_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self.lib.ocn_kernel_launches(self.ptr))

    @property
    def stream(self) -> int:
        return int(self.lib.ocn_stream(self.ptr) or 0)

    def haydock_dev(self, niter: int, d_pr: int, d_pi: int):
        """Haydock with psi0 already in device memory (raw device addresses)."""
        ra, ia, rb = np.zeros(niter + 1), np.zeros(niter + 1), np.zeros(niter + 1)
        done = C.c_int(0)
        self._chk(self.lib.ocn_haydock_dev(self.ptr, C.c_void_p(d_pr), C.c_void_p(d_pi), niter,
                                           _dp(ra), _dp(ia), _dp(rb), C.byref(done)))
        return ra, ia, rb, done.value

    def timing(self, on: bool = True):
        self._chk(self.lib.ocn_timing_enable(self.ptr, int(on)))

    def starve_tc(self, on: bool = True):
        """Test hook: the tensor-core contractions' load warp issues nothing, so
        their bounded waits run out and calls report OCN_ERR_TIMEOUT."""
        self._chk(self.lib.ocn_test_starve_tc(self.ptr, int(on)))

    def timing_reset(self):
        self._chk(self.lib.ocn_timing_reset(self.ptr))

    def timing_read(self) -> dict:
        counts = (C.c_longlong * 6)()
        ms = (C.c_double * 6)()
        self._chk(self.lib.ocn_timing_read(self.ptr, counts, ms))
        return {name: (int(counts[i]), float(ms[i])) for i, name in enumerate(TIMED_CLASSES)}

    def get_W(self):
        W = np.zeros(self.w.nk * self.w.nx)
        xs = (C.c_int * 3)()
        tau = (C.c_double * 3)()
        self._chk(self.lib.ocn_get_W(self.ptr, _dp(W), xs, tau))
        return W, tuple(xs), tuple(tau)

    def get_bloch(self):
        n = self.w.nb * self.w.nk * self.w.nx * self.w.nspn
        r, i = np.zeros(n), np.zeros(n)
        self._chk(self.lib.ocn_get_bloch(self.ptr, _dp(r), _dp(i)))
        return r, i

    def apply_H(self, pr, pi, hflag=None, backwards=False):
        n = self.w.npsi
        outr, outi = np.zeros(n), np.zeros(n)
        hf = None if hflag is None else (C.c_int * 6)(*hflag)
        self._chk(self.lib.ocn_apply_H(self.ptr, _dp(_f64(pr)), _dp(_f64(pi)), _dp(outr), _dp(outi),
                                       hf, int(bool(backwards))))
        return outr, outi

    def haydock(self, niter: int, pr=None, pi=None):
        w = self.w
        pr = w.psi_r if pr is None else pr
        pi = w.psi_i if pi is None else pi
        ra, ia, rb = np.zeros(niter + 1), np.zeros(niter + 1), np.zeros(niter + 1)
        done = C.c_int(0)
        rc = self.lib.ocn_haydock(self.ptr, _dp(_f64(pr)), _dp(_f64(pi)), niter, _dp(ra), _dp(ia),
                                  _dp(rb), C.byref(done))
        self._chk(rc)
        return ra, ia, rb, done.value

    def apply_H_block(self, pr, pi, hflag=None, backwards=False):
        """H on a block of vectors: pr/pi of shape (nv, npsi)."""
        pr, pi = np.ascontiguousarray(pr, dtype=np.float64), np.ascontiguousarray(pi, dtype=np.float64)
        nv = pr.shape[0]
        outr, outi = np.zeros_like(pr), np.zeros_like(pi)
        hf = None if hflag is None else (C.c_int * 6)(*hflag)
        self._chk(self.lib.ocn_apply_H_block(self.ptr, nv, _dp(pr), _dp(pi), _dp(outr), _dp(outi), hf,
                                             int(bool(backwards))))
        return outr, outi

    def haydock_nonherm(self, niter: int, pr=None, pi=None):
        """Two-sided Lanczos (ocn_haydock_nonherm): returns ([a_r, a_i, b_r, b_i, c_r, c_i], done)."""
        w = self.w
        pr = _f64(w.psi_r if pr is None else pr)
        pi = _f64(w.psi_i if pi is None else pi)
        co = [np.zeros(niter + 1) for _ in range(6)]
        done = C.c_int(0)
        self._chk(self.lib.ocn_haydock_nonherm(self.ptr, _dp(pr), _dp(pi), niter, *[_dp(x) for x in co],
                                               C.byref(done)))
        return co, done.value

    def haydock_block(self, niter: int, pr, pi):
        """nv Lanczos chains in lockstep: pr/pi of shape (nv, npsi); returns arrays
        of shape (nv, niter+1) and the per-chain iteration counts."""
        pr, pi = np.ascontiguousarray(pr, dtype=np.float64), np.ascontiguousarray(pi, dtype=np.float64)
        nv = pr.shape[0]
        ra, ia, rb = (np.zeros((nv, niter + 1)) for _ in range(3))
        done = np.zeros(nv, dtype=np.int32)
        self._chk(self.lib.ocn_haydock_block(self.ptr, nv, _dp(pr), _dp(pi), niter, _dp(ra), _dp(ia),
                                             _dp(rb), done.ctypes.data_as(IP)))
        return ra, ia, rb, done

    def haydock_block_dev(self, niter: int, nv: int, d_psi0: int):
        """Block Haydock on device psi0 (vector v at d_psi0 + 2*v*npsi doubles)."""
        ra, ia, rb = (np.zeros((nv, niter + 1)) for _ in range(3))
        done = np.zeros(nv, dtype=np.int32)
        self._chk(self.lib.ocn_haydock_block_dev(self.ptr, nv, C.c_void_p(d_psi0), niter, _dp(ra), _dp(ia),
                                                 _dp(rb), done.ctypes.data_as(IP)))
        return ra, ia, rb, done

    def autotune(self, nv: int = 1, reps: int = 3):
        """Times the candidate tilings of the tensor-core contractions and keeps
        the fastest; returns (ms per long-range application, tiles)."""
        ms, cur = C.c_double(0.0), C.c_double(0.0)
        t = (C.c_int * 7)()
        self._chk(self.lib.ocn_autotune(self.ptr, nv, reps, C.byref(ms), C.byref(cur), t))
        self.last_tune_current_ms = cur.value
        return ms.value, tuple(t)

    def tiles(self):
        t = (C.c_int * 7)()
        self._chk(self.lib.ocn_get_tiles(self.ptr, t))
        return tuple(t)

    def set_tiles(self, tiles):
        self._chk(self.lib.ocn_set_tiles(self.ptr, (C.c_int * 7)(*tiles)))

    def set_W(self, W):
        self._chk(self.lib.ocn_set_W(self.ptr, _dp(_f64(W))))

    def set_energies(self, er, ei=None):
        self._chk(self.lib.ocn_set_energies(self.ptr, _dp(_f64(er)), None if ei is None else _dp(_f64(ei))))

    def _gmres_params(self, depth, resolution, preconditioner, tol, max_restarts):
        p = OcnGmresParams()
        p.depth = depth
        p.resolution = self.w.gam0 if resolution is None else resolution
        p.preconditioner = self.w.gmres_gprc if preconditioner is None else preconditioner
        p.convergence = tol
        p.max_restarts = max_restarts
        return p

    def set_haydock_conv(self, threshold: float, spacing: int = 1, ne: int = 200, el=None, eh=None, gam0=None,
                         kpref=None):
        """haydockconv.ipt early exit for single-chain Haydock runs (threshold <= 0: off)."""
        w = self.w
        p = OcnHaydockConv()
        p.threshold = threshold
        p.spacing = spacing
        p.ne = ne
        p.el = w.el if el is None else el
        p.eh = w.eh if eh is None else eh
        p.gam0 = w.gam0 if gam0 is None else gam0
        p.kpref = w.kpref if kpref is None else kpref
        self._chk(self.lib.ocn_set_haydock_conv(self.ptr, C.byref(p)))

    def set_gmres_lanes(self, nlanes: int):
        """Energy lanes of the GMRES sweeps of this context (1: the reference's single sweep)."""
        self._chk(self.lib.ocn_gmres_set_lanes(self.ptr, int(nlanes)))

    def gmres_dev(self, d_hay: int, energies_ev, depth=80, resolution=None, preconditioner=None, tol=1e-6,
                  max_restarts=50, kpref=None, d_x: int = 0):
        """GMRES with psi0 at device address d_hay (re plane, im plane); the
        solutions go to device address d_x (nomega blocks of 2*npsi) when given."""
        e = _f64(energies_ev)
        n = len(e)
        p = self._gmres_params(depth, resolution, preconditioner, tol, max_restarts)
        ore, oim, rel = np.zeros(n), np.zeros(n), np.zeros(n)
        its = np.zeros(n, dtype=np.int32)
        kp = self.w.kpref if kpref is None else kpref
        self._chk(self.lib.ocn_gmres_dev(self.ptr, C.c_void_p(d_hay), C.c_double(kp), _dp(e), n, C.byref(p),
                                         _dp(ore), _dp(oim), _dp(rel), its.ctypes.data_as(IP),
                                         C.c_void_p(d_x) if d_x else None))
        return ore, oim, rel, its

    def gmres_vjp(self, d_hay: int, energies_ev, d_x: int, d_gW: int, grad_re=None, grad_im=None, depth=80,
                  resolution=None, preconditioner=None, tol=1e-6, max_restarts=50, kpref=None):
        """Adjoint GMRES: returns (dL/dGamma, dL/dscissor); dL/dW lands at device address d_gW."""
        e = _f64(energies_ev)
        n = len(e)
        p = self._gmres_params(depth, resolution, preconditioner, tol, max_restarts)
        kp = self.w.kpref if kpref is None else kpref
        gg, gs = C.c_double(0.0), C.c_double(0.0)
        gr = None if grad_re is None else _dp(_f64(grad_re))
        gi = None if grad_im is None else _dp(_f64(grad_im))
        self._chk(self.lib.ocn_gmres_vjp(self.ptr, C.c_void_p(d_hay), C.c_double(kp), _dp(e), n, C.byref(p),
                                         C.c_void_p(d_x), gr, gi, C.byref(gg), C.byref(gs), C.c_void_p(d_gW)))
        return gg.value, gs.value

    def gmres(self, energies_ev, depth=80, resolution=None, preconditioner=None, tol=1e-6,
              max_restarts=50, kpref=None):
        w = self.w
        e = _f64(energies_ev)
        n = len(e)
        p = OcnGmresParams()
        p.depth = depth
        p.resolution = w.gam0 if resolution is None else resolution
        p.preconditioner = w.gmres_gprc if preconditioner is None else preconditioner
        p.convergence = tol
        p.max_restarts = max_restarts
        ore, oim, rel = np.zeros(n), np.zeros(n), np.zeros(n)
        its = np.zeros(n, dtype=np.int32)
        kp = w.kpref if kpref is None else kpref
        self._chk(self.lib.ocn_gmres(self.ptr, _dp(_f64(w.psi_r)), _dp(_f64(w.psi_i)), C.c_double(kp),
                                     _dp(e), n, C.byref(p), _dp(ore), _dp(oim), _dp(rel),
                                     its.ctypes.data_as(IP)))
        return ore, oim, rel, its


def spectrum_cf_bc(ra, ia, rb, ib, rc, ic, iteration: int, kpref: float, el: float, eh: float, ne: int,
                   gam0: float, ebase: float = 0.0, ucvol: float = 1.0) -> np.ndarray:
    """write_core rows for the complex b and c of a non-Hermitian run."""
    lib = load()
    p = OcnCfParams()
    p.el, p.eh, p.gam0, p.ebase, p.gam_gauss = el, eh, gam0, ebase, 0.0
    p.ne, p.ucvol, p.old_broaden, p.nval, p.eps = ne, ucvol, 0, 0.0, 1.0
    out = np.zeros((ne + 1) * 9)
    arrs = [None if x is None else _dp(_f64(x)) for x in (ra, ia, rb, ib, rc, ic)]
    check(lib.ocn_spectrum_cf_bc(*arrs, iteration, C.c_double(kpref), C.byref(p), _dp(out)))
    return out.reshape(ne + 1, 9)


def spectrum_cf(ra, ia, rb, iteration: int, kpref: float, el: float, eh: float, ne: int, gam0: float,
                ebase: float = 0.0, gam_gauss: float = 0.0, ucvol: float = 1.0,
                old_broaden: int = 0, nval: float = 0.0, eps: float = 1.0) -> np.ndarray:
    lib = load()
    p = OcnCfParams()
    p.el, p.eh, p.gam0, p.ebase, p.gam_gauss = el, eh, gam0, ebase, gam_gauss
    p.ne, p.ucvol, p.old_broaden, p.nval, p.eps = ne, ucvol, old_broaden, nval, eps
    out = np.zeros((ne + 1) * 9)
    ia_p = None if ia is None else _dp(_f64(ia))
    check(lib.ocn_spectrum_cf(_dp(_f64(ra)), ia_p, _dp(_f64(rb)), iteration, C.c_double(kpref),
                              C.byref(p), _dp(out)))
    return out.reshape(ne + 1, 9)


def spectrum_cf_noalloc(ra, ia, rb, iteration: int, kpref: float, el: float, eh: float, ne: int,
                        gam0: float, ebase: float = 0.0, ucvol: float = 1.0, old_broaden: int = 0,
                        nval: float = 0.0, eps: float = 1.0) -> np.ndarray:
    """write_core through ocn_spectrum_cf_noalloc (static device scratch, no allocation)."""
    lib = load()
    p = OcnCfParams()
    p.el, p.eh, p.gam0, p.ebase, p.gam_gauss = el, eh, gam0, ebase, 0.0
    p.ne, p.ucvol, p.old_broaden, p.nval, p.eps = ne, ucvol, old_broaden, nval, eps
    out = np.zeros((ne + 1) * 9)
    ia_p = None if ia is None else _dp(_f64(ia))
    check(lib.ocn_spectrum_cf_noalloc(_dp(_f64(ra)), ia_p, _dp(_f64(rb)), iteration, C.c_double(kpref),
                                      C.byref(p), _dp(out)))
    return out.reshape(ne + 1, 9)


def read_haydockconv(path: str):
    """haydockconv.ipt: (threshold, spacing)."""
    lib = load()
    t, sp = C.c_double(0.0), C.c_int(0)
    check(lib.ocn_read_haydockconv(path.encode(), C.byref(t), C.byref(sp)))
    return t.value, sp.value


def read_bse_in(path: str) -> dict:
    """bse.in as ocean.x reads it; energies (eV) of a GMRES run under 'energies'."""
    lib = load()
    b = OcnBseIn()
    check(lib.ocn_read_bse_in(path.encode(), C.byref(b), None, 0))
    e = np.zeros(max(b.nomega, 1))
    if b.nomega > 0:
        check(lib.ocn_read_bse_in(path.encode(), C.byref(b), _dp(e), len(e)))
    d = {k: getattr(b, k) for k, _ in OcnBseIn._fields_}
    d["style"], d["inv_style"] = b.style.decode(), b.inv_style.decode()
    d["energies"] = e[:b.nomega]
    return d


def write_abslanc(path: str, n: int, kpref: float, ra, rb, ia=None, ib=None, rc=None, ic=None, eigs=None):
    opt = [None if a is None else _dp(_f64(a)) for a in (ia, ib, rc, ic, eigs)]
    check(load().ocn_write_abslanc(path.encode(), n, C.c_double(kpref), _dp(_f64(ra)), opt[0], _dp(_f64(rb)),
                                   opt[1], opt[2], opt[3], opt[4]))


def write_absspct(path: str, iteration: int, gam0: float, kpref: float, ucvol: float, rows, voigt: bool = False):
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    ne = rows.shape[0] - 1
    check(load().ocn_write_absspct(path.encode(), iteration, C.c_double(gam0), C.c_double(kpref),
                                   C.c_double(ucvol), ne, _dp(rows.reshape(-1)), int(bool(voigt))))


def write_abs_gmres(path: str, energies_ev, out_re, out_im, rel_err, iters):
    it = np.ascontiguousarray(iters, dtype=np.int32)
    check(load().ocn_write_abs_gmres(path.encode(), len(it), _dp(_f64(energies_ev)), _dp(_f64(out_re)),
                                     _dp(_f64(out_im)), _dp(_f64(rel_err)), it.ctypes.data_as(IP)))


def output_filename(kind: str, calc_type: str, elname: str, indx: int, corelevel: str, photon: int) -> str:
    buf = C.create_string_buffer(64)
    check(load().ocn_output_filename(kind.encode(), calc_type.encode(), elname.encode(), indx,
                                     corelevel.encode(), photon, buf, 64))
    return buf.value.decode()


def input_filename(kind: str, elname: str, indx: int, n: int = 0, l: int = 0, calc_type: str = "XAS") -> str:
    buf = C.create_string_buffer(64)
    check(load().ocn_input_filename(kind.encode(), calc_type.encode(), elname.encode(), indx, n, l, buf, 64))
    return buf.value.decode()


def read_u2dat(path: str, nx: int, ny: int, nz: int, nkpts: int, nspn: int, nband_file: int, first, nbd: int):
    """u2.dat -> (re, im) of shape (nspn, Nx, nkpts, nbd) in C order, i.e. the
    Fortran re_bloch_state(nbd, nkpts, Nx, nspn).  first: one int or one per
    (k-point, spin), k fastest."""
    f = np.ascontiguousarray(np.atleast_1d(first), dtype=np.int32)
    nxyz = nx * ny * nz
    re = np.zeros((nspn, nxyz, nkpts, nbd))
    im = np.zeros_like(re)
    check(load().ocn_read_u2dat(path.encode(), nx, ny, nz, nkpts, nspn, nband_file, f.ctypes.data_as(IP), len(f),
                                nbd, _dp(re), _dp(im)))
    return re, im


def read_u2par(path: str, xmesh, nkpts: int, nspn: int, width3: int, first, nbd: int):
    """u2par.dat ('new' format) -> (re, im) shaped like read_u2dat's."""
    f = np.ascontiguousarray(np.atleast_1d(first), dtype=np.int32)
    nxyz = int(np.prod(xmesh))
    re = np.zeros((nspn, nxyz, nkpts, nbd))
    im = np.zeros_like(re)
    check(load().ocn_read_u2par(path.encode(), (C.c_int * 3)(*xmesh), nkpts, nspn, int(width3),
                                f.ctypes.data_as(IP), len(f), nbd, _dp(re), _dp(im)))
    return re, im


def read_con_u2(path: str, nxpts: int, nkpts: int, nspn: int, bands_in_file: int, nbd: int):
    """con.u2.dat of a core run ('par' route) -> (re, im) shaped like read_u2dat's."""
    re = np.zeros((nspn, nxpts, nkpts, nbd))
    im = np.zeros_like(re)
    check(load().ocn_read_con_u2(path.encode(), nxpts, nkpts, nspn, bands_in_file, nbd, _dp(re), _dp(im)))
    return re, im


def read_obf_control(path: str):
    w = (C.c_int * 3)()
    check(load().ocn_read_obf_control(path.encode(), w))
    return tuple(w)


def load_bloch_states(run_dir: str, xmesh, nkpts: int, nspn: int, nbd: int, first=0, bands_in_file=None,
                      calc_type: str = "XAS"):
    """The Bloch states of a core-level run directory, chosen as ocean.x chooses
    (OCEAN_bloch.f90:470-482): con.u2.dat (val.u2.dat for XES) present -> the
    'par' stream file; else bloch_type 'new' -> u2par.dat with obf_control's
    widths; else u2.dat ('old').  bands_in_file: bands per k-point in the 'par'
    file (brange(4) - brange(3) + 1) or in u2.dat; first: the skipped bands of
    the 'old' and 'new' formats.  Returns (format, re, im)."""
    par = os.path.join(run_dir, "val.u2.dat" if calc_type == "XES" else "con.u2.dat")
    if os.path.exists(par):
        nb_file = nbd if bands_in_file is None else bands_in_file
        return ("par",) + read_con_u2(par, int(np.prod(xmesh)), nkpts, nspn, nb_file, nbd)
    btype = "old"
    bt = os.path.join(run_dir, "bloch_type")
    if os.path.exists(bt):
        with open(bt) as fh:
            btype = fh.read().split()[0].strip("'\"")
    if btype == "new":
        width = read_obf_control(os.path.join(run_dir, "obf_control"))
        return ("new",) + read_u2par(os.path.join(run_dir, "u2par.dat"), xmesh, nkpts, nspn, width[2], first, nbd)
    nb_file = nbd if bands_in_file is None else bands_in_file
    return ("old",) + read_u2dat(os.path.join(run_dir, "u2.dat"), *xmesh, nkpts, nspn, nb_file, first, nbd)


def mult_exchange(lc: int, lv: int, fk: dict, gk: dict, scfk: dict = None, scgk: dict = None, scfac: float = 1.0):
    """nbsemhsetup2: the exchange matrix of valence l = lv (Hartree, the
    reference's (mham, mham) layout flattened) from Slater integrals in eV.
    fk / gk: {k: (np, np) array} (F^k for k = 2..min(2lc, 2lv), G^k for
    k = |lc-lv|..lc+lv); scfk / scgk: {k: scale} (default 1)."""
    np_ = None
    for d in (fk, gk):
        for a in d.values():
            np_ = np.asarray(a).shape[0]
    kf = sorted(fk)
    kg = sorted(gk)

    def stack(d, ks, sc):
        if not ks:
            return None, None, 0, -1
        arr = np.concatenate([np.asarray(d[k], dtype=np.float64).reshape(np_, np_).T.reshape(-1) for k in ks])
        scl = np.array([1.0 if sc is None else sc.get(k, 1.0) for k in ks])
        return arr, scl, ks[0], ks[-1]

    fa, fs, kfl, kfh = stack(fk, kf, scfk)
    ga, gs, kgl, kgh = stack(gk, kg, scgk)
    mham = 4 * (2 * lc + 1) * (2 * lv + 1) * np_
    mhr, mhi = np.zeros(mham * mham), np.zeros(mham * mham)
    lib = load()
    check(lib.ocn_mult_exchange(lc, lv, np_, kfl, kfh, None if fa is None else _dp(fa), None if fs is None else _dp(fs),
                                kgl, kgh, None if ga is None else _dp(ga), None if gs is None else _dp(gs),
                                C.c_double(scfac), _dp(mhr), _dp(mhi)))
    return mhr, mhi


def threey(ll, ml, lm, mm, lr, mr, conjug=False) -> float:
    lib = load()
    lib.ocn_threey.restype = C.c_double
    return float(lib.ocn_threey(ll, ml, lm, mm, lr, mr, int(bool(conjug))))


def read_slater(path: str, np_: int):
    """fk/gk/kk file -> ((np, np) array as fk(:, :, k), scale)."""
    f = np.zeros(np_ * np_)
    sc = C.c_double(0.0)
    check(load().ocn_read_slater(path.encode(), np_, _dp(f), C.byref(sc)))
    return f.reshape(np_, np_, order="F"), sc.value


def read_rpottrim(path: str):
    lib = load()
    n = C.c_int(0)
    check(lib.ocn_read_rpottrim(path.encode(), C.byref(n), None, None, 0))
    p, r = np.zeros(n.value), np.zeros(n.value)
    check(lib.ocn_read_rpottrim(path.encode(), C.byref(n), _dp(p), _dp(r), n.value))
    return p, r


def read_energies(path: str, nspn: int = 1):
    """wvfcninfo -> energies of shape (nspn, nq, nbd) in C order (Fortran (nbd, nq, nspn))."""
    lib = load()
    nbd, nq = C.c_int(0), C.c_int(0)
    check(lib.ocn_read_energies(path.encode(), nspn, C.byref(nbd), C.byref(nq), None, C.c_size_t(0)))
    e = np.zeros((nspn, nq.value, nbd.value))
    check(lib.ocn_read_energies(path.encode(), nspn, C.byref(nbd), C.byref(nq), _dp(e), C.c_size_t(e.size)))
    return e


def read_cks(path: str, stream: bool, nptot: int, nb: int, nkpts: int, nspn: int = 1):
    """cksc / parcksc -> (pcr, pci) of shape (nspn, nkpts, nb, nptot) in C order."""
    pr, pi = np.zeros((nspn, nkpts, nb, nptot)), np.zeros((nspn, nkpts, nb, nptot))
    check(load().ocn_read_cks(path.encode(), int(stream), nptot, nb, nkpts, nspn, _dp(pr), _dp(pi)))
    return pr, pi


def cks_to_mpc(lmin: int, lmax: int, nproj, pcr, pci):
    """(nspn, nkpts, nb, nptot) coefficients -> mpcr/mpci of shape
    (nspn, lmax-lmin+1, 2*lmax+1, npmax, nkpts, nb) in C order."""
    nspn, nkpts, nb, _ = pcr.shape
    npj = np.ascontiguousarray(nproj, dtype=np.int32)
    npmax = int(npj.max())
    shape = (nspn, lmax - lmin + 1, 2 * lmax + 1, npmax, nkpts, nb)
    mr, mi = np.zeros(shape), np.zeros(shape)
    check(load().ocn_cks_to_mpc(lmin, lmax, npj.ctypes.data_as(IP), nb, nkpts, nspn, _dp(_f64(pcr)), _dp(_f64(pci)),
                                _dp(mr), _dp(mi)))
    return mr, mi


def read_cmel(path: str, nproj: int) -> np.ndarray:
    """cmel<l> -> mpm block (nproj, nproj) as mpm[nu', nu] (C index [nu][nu'] of the Fortran column-major fill)."""
    m = np.zeros((nproj, nproj))
    check(load().ocn_read_cmel(path.encode(), nproj, _dp(m)))
    return m


def redtrid(n: int, ra, rb) -> np.ndarray:
    w = np.zeros(n + 1)
    check(load().ocn_redtrid(n, _dp(_f64(ra)), _dp(_f64(rb)), _dp(w)))
    return w


def pnorm(pr, pi, nkpts: int, celvol: float):
    pr = _f64(pr).copy()
    pi = _f64(pi).copy()
    kp = C.c_double(0.0)
    check(load().ocn_psi_pnorm(len(pr), nkpts, C.c_double(celvol), _dp(pr), _dp(pi), C.byref(kp)))
    return pr, pi, kp.value


# ---------------------------------------------------------------- valence BSE

class OcnValDims(C.Structure):
    _fields_ = [("nc", C.c_int), ("nv", C.c_int), ("kmesh", C.c_int * 3), ("xmesh", C.c_int * 3),
                ("precision", C.c_int), ("device", C.c_int), ("nspn", C.c_int), ("vspin", C.c_int)]


def val_last_error(ctx=None) -> str:
    buf = C.create_string_buffer(1024)
    load().ocn_val_last_error(ctx, buf, 1024)
    return buf.value.decode(errors="replace")


def val_bubble(xmesh, bvec, qinb, celvol: float, nkpts: int):
    """bubble(x) of AI_bubble_populate (host code of the library); returns (bubble, ngvec)."""
    out = np.zeros(int(np.prod(xmesh)))
    ng = C.c_int(0)
    rc = load().ocn_val_bubble_populate((C.c_int * 3)(*xmesh), (C.c_double * 9)(*list(bvec)),
                                        (C.c_double * 3)(*list(qinb)), C.c_double(celvol), int(nkpts), _dp(out),
                                        C.byref(ng))
    if rc != 0:
        raise OcnError(rc, val_last_error())
    return out, ng.value


def val_fxc_from_rho(rho, celvol: float, nkpts: int):
    """OCEAN_fxc_prep's ALDA kernel on the x-mesh (host code of the library)."""
    r = _f64(rho)
    out = np.zeros(len(r))
    rc = load().ocn_val_fxc_from_rho(len(r), _dp(r), C.c_double(celvol), int(nkpts), _dp(out))
    if rc != 0:
        raise OcnError(rc, val_last_error())
    return out


class ValContext:
    """One valence BSE problem on one GPU: the module state of OCEAN_val_states,
    OCEAN_val_energy, OCEAN_bubble and OCEAN_ladder, and the valence action."""

    def __init__(self, w, precision: int = OCN_PREC_FP64, device: int = 0):
        lib = load()
        self.w = w
        self.lib = lib
        d = OcnValDims()
        d.nc, d.nv = w.nc, w.nv
        d.kmesh[:] = list(w.kmesh)
        d.xmesh[:] = list(w.xmesh)
        d.precision = precision
        d.device = device
        d.nspn = getattr(w, "nspn", 1)
        d.vspin = getattr(w, "vspin", 1)
        self.ptr = C.c_void_p()
        rc = lib.ocn_val_create(C.byref(d), C.byref(self.ptr))
        if rc != 0:
            raise OcnError(rc, val_last_error())
        try:
            self._chk(lib.ocn_val_set_energies(self.ptr, _dp(_f64(w.er)), _dp(_f64(w.ei))))
            self._chk(lib.ocn_val_set_allow(self.ptr, _dp(_f64(w.allow))))
            self.bubble, self.ngvec = val_bubble(w.xmesh, w.bvec, w.qinb, w.celvol, w.nk)
            self._chk(lib.ocn_val_set_bubble(self.ptr, _dp(self.bubble)))
            if getattr(w, "rho", None) is not None:
                self.fxc = val_fxc_from_rho(w.rho, w.celvol, w.nk)
                self._chk(lib.ocn_val_set_fxc(self.ptr, _dp(self.fxc)))
            if w.conr is not None:
                self._chk(lib.ocn_val_set_states(self.ptr, _dp(_f64(w.conr)), _dp(_f64(w.coni)),
                                                 _dp(_f64(w.valr)), _dp(_f64(w.vali))))
                self._chk(lib.ocn_val_set_ladder(self.ptr, _dp(_f64(w.ladder))))
            else:
                a = w.device_arrays
                self._chk(lib.ocn_val_set_states_dev(self.ptr, *[C.c_void_p(a[k].data_ptr()) for k in
                                                                 ("conr", "coni", "valr", "vali")]))
                self._chk(lib.ocn_val_set_ladder_dev(self.ptr, C.c_void_p(a["ladder"].data_ptr())))
        except Exception:
            self.close()
            raise

    def _chk(self, rc):
        if rc != 0:
            raise OcnError(rc, val_last_error(self.ptr))

    def close(self):
        if self.ptr:
            self.lib.ocn_val_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self.lib.ocn_val_kernel_launches(self.ptr))

    @property
    def stream(self) -> int:
        return int(self.lib.ocn_val_stream(self.ptr) or 0)

    def apply_H(self, pr, pi, flags=(1, 1, 1), backwards=False):
        n = self.w.npsi
        hr, hi = np.zeros(n), np.zeros(n)
        self._chk(self.lib.ocn_val_apply_H(self.ptr, _dp(_f64(pr)), _dp(_f64(pi)), _dp(hr), _dp(hi),
                                           (C.c_int * 3)(*flags), int(bool(backwards))))
        return hr, hi

    def apply_H_dev(self, d_in: int, d_out: int, flags=(1, 1, 1), backwards=False):
        self._chk(self.lib.ocn_val_apply_H_dev(self.ptr, C.c_void_p(d_in), C.c_void_p(d_out),
                                               (C.c_int * 3)(*flags), int(bool(backwards))))

    def gmres(self, energies_ev, depth=80, resolution=None, preconditioner=0.5, tol=1e-6, max_restarts=50,
              flags=(1, 1, 1)):
        """GMRES over the valence action (ocn_val_gmres): out_re, out_im, rel_err, iters."""
        w = self.w
        e = _f64(energies_ev)
        n = len(e)
        p = OcnGmresParams()
        p.depth = depth
        p.resolution = w.gam0 if resolution is None else resolution
        p.preconditioner = preconditioner
        p.convergence = tol
        p.max_restarts = max_restarts
        ore, oim, rel = np.zeros(n), np.zeros(n), np.zeros(n)
        its = np.zeros(n, dtype=np.int32)
        self._chk(self.lib.ocn_val_gmres(self.ptr, _dp(_f64(w.psi_r)), _dp(_f64(w.psi_i)), C.c_double(w.kpref),
                                         C.c_double(w.celvol), _dp(e), n, C.byref(p), (C.c_int * 3)(*flags),
                                         _dp(ore), _dp(oim), _dp(rel), its.ctypes.data_as(IP)))
        return ore, oim, rel, its

    def haydock(self, niter: int, pr=None, pi=None, flags=(1, 1, 1)):
        w = self.w
        pr = _f64(w.psi_r if pr is None else pr)
        pi = _f64(w.psi_i if pi is None else pi)
        ra, ia, rb = np.zeros(niter + 1), np.zeros(niter + 1), np.zeros(niter + 1)
        done = C.c_int(0)
        self._chk(self.lib.ocn_val_haydock(self.ptr, _dp(pr), _dp(pi), niter, (C.c_int * 3)(*flags), _dp(ra),
                                           _dp(ia), _dp(rb), C.byref(done)))
        return ra, ia, rb, done.value

    def haydock_dev(self, niter: int, d_psi0: int, flags=(1, 1, 1)):
        ra, ia, rb = np.zeros(niter + 1), np.zeros(niter + 1), np.zeros(niter + 1)
        done = C.c_int(0)
        self._chk(self.lib.ocn_val_haydock_dev(self.ptr, C.c_void_p(d_psi0), niter, (C.c_int * 3)(*flags),
                                               _dp(ra), _dp(ia), _dp(rb), C.byref(done)))
        return ra, ia, rb, done.value


class OcnValCfParams(C.Structure):
    _fields_ = [("kpref", C.c_double), ("ucvol", C.c_double), ("el", C.c_double), ("eh", C.c_double),
                ("gam0", C.c_double), ("ne", C.c_int), ("val_ham_spin", C.c_int), ("semi_tda", C.c_int),
                ("backf", C.c_int)]


def val_spectrum(ra, ia, rb, iteration: int, kpref: float, ucvol: float, el: float, eh: float, ne: int,
                 gam0: float, val_ham_spin: int = 1, semi_tda: bool = False, backf: bool = False,
                 ib=None, rc=None, ic=None):
    """write_val rows (ne x 8: omega eV, eps1, eps2, Re n - 1, Im n, mu, R, epsinv) on the GPU."""
    p = OcnValCfParams(kpref, ucvol, el, eh, gam0, ne, val_ham_spin, int(bool(semi_tda)), int(bool(backf)))
    out = np.zeros(ne * 8)
    opt = [None if a is None else _f64(a) for a in (ia, ib, rc, ic)]
    ptr = [None if a is None else _dp(a) for a in opt]
    check(load().ocn_val_spectrum(_dp(_f64(ra)), ptr[0], _dp(_f64(rb)), ptr[1], ptr[2], ptr[3], int(iteration),
                                  C.byref(p), _dp(out)))
    return out.reshape(ne, 8)


def val_optical_constants(omega_ha, eps_re, eps_im):
    om, er, ei = _f64(omega_ha), _f64(eps_re), _f64(eps_im)
    out = np.zeros(len(om) * 8)
    check(load().ocn_val_optical_constants(len(om), _dp(om), _dp(er), _dp(ei), _dp(out)))
    return out.reshape(len(om), 8)


def write_opcons(path: str, rows):
    r = _f64(np.asarray(rows).reshape(-1))
    check(load().ocn_write_opcons(path.encode(), len(r) // 8, _dp(r)))


def read_val_u2(path: str, xmesh, nkpts: int, nspn: int, file_b0: int, file_b1: int, band_lo: int, nb: int):
    """val.u2.dat / con.u2.dat -> (re, im) flat arrays in the ocn_val_set_states layout."""
    n = int(np.prod(xmesh)) * nb * nkpts * nspn
    re, im = np.zeros(n), np.zeros(n)
    check(load().ocn_read_val_u2(path.encode(), (C.c_int * 3)(*xmesh), nkpts, nspn, file_b0, file_b1, band_lo, nb,
                                 _dp(re), _dp(im)))
    return re, im


def val_pair_energies(nc, nv, nkpts, nspn, vspin, con_e, ncon_file, con_lo, val_e, nval_file, val_lo):
    out = np.zeros(nc * nv * nkpts * vspin * vspin)
    check(load().ocn_val_pair_energies(nc, nv, nkpts, nspn, vspin, _dp(_f64(con_e)), ncon_file, con_lo,
                                       _dp(_f64(val_e)), nval_file, val_lo, _dp(out)))
    return out
