"""Seeded synthetic workloads for the OCEAN core-level BSE hot path.

The reference ships none of the pipeline files its BSE solver reads (u2.dat,
rpottrim.*, wvfcninfo, cks*, Slater files), so these generators stand in for
them with the shapes and value distributions of the five benchmark cases:

  c1  cubic a = 4.0 A, k-mesh 4^3, 32 bands, x-mesh 8^3, 1s edge (Na = 4)
  c2  k-mesh 8^3, 100 bands, x-mesh 12^3, 1s edge
  c3  2p edge with multiplets and spin-orbit (Na = 12), k-mesh 6^3, 64 bands,
      x-mesh 10^3, projectors l = 0..3 x 8 radial
  c4  uneven batched instances (k-mesh from {4^3,5^3,6^3,8^3}, 24..128 bands)
  c5  c2 sizes for the adjoint-gradient study

Value recipe (identical bytes are fed to the oracle and the GPU library):
  * band energies  U(0, 30) eV sorted per k, converted to Hartree, Sigma'' = 0
  * allow mask     1
  * u2 per k       QR-orthonormalised complex Gaussian (Nx x Nb), raw (before the
                   core-hole phase of OCEAN_bloch_lrLOAD)
  * W(r)           rpottrim-style table of 64 samples of erf(r/0.5 A)/(eps r),
                   eps = 4, on 0..10 Bohr; beyond the table lr_populate_W2 uses
                   1/(eps r) itself.  The table is positive: long_range.f90:943-961
                   subtracts conj(u) phi, which supplies the attraction.
  * psi0           complex Gaussian normalised by core_pnorm (kpref returned)
  * multiplet      (c3) projector coefficients complex Gaussian / sqrt(Nb Nk);
                   monopole matrices mpm and the Slater integrals F^k, G^k
                   U(0.5, 8) eV, symmetric in the radial indices; the exchange
                   matrices built from F^k, G^k by the library's restatement of
                   nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181)

Everything is in Hartree / Bohr, the units ocean.x works in.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

# OCEAN2/OCEAN_constants.f90:15-20
EV2HARTREE = 0.036749322175666
HARTREE2EV = 27.211386245980
BOHR = 0.529177210544  # Angstrom per Bohr


@dataclass
class Workload:
    name: str
    nb: int
    kmesh: tuple
    xmesh: tuple
    na: int
    nspn: int
    core_l: int
    celvol: float
    avec: np.ndarray            # (9,) Fortran avec(3,3), Bohr
    tau: np.ndarray             # (3,)
    epsilon0: float
    interaction_scale: float
    rtab: np.ndarray
    ptab: np.ndarray
    er: np.ndarray              # (Nb*Nk*Na,) Fortran order
    ei: np.ndarray
    allow: np.ndarray
    ur: np.ndarray              # raw u2 (Nb*Nk*Nx*nspn,)
    ui: np.ndarray
    psi_r: np.ndarray           # normalised psi0
    psi_i: np.ndarray
    kpref: float
    # Haydock / spectrum settings
    niter: int = 200
    gam0: float = 0.5 * EV2HARTREE
    ne: int = 2000
    el: float = -10.0 * EV2HARTREE
    eh: float = 40.0 * EV2HARTREE
    # GMRES settings
    gmres_nomega: int = 0
    gmres_tol: float = 1e-6
    gmres_depth: int = 80
    gmres_gprc: float = 0.5
    # multiplet / spin-orbit (None when off)
    mult: Optional[dict] = None
    so_xi: float = 0.0
    extra: dict = field(default_factory=dict)

    @property
    def nk(self) -> int:
        return int(np.prod(self.kmesh))

    @property
    def nx(self) -> int:
        return int(np.prod(self.xmesh))

    @property
    def npsi(self) -> int:
        return self.nb * self.nk * self.na


def w_table(epsilon0: float = 4.0, width_angstrom: float = 0.5, nptab: int = 64,
            rmax_bohr: float = 10.0):
    """rpottrim-style table of the screened core-hole potential erf(r/a)/(eps r)."""
    a = width_angstrom / BOHR
    rtab = np.linspace(0.0, rmax_bohr, nptab)
    ptab = np.empty_like(rtab)
    for i, r in enumerate(rtab):
        if r == 0.0:
            ptab[i] = 2.0 / (a * math.sqrt(math.pi) * epsilon0)
        else:
            ptab[i] = math.erf(r / a) / (epsilon0 * r)
    return rtab, ptab


def pnorm(psi_r: np.ndarray, psi_i: np.ndarray, nkpts: int, celvol: float):
    """core_pnorm (OCEAN_psi.f90:5589-5638): normalise and return kpref."""
    val = math.sqrt(float(np.sum(psi_r * psi_r + psi_i * psi_i)))
    kpref = 4.0 * math.pi * val * val / (nkpts * celvol * celvol)
    return psi_r / val, psi_i / val, kpref


def _orthonormal_u2(rng, nk: int, nx: int, nb: int, nspn: int):
    """u2 per k = Q of a QR of an (Nx x Nb) complex Gaussian; returns Fortran
    (Nb, Nk, Nx, nspn) planes flattened."""
    ur = np.empty((nspn, nx, nk, nb), dtype=np.float64)
    ui = np.empty_like(ur)
    for s in range(nspn):
        chunk = 64
        for k0 in range(0, nk, chunk):
            k1 = min(nk, k0 + chunk)
            g = rng.standard_normal((k1 - k0, nx, nb)) + 1j * rng.standard_normal((k1 - k0, nx, nb))
            q, _ = np.linalg.qr(g)
            # q[k, x, n] -> u(n, k, x)
            ur[s, :, k0:k1, :] = np.transpose(q.real, (1, 0, 2))
            ui[s, :, k0:k1, :] = np.transpose(q.imag, (1, 0, 2))
    return ur.reshape(-1), ui.reshape(-1)


def _orthonormal_u2_torch(seed: int, nk: int, nx: int, nb: int, nspn: int, device: str):
    """Same distribution as _orthonormal_u2, drawn and factorised on a GPU with
    torch (the batched-instance sets are too large for host QR in a benchmark)."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(1_000_003 * seed + 17)
    ur = np.empty((nspn, nx, nk, nb), dtype=np.float64)
    ui = np.empty_like(ur)
    chunk = max(1, min(nk, (1 << 27) // max(1, nx * nb)))
    for s in range(nspn):
        for k0 in range(0, nk, chunk):
            k1 = min(nk, k0 + chunk)
            g = torch.complex(torch.randn((k1 - k0, nx, nb), generator=gen, device=device, dtype=torch.float64),
                              torch.randn((k1 - k0, nx, nb), generator=gen, device=device, dtype=torch.float64))
            q, _ = torch.linalg.qr(g)
            q = q.permute(1, 0, 2).contiguous()
            ur[s, :, k0:k1, :] = q.real.cpu().numpy()
            ui[s, :, k0:k1, :] = q.imag.cpu().numpy()
    return ur.reshape(-1), ui.reshape(-1)


def batch_instance(i: int, u2_device: Optional[str] = None) -> "Workload":
    """Instance i of the batched uneven set: k-mesh n^3 with n in {4,5,6,8},
    bands U{24..128}, 1s or 2p edge, x-mesh m^3 with m in 8..12, seed i."""
    rng = np.random.Generator(np.random.PCG64(10_000 + i))
    n = int(rng.choice([4, 5, 6, 8]))
    nb = int(rng.integers(24, 129))
    lc = int(rng.integers(0, 2))
    m = int(rng.integers(8, 13))
    return make("batch", seed=i, nb=nb, kmesh=(n, n, n), xmesh=(m, m, m), core_l=lc, with_mult=False,
                u2_device=u2_device)


def _library():
    """The library (built in-tree when missing): the multiplet workloads take
    their exchange matrices from its nbsemhsetup2 restatement."""
    from ocean_gb300 import capi

    try:
        capi.load()
    except RuntimeError:
        from ocean_gb300 import build

        build.build()
        capi.load()


def make(name: str, seed: int = 0, nb: Optional[int] = None, kmesh=None, xmesh=None,
         core_l: Optional[int] = None, with_mult: Optional[bool] = None,
         u2_device: Optional[str] = None, nspn: int = 1) -> Workload:
    """Build a named workload: 'c1', 'c2', 'c3', 'c5', 'batch' (shape given by the
    caller), or 'tiny' (test sizes).  u2_device: draw u2 on that torch device;
    nspn = 2 gives spin-polarised Bloch functions (valence spin = alpha mod 2)."""
    presets = {
        "tiny": dict(nb=8, kmesh=(2, 2, 2), xmesh=(3, 3, 3), core_l=0, mult=False, niter=24),
        "small": dict(nb=12, kmesh=(3, 2, 2), xmesh=(4, 3, 2), core_l=0, mult=False, niter=40),
        "c1": dict(nb=32, kmesh=(4, 4, 4), xmesh=(8, 8, 8), core_l=0, mult=False, niter=200),
        "c2": dict(nb=100, kmesh=(8, 8, 8), xmesh=(12, 12, 12), core_l=0, mult=False, niter=1000,
                   gmres_nomega=200),
        # c2 k-mesh and bands on an 8^3 x-mesh: the profiling case (~1.3 GB on the device)
        "c2s": dict(nb=100, kmesh=(8, 8, 8), xmesh=(8, 8, 8), core_l=0, mult=False, niter=100),
        "c3": dict(nb=64, kmesh=(6, 6, 6), xmesh=(10, 10, 10), core_l=1, mult=True, niter=200),
        "c3small": dict(nb=16, kmesh=(2, 2, 3), xmesh=(4, 4, 4), core_l=1, mult=True, niter=40),
        "c5": dict(nb=100, kmesh=(8, 8, 8), xmesh=(12, 12, 12), core_l=0, mult=False, niter=1000,
                   gmres_nomega=400),
        "batch": dict(nb=32, kmesh=(4, 4, 4), xmesh=(8, 8, 8), core_l=0, mult=False, niter=500),
    }
    if name not in presets:
        raise ValueError(f"unknown workload {name!r}")
    p = dict(presets[name])
    if nb is not None:
        p["nb"] = nb
    if kmesh is not None:
        p["kmesh"] = tuple(kmesh)
    if xmesh is not None:
        p["xmesh"] = tuple(xmesh)
    if core_l is not None:
        p["core_l"] = core_l
    if with_mult is not None:
        p["mult"] = with_mult

    rng = np.random.Generator(np.random.PCG64(seed))
    nbv, km, xm, lc = p["nb"], tuple(p["kmesh"]), tuple(p["xmesh"]), p["core_l"]
    na = 4 * (2 * lc + 1)
    if nspn not in (1, 2):
        raise ValueError("nspn must be 1 or 2")
    nk, nx = int(np.prod(km)), int(np.prod(xm))
    a_bohr = 4.0 / BOHR
    avec = np.zeros(9)
    avec[0] = avec[4] = avec[8] = a_bohr
    celvol = a_bohr ** 3
    eps0 = 4.0
    rtab, ptab = w_table(eps0)

    # energies: U(0,30) eV sorted per k, (Nb, Nk) -> stubby to (Nb, Nk, Na)
    e = np.sort(rng.uniform(0.0, 30.0, size=(nk, nbv)), axis=1) * EV2HARTREE
    er = np.broadcast_to(e[None, :, :], (na, nk, nbv)).reshape(-1).copy()
    ei = np.zeros_like(er)
    allow = np.ones_like(er)

    if u2_device is None:
        ur, ui = _orthonormal_u2(rng, nk, nx, nbv, nspn)
    else:
        ur, ui = _orthonormal_u2_torch(seed, nk, nx, nbv, nspn, u2_device)

    g_r = rng.standard_normal(na * nk * nbv)
    g_i = rng.standard_normal(na * nk * nbv)
    psi_r, psi_i, kpref = pnorm(g_r, g_i, nk, celvol)

    w = Workload(name=name, nb=nbv, kmesh=km, xmesh=xm, na=na, nspn=nspn, core_l=lc,
                 celvol=celvol, avec=avec, tau=np.zeros(3), epsilon0=eps0,
                 interaction_scale=1.0, rtab=rtab, ptab=ptab, er=er, ei=ei, allow=allow,
                 ur=ur, ui=ui, psi_r=psi_r, psi_i=psi_i, kpref=kpref, niter=p["niter"],
                 gmres_nomega=p.get("gmres_nomega", 0))

    if p["mult"]:
        lmin, lmax, nproj = 0, 3, [8, 8, 8, 8]
        if name == "c3small":
            nproj = [2, 2, 2, 2]
        npmax = max(nproj)
        nl = lmax - lmin + 1
        shape = (nspn, nl, 2 * lmax + 1, npmax, nk, nbv)  # C order of Fortran mpc
        scale = 1.0 / math.sqrt(nbv * nk)
        mpcr = rng.standard_normal(shape) * scale
        mpci = rng.standard_normal(shape) * scale
        # zero the unused (m, nu) slots so both sides see identical padding
        for li, l in enumerate(range(lmin, lmax + 1)):
            for mi in range(2 * lmax + 1):
                m = mi - lmax
                if abs(m) > l:
                    mpcr[:, li, mi] = 0.0
                    mpci[:, li, mi] = 0.0
            mpcr[:, li, :, nproj[li]:] = 0.0
            mpci[:, li, :, nproj[li]:] = 0.0
        mpm = np.zeros((nl, npmax, npmax))
        for li in range(nl):
            npl = nproj[li]
            f = rng.uniform(0.5, 8.0, size=(npl, npl))
            mpm[li, :npl, :npl] = 0.5 * (f + f.T) * EV2HARTREE
        # exchange matrices from Slater radial integrals F^k, G^k ~ U(0.5, 8) eV
        # (symmetric in the two radial indices) through nbsemhsetup2's angular
        # algebra (OCEAN_multiplet.f90:2007-2181), as the library builds them
        from ocean_gb300 import capi

        _library()
        mh_r, mh_i = [], []
        for li, l in enumerate(range(lmin, lmax + 1)):
            npl = nproj[li]

            def slater():
                a = rng.uniform(0.5, 8.0, size=(npl, npl))
                return 0.5 * (a + a.T)

            fk = {k: slater() for k in range(2, min(2 * lc, 2 * l) + 1, 2)}
            gk = {k: slater() for k in range(abs(lc - l), lc + l + 1, 2)}
            mr, mi = capi.mult_exchange(lc, l, fk, gk)
            mh_r.append(mr)
            mh_i.append(mi)
        w.mult = dict(lmin=lmin, lmax=lmax, nproj=np.array(nproj, dtype=np.int32), npmax=npmax,
                      mpcr=mpcr.reshape(-1), mpci=mpci.reshape(-1),
                      mpm=mpm.reshape(-1), mhr=np.concatenate(mh_r), mhi=np.concatenate(mh_i))
        w.so_xi = 5.0 * EV2HARTREE
    return w


# ------------------------------------------------------------------ valence BSE
#
# Synthetic stand-ins for the valence BSE inputs (OCEAN_val_states' real-space
# states, OCEAN_val_energy's pair energies, OCEAN_WRR's ladder):
#   * states per k   one QR-orthonormal complex Gaussian (Nx x (Nv + Nc)):
#                    the first Nv columns are val(x, v, k), the rest con(x, c, k)
#   * energies       E(c, v, k) = e_c(k) - e_v(k), e_v ~ U(-8, 0) eV and
#                    e_c ~ U(1, 16) eV sorted per k, Hartree, Sigma'' = 0
#   * allow          1
#   * bubble         built by the library from the cubic cell (a = 4.0 A)
#   * ladder(R,x,y)  W(|R + x - y|) fcn(q |R + x - y|)^2 with W = erf(r/0.5 A)/(eps r),
#                    eps = 4, and the smoothing of OCEAN_WRR_LocalRPA
#                    (OCEAN_WRR.f90:156, 286-304), q = (6 pi^2 / (V Nk))^(1/3);
#                    R runs over the k-mesh's lattice vectors in FFT order
#                    (index j -> j or j - n), and a Nyquist index of an even
#                    mesh averages R = +n/2 and -n/2 so that
#                    ladder(-R, y, x) = ladder(R, x, y) (the direct term is Hermitian).
#   * psi0           complex Gaussian normalised by core_pnorm


@dataclass
class ValWorkload:
    name: str
    nc: int
    nv: int
    kmesh: tuple
    xmesh: tuple
    celvol: float
    avec: np.ndarray          # (9,) Fortran avec(3,3), Bohr
    bvec: np.ndarray          # (9,) Fortran bvec(3,3), Bohr^-1
    qinb: np.ndarray          # (3,)
    epsilon0: float
    er: np.ndarray            # (Nc*Nv*Nk,) Fortran order (c fastest)
    ei: np.ndarray
    allow: np.ndarray
    conr: Optional[np.ndarray]   # (Nx*Nc*Nk,) Fortran order (x fastest), None when on the device
    coni: Optional[np.ndarray]
    valr: Optional[np.ndarray]   # (Nx*Nv*Nk,)
    vali: Optional[np.ndarray]
    ladder: Optional[np.ndarray]  # (Nk*Nx*Nx,) Fortran ladder(k, x, y)
    psi_r: np.ndarray
    psi_i: np.ndarray
    kpref: float
    niter: int = 200
    gam0: float = 0.2 * EV2HARTREE
    el: float = 0.0
    eh: float = 30.0 * EV2HARTREE
    device_arrays: dict = field(default_factory=dict)  # torch tensors when built on a device
    nspn: int = 1              # DFT spins of the states
    vspin: int = 1             # valence_ham_spin: psi has vspin^2 spin blocks
    rho: Optional[np.ndarray] = None  # (Nx) valence density (electrons / Bohr^3); set: the f_xc term is on

    @property
    def nk(self) -> int:
        return int(np.prod(self.kmesh))

    @property
    def nx(self) -> int:
        return int(np.prod(self.xmesh))

    @property
    def npsi(self) -> int:
        return self.nc * self.nv * self.nk * self.vspin * self.vspin


def _mesh_frac(mesh):
    """Fractional positions of a mesh in its flat order (last extent fastest)."""
    g = np.stack(np.meshgrid(*[np.arange(n) / n for n in mesh], indexing="ij"), axis=-1)
    return g.reshape(-1, 3)


def _lattice_images(kmesh):
    """Per flat k index the lattice vectors R (integer, FFT order) it stands for."""
    per_axis = []
    for n in kmesh:
        opts = []
        for j in range(n):
            if n % 2 == 0 and 2 * j == n:
                opts.append((j, j - n))
            else:
                opts.append((j if j < (n + 1) // 2 else j - n,))
        per_axis.append(opts)
    images = []
    for j1 in range(kmesh[0]):
        for j2 in range(kmesh[1]):
            for j3 in range(kmesh[2]):
                images.append([(a, b, c) for a in per_axis[0][j1] for b in per_axis[1][j2]
                               for c in per_axis[2][j3]])
    return images


def val_ladder(kmesh, xmesh, avec, celvol, epsilon0=4.0, width_angstrom=0.5, device=None, dtype=None):
    """ladder(k, x, y) of the synthetic screened interaction as a torch tensor of
    shape (Nx_y, Nx_x, Nk) (= Fortran ladder(k, x, y) flattened), built on `device`."""
    import torch

    dtype = dtype or torch.float64
    nk, nx = int(np.prod(kmesh)), int(np.prod(xmesh))
    a = width_angstrom / BOHR
    q = (6.0 * math.pi ** 2 / (celvol * nk)) ** (1.0 / 3.0)
    A = torch.tensor(np.asarray(avec, dtype=np.float64).reshape(3, 3, order="F"), dtype=torch.float64,
                     device=device)
    fx = torch.tensor(_mesh_frac(xmesh), dtype=torch.float64, device=device)
    images = _lattice_images(kmesh)
    nimg = max(len(i) for i in images)
    R = np.zeros((nk, nimg, 3))
    wts = np.zeros((nk, nimg))
    for k, im in enumerate(images):
        for j, r in enumerate(im):
            R[k, j] = r
            wts[k, j] = 1.0 / len(im)
    R = torch.tensor(R, dtype=torch.float64, device=device)
    wts = torch.tensor(wts, dtype=torch.float64, device=device)
    out = torch.empty((nx, nx, nk), dtype=dtype, device=device)
    for y in range(nx):
        d = fx[:, None, None, :] - fx[y][None, None, None, :] + R[None, :, :, :]
        # d: (x, k, img, 3) fractional -> Cartesian
        cart = torch.einsum("ij,xkmj->xkmi", A, d)
        r = torch.linalg.norm(cart, dim=-1)
        safe = torch.where(r > 0, r, torch.ones_like(r))
        w = torch.where(r > 0, torch.erf(safe / a) / (epsilon0 * safe),
                        torch.full_like(r, 2.0 / (a * math.sqrt(math.pi) * epsilon0)))
        qd = q * r
        qs = torch.where(qd > 1e-6, qd, torch.ones_like(qd))
        fcn = torch.where(qd > 1e-6, 3.0 * (torch.sin(qs) - qs * torch.cos(qs)) / qs ** 3, 1.0 - 0.1 * qd ** 2)
        out[y] = ((w * fcn ** 2) * wts[None, :, :]).sum(-1).to(dtype)
    return out


def make_val(name: str, seed: int = 0, nc: Optional[int] = None, nv: Optional[int] = None, kmesh=None,
             xmesh=None, device: Optional[str] = None, nspn: int = 1, vspin: int = 1,
             with_fxc: bool = False) -> ValWorkload:
    """Valence workloads: 'vtiny', 'vsmall' (oracle sizes), 'v2' (k-mesh 8^3,
    x-mesh 10^3, 8 conduction and 4 valence bands: the benchmark case).
    device: build the states and the ladder as torch tensors there (kept in
    w.device_arrays; the numpy fields are then None).  nspn: DFT spins (states
    and band energies per spin); vspin: valence_ham_spin (psi gets vspin^2
    blocks, block (i, j) pairing valence spin i with conduction spin j)."""
    if nspn not in (1, 2) or vspin not in (1, 2):
        raise ValueError("nspn and vspin must be 1 or 2")
    presets = {
        "vtiny": dict(nc=4, nv=2, kmesh=(2, 2, 2), xmesh=(3, 3, 3), niter=24),
        "vsmall": dict(nc=6, nv=3, kmesh=(4, 4, 4), xmesh=(4, 4, 4), niter=40),
        "vodd": dict(nc=5, nv=3, kmesh=(3, 2, 5), xmesh=(3, 4, 3), niter=30),
        "v2": dict(nc=8, nv=4, kmesh=(8, 8, 8), xmesh=(10, 10, 10), niter=200),
    }
    if name not in presets:
        raise ValueError(f"unknown valence workload {name!r}")
    p = dict(presets[name])
    for key, val in (("nc", nc), ("nv", nv), ("kmesh", kmesh), ("xmesh", xmesh)):
        if val is not None:
            p[key] = tuple(val) if key in ("kmesh", "xmesh") else val
    km, xm = tuple(p["kmesh"]), tuple(p["xmesh"])
    nk, nx = int(np.prod(km)), int(np.prod(xm))
    ncb, nvb = p["nc"], p["nv"]
    if nx < ncb + nvb:
        raise ValueError("x-mesh too small for orthonormal states")
    rng = np.random.Generator(np.random.PCG64(seed))
    a_bohr = 4.0 / BOHR
    avec = np.zeros(9)
    avec[0] = avec[4] = avec[8] = a_bohr
    bvec = np.zeros(9)
    bvec[0] = bvec[4] = bvec[8] = 2.0 * math.pi / a_bohr
    celvol = a_bohr ** 3
    ev = np.sort(rng.uniform(-8.0, 0.0, size=(nspn, nk, nvb)), axis=2)
    ec = np.sort(rng.uniform(1.0, 16.0, size=(nspn, nk, ncb)), axis=2)
    blocks = []
    for iv in range(vspin):          # ibeta = (i - 1) vspin + j: valence spin outer
        for jc in range(vspin):
            sv, sc = min(iv, nspn - 1), min(jc, nspn - 1)
            blocks.append((ec[sc][:, None, :] - ev[sv][:, :, None]) * EV2HARTREE)  # (k, v, c)
    er = np.concatenate([b.reshape(-1) for b in blocks])
    ei = np.zeros_like(er)
    allow = np.ones_like(er)
    g_r = rng.standard_normal(er.size)
    g_i = rng.standard_normal(er.size)
    psi_r, psi_i, kpref = pnorm(g_r, g_i, nk, celvol)
    w = ValWorkload(name=name, nc=ncb, nv=nvb, kmesh=km, xmesh=xm, celvol=celvol, avec=avec, bvec=bvec,
                    qinb=np.zeros(3), epsilon0=4.0, er=er, ei=ei, allow=allow, conr=None, coni=None,
                    valr=None, vali=None, ladder=None, psi_r=psi_r, psi_i=psi_i, kpref=kpref,
                    niter=p["niter"], nspn=nspn, vspin=vspin)
    if with_fxc:  # a smooth density with the mean of 8 valence electrons per cell
        f = _mesh_frac(xm)
        shape = 1.0 + 0.5 * np.prod(np.cos(2.0 * math.pi * f), axis=1)
        w.rho = 8.0 / celvol * shape / shape.mean()
    if device is None:
        st = np.empty((nspn, nk, ncb + nvb, nx), dtype=np.complex128)
        for sp in range(nspn):
            for k in range(nk):
                g = rng.standard_normal((nx, ncb + nvb)) + 1j * rng.standard_normal((nx, ncb + nvb))
                qm, _ = np.linalg.qr(g)
                st[sp, k] = qm.T
        val = st[:, :, :nvb, :]   # (s, k, v, x): Fortran (x, v, k, s) flattened
        con = st[:, :, nvb:, :]
        w.valr, w.vali = val.real.reshape(-1).copy(), val.imag.reshape(-1).copy()
        w.conr, w.coni = con.real.reshape(-1).copy(), con.imag.reshape(-1).copy()
        w.ladder = val_ladder(km, xm, avec, celvol, w.epsilon0).numpy().reshape(-1)
    else:
        import torch

        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        st = torch.empty((nspn, nk, ncb + nvb, nx), dtype=torch.complex128, device=device)
        for sp in range(nspn):
            for k in range(nk):
                g = torch.complex(torch.randn((nx, ncb + nvb), generator=gen, device=device, dtype=torch.float64),
                                  torch.randn((nx, ncb + nvb), generator=gen, device=device, dtype=torch.float64))
                qm, _ = torch.linalg.qr(g)
                st[sp, k] = qm.T
        val = st[:, :, :nvb, :].contiguous()
        con = st[:, :, nvb:, :].contiguous()
        w.device_arrays = dict(valr=val.real.contiguous().reshape(-1), vali=val.imag.contiguous().reshape(-1),
                               conr=con.real.contiguous().reshape(-1), coni=con.imag.contiguous().reshape(-1),
                               ladder=val_ladder(km, xm, avec, celvol, w.epsilon0, device=device).reshape(-1))
    return w
