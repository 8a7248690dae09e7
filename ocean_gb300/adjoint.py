"""Reverse-mode derivatives of the GMRES core-level spectrum.

The spectrum that OCEAN_gmres_do_recycle writes (OCEAN2/OCEAN_gmres.f90:864-869)
is, per energy w,

    out_re(w) = 1 - kpref Re F(w),   out_im(w) = -kpref Im F(w),
    F(w) = <b|x(w)>,  (w + i Gamma - H) x = b,  b = allow o psi0.

GmresSpectrum is a torch.autograd.Function over libocean_gpu.so with four
parameters:

  scale    interactionScale as it multiplies W(R, x) in lr_populate_W2
           (OCEAN2/long_range.f90:1840); the multiplet term is off here, so this
           is the "W scale"
  ptab     the radial table W(r) that lr_populate_W2 interpolates (64 samples)
  gamma    the resolution Gamma of the resolvent (Hartree)
  scissor  a shift s of every energy E -> E + s (the core_offset shift of
           OCEAN2/OCEAN_energies.f90:859-866; Hartree)

forward runs ocn_gmres_dev and keeps every solution x(w) on the device;
backward runs ocn_gmres_vjp (one adjoint GMRES at -Gamma plus one dL/dW map)
and ocn_w2_vjp (the chain rule through the W(r) interpolation).  Nothing here
computes the spectrum itself: every number comes from the library.

Memory: the solutions take 16 Npsi bytes per energy.  When that exceeds
max_stored_bytes (80 GB by default) the energies are taken in windows of at
most max_stored_bytes worth of solutions: forward solves window by window and
keeps nothing, backward solves each window again (the same kernels in the
same order give the same x) and runs the window's adjoint on it.  Each window
starts GMRES afresh (no recycled basis from the previous window), in both
passes, so the stored and the recomputed schedules with the same windows give
identical results.
"""
import dataclasses

import numpy as np
import torch

from . import capi


class GmresProblem:
    """One site on one GPU with the settings of a GMRES spectrum run."""

    def __init__(self, w, energies_ev, precision=capi.OCN_PREC_FP64, device: int = 0, depth: int = 80,
                 tol: float = 1e-6, preconditioner=None, max_restarts: int = 100,
                 max_stored_bytes: float = 80e9, window: int = 0):
        """window > 0 forces windows of that many energies with stored solutions
        (the schedule a recomputing run with the same window follows)."""
        self.w = w
        self.energies = np.ascontiguousarray(energies_ev, dtype=np.float64)
        per_x = 2 * w.npsi * 8
        nw = len(self.energies)
        if nw * per_x > max_stored_bytes:
            self.window = max(1, int(max_stored_bytes // per_x))
            self.recompute = True
        else:
            self.window = window if window > 0 else nw
            self.recompute = False
        self.ctx = capi.Context(w, precision=precision, device=device, set_mult=False)
        self.dev = torch.device(f"cuda:{device}")
        n = w.npsi
        self.d_hay = torch.empty(2 * n, dtype=torch.float64, device=self.dev)
        self.d_hay[:n].copy_(torch.from_numpy(np.ascontiguousarray(w.psi_r)))
        self.d_hay[n:].copy_(torch.from_numpy(np.ascontiguousarray(w.psi_i)))
        self.kw = dict(depth=depth, preconditioner=preconditioner, tol=tol, max_restarts=max_restarts)
        torch.cuda.synchronize(self.dev)

    def set_parameters(self, scale: float, ptab: np.ndarray, scissor: float):
        """Installs W(scale, ptab) and the shifted energies; returns the workload
        view whose ptab / interaction_scale the W table was built from."""
        wv = dataclasses.replace(self.w, ptab=np.ascontiguousarray(ptab, dtype=np.float64),
                                 interaction_scale=float(scale))
        W, _, _ = capi.w2_host(wv)
        self.ctx.set_W(W)
        self.ctx.set_energies(self.w.er + float(scissor), self.w.ei)
        return wv

    def close(self):
        self.ctx.close()


class GmresSpectrum(torch.autograd.Function):
    """(scale, ptab, gamma, scissor) -> (out_re, out_im) of the GMRES spectrum."""

    @staticmethod
    def forward(fctx, scale, ptab, gamma, scissor, prob: GmresProblem):
        n = prob.w.npsi
        nw = len(prob.energies)
        wv = prob.set_parameters(float(scale), ptab.detach().cpu().numpy(), float(scissor))
        nwin = prob.window
        keep = not prob.recompute
        d_x = torch.empty((nw if keep else nwin) * 2 * n, dtype=torch.float64, device=prob.dev)
        ore, oim, its = np.zeros(nw), np.zeros(nw), np.zeros(nw, dtype=np.int32)
        for w0 in range(0, nw, nwin):
            w1 = min(nw, w0 + nwin)
            dst = d_x.data_ptr() + (w0 * 2 * n * 8 if keep else 0)
            ore[w0:w1], oim[w0:w1], _, its[w0:w1] = prob.ctx.gmres_dev(
                prob.d_hay.data_ptr(), prob.energies[w0:w1], resolution=float(gamma), d_x=dst, **prob.kw)
        fctx.prob, fctx.wv, fctx.gamma = prob, wv, float(gamma)
        fctx.d_x = d_x if keep else None
        fctx.params = (float(scale), ptab.detach().cpu().numpy().copy(), float(scissor))
        fctx.iterations = its
        return torch.from_numpy(ore), torch.from_numpy(oim)

    @staticmethod
    def backward(fctx, g_re, g_im):
        prob, wv = fctx.prob, fctx.wv
        w = prob.w
        n = w.npsi
        nw = len(prob.energies)
        # the operator of this forward pass (another forward may have run since)
        prob.set_parameters(*fctx.params)
        d_gW = torch.empty(w.nk * w.nx, dtype=torch.float64, device=prob.dev)
        G = torch.zeros(w.nk * w.nx, dtype=torch.float64, device=prob.dev)
        gr = np.zeros(nw) if g_re is None else g_re.detach().cpu().numpy().astype(np.float64)
        gi = np.zeros(nw) if g_im is None else g_im.detach().cpu().numpy().astype(np.float64)
        g_gamma, g_scissor = 0.0, 0.0
        d_x = fctx.d_x
        if d_x is None:
            d_x = torch.empty(prob.window * 2 * n, dtype=torch.float64, device=prob.dev)
        for w0 in range(0, nw, prob.window):
            w1 = min(nw, w0 + prob.window)
            if fctx.d_x is None:  # solve the window again
                prob.ctx.gmres_dev(prob.d_hay.data_ptr(), prob.energies[w0:w1], resolution=fctx.gamma,
                                   d_x=d_x.data_ptr(), **prob.kw)
                src = d_x.data_ptr()
            else:
                src = d_x.data_ptr() + w0 * 2 * n * 8
            gg, gs = prob.ctx.gmres_vjp(prob.d_hay.data_ptr(), prob.energies[w0:w1], src, d_gW.data_ptr(),
                                        grad_re=gr[w0:w1], grad_im=gi[w0:w1], resolution=fctx.gamma, **prob.kw)
            g_gamma += gg
            g_scissor += gs
            G += d_gW
            torch.cuda.current_stream(prob.dev).synchronize()  # before the next call clears d_gW
        G = G.cpu().numpy()
        g_ptab, g_scale = capi.w2_vjp(wv, G)
        dt = torch.float64
        return (torch.tensor(g_scale, dtype=dt), torch.from_numpy(g_ptab), torch.tensor(g_gamma, dtype=dt),
                torch.tensor(g_scissor, dtype=dt), None)


def gmres_spectrum(prob: GmresProblem, scale, ptab, gamma, scissor):
    """Differentiable (out_re, out_im) over prob.energies."""
    return GmresSpectrum.apply(scale, ptab, gamma, scissor, prob)
