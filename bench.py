"""Benchmark of the BSE hot path: Haydock spectra of the 8x8x8 k-mesh, 100-band,
12^3 x-mesh 1s-edge workload (Nk=512, Nb=100, Nx=1728, Na=4), one step = one full
Haydock run (1000 Lanczos iterations, each one H*psi) plus its 2001-point
continued-fraction spectrum.

Our arm (default):  libocean_gpu.so through its C ABI.
  value  H*psi/s with psi0 resident in HBM (ocn_haydock_dev), device time from
         CUDA events on the library's stream.
  e2e    the same through ocn_haydock + ocn_spectrum_cf with host buffers
         (pinned psi0 uploaded and coefficients / spectrum read back every step).
Reference arm (--impl reference): the reference's algorithm restated on the host
  cores (the oracle, OpenMP, FP64): the reference itself is Fortran+MPI+FFTW+LAPACK
  and cannot be built in this environment.

Multi-GPU: the path does not shard in this design (replicas only); each rank runs
an independent replica with its own seed and value sums the ranks' H*psi.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H*psi/s (Haydock, 8^3 k, 100 bands, 12^3 x-mesh, 1s edge)"
UNIT = "H*psi/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("OCN_BENCH_PRECISION", "mixed"),
                    choices=["fp64", "mixed"])
    ap.add_argument("--niter", type=int, default=1000)
    ap.add_argument("--ne", type=int, default=2000)
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--autotune", action="store_true",
                    help="the library's tile autotuner for the main and block legs (default tiles otherwise: the "
                         "tuner times the long-range term alone, and its choice measured no faster in the full step)")
    ap.add_argument("--block", type=int, default=3,
                    help="chains of the block-Haydock leg (polarisations sharing H); 0 = off")
    ap.add_argument("--c1-steps", type=int, default=200,
                    help="Lanczos steps of the 4^3 k / 32-band / 8^3 x leg, with the oracle's full run beside it; 0 = off")
    ap.add_argument("--multiplet-steps", type=int, default=200,
                    help="Lanczos steps of the 2p-edge multiplet leg (c3 sizes); 0 = off")
    ap.add_argument("--nonherm-steps", type=int, default=60,
                    help="steps of the non-Hermitian (two-sided Lanczos) leg on the main workload with a "
                         "lifetime Sigma'' on the bands, both precisions; 0 = off")
    ap.add_argument("--valence-steps", type=int, default=40,
                    help="Lanczos steps of the valence BSE leg (8^3 k, 10^3 x, 8+4 bands; exchange + screened "
                         "direct), both precisions, with the oracle timed on a y-slab; 0 = off")
    ap.add_argument("--valence-xmesh", type=int, default=10,
                    help="x-mesh extent n (n^3 points) of the valence leg (10 = the v2 case)")
    ap.add_argument("--valence-only", action="store_true",
                    help="run the valence leg alone and print its JSON object (profiling)")
    ap.add_argument("--batch", type=int, default=64,
                    help="instances of the batched uneven-Haydock leg (3 polarisations each); 0 = off")
    ap.add_argument("--adjoint-omega", type=int, default=400,
                    help="energies of the adjoint-gradient leg (GMRES forward + reverse); 0 = off")
    ap.add_argument("--gmres-omega", type=int, default=200,
                    help="energies of the GMRES leg (0 disables it)")
    ap.add_argument("--gmres-fp64-omega", type=int, default=50,
                    help="energies (every k-th of the GMRES leg's) solved by both precisions for the "
                         "FP64 comparison; 0 = off")
    ap.add_argument("--gmres-lanes", type=int, default=16,
                    help="energy lanes of the GMRES leg (one block action serves all lanes); the single "
                         "reference-order sweep is timed beside it")
    ap.add_argument("--oracle-steps", type=int, default=200,
                    help="Lanczos steps of the main workload run by the FP64 oracle on the host to state "
                         "the spectral error of both GPU precisions against it; 0 = off")
    ap.add_argument("--batch-fp64", type=int, default=8,
                    help="instances of the batched set run by both precisions (100 steps) for the FP64 "
                         "comparison; 0 = off")
    return ap.parse_args()


def max_over_ranks(pg, value: float, device="cpu") -> float:
    """The slowest rank's value (the whole job's clock); value itself at N=1."""
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_rate(pg, ws: int, local_ms: float, hpsi_per_rank: int, device="cpu"):
    """Replicas: every rank runs its own problem (seed = rank) for the same
    number of H*psi; the job's rate is all ranks' H*psi over the slowest rank's
    time.  Returns (rate in H*psi/s, the slowest rank's ms)."""
    ms = max_over_ranks(pg, local_ms, device)
    return hpsi_per_rank * ws / (ms / 1000.0), ms


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return ws, rank, local, pg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def traffic_summary():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def describe(w) -> str:
    k, x = w.kmesh, w.xmesh
    return (f"Nk={w.nk} ({k[0]}x{k[1]}x{k[2]}), Nb={w.nb}, Nx={w.nx} ({x[0]}x{x[1]}x{x[2]}), "
            f"Na={w.na}")


def algorithmic_bytes(w, cls: str, precision: str, ksplit: int = 2) -> float:
    """Bytes one launch of a long-range kernel must move (read + write).

    FP64 path: u2 (16 B/complex), psi in, phi out (16 B/complex).
    Mixed path: u2 as split-bf16 (8 B/complex); the psi operand B1 and the phi'
    operand B2 are split-bf16 tiles of 4*Na rows; band->x writes FP32 phi; x->band
    writes ksplit FP64 partial planes."""
    nb, nk, nx, na = w.nb, w.nk, w.nx, w.na
    psi = 2 * nb * nk * na * 8
    if precision == "fp64":
        ubytes = nb * nk * nx * w.nspn * 16
        phi = nk * nx * na * 16
        if cls in ("lr_band_to_x", "lr_x_to_band"):
            return ubytes + psi + phi
        if cls == "lr_kmesh_transform":
            return 2 * phi + nk * nx * 8
        return float("nan")
    ubytes = nb * nk * nx * 8
    phi = nk * nx * na * 8
    if cls == "lr_band_to_x":
        return ubytes + nk * 4 * na * 2 * nb * 2 + phi
    if cls == "lr_x_to_band":
        return ubytes + nk * 4 * na * 2 * nx * 2 + ksplit * psi
    if cls == "lr_kmesh_transform":
        return 2 * phi + nk * nx * 4
    return float("nan")


def cpu_baseline(w, seconds: float = 15.0):
    """Oracle H*psi (FP64, all host cores) on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cores = os.cpu_count() or 1
    P = O.OracleProblem(w, nthreads=cores)
    pr, pi = w.psi_r.copy(), w.psi_i.copy()
    P.xact(pr, pi)  # warm-up
    n = 0
    t0 = time.perf_counter()
    while True:
        P.xact(pr, pi)
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    # the same on one core (two applications)
    P1 = O.OracleProblem(w, nthreads=1)
    P1.xact(pr, pi)
    t1 = time.perf_counter()
    for _ in range(2):
        P1.xact(pr, pi)
    dt1 = (time.perf_counter() - t1) / 2
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} oracle H*psi applications (FP64, OpenMP over x-points) of the same "
                      f"workload in {dt:.1f} s",
            "value_1core": 1.0 / dt1}


def run_reference(args, ws, rank, pg):
    from ocean_gb300 import workloads as WL

    if rank != 0:
        return
    w = WL.make(args.workload, seed=0)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cores = os.cpu_count() or 1
    P = O.OracleProblem(w, nthreads=cores)
    sample_iters = 3  # Lanczos iterations per step: bounded sample of the 1000-iteration run
    for _ in range(args.warmup):
        P.haydock(1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        P.haydock(sample_iters)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = sample_iters * args.steps / tot
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded; u2 QR-orthonormal complex Gaussian, U(0,30) eV bands)",
            "config": {"workload": f"{args.workload}: {describe(w)}",
                       "step": f"{sample_iters} Lanczos iterations (bounded sample of the "
                               f"{args.niter}-iteration Haydock run)",
                       "same_config": False,
                       "comparison": "per-H*psi rates: one oracle Lanczos iteration costs the same at "
                                     "every iteration (one H*psi plus O(npsi) vector work), so the "
                                     "sample's rate is the full run's rate"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample_iters} oracle Lanczos iterations per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _device_steps(ctx, w, niter, ne, pr_ptr, pi_ptr, steps, stream, torch):
    """steps full Haydock runs (+ spectra) with psi0 in HBM; CUDA-event ms on the
    library's stream."""
    from ocean_gb300 import capi

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    last = None
    for _ in range(steps):
        ra, ia, rb, done = ctx.haydock_dev(niter, pr_ptr, pi_ptr)
        last = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, ne, w.gam0)
    ev1.record(stream)
    torch.cuda.synchronize()
    ev1.synchronize()
    return ev0.elapsed_time(ev1), last


def run_small(args, torch, capi, WL, local):
    """c1 (4^3 k, 32 bands, 8^3 x, 1s): 200 Lanczos steps + 2001-point spectrum on
    the GPU (both precisions) and the same run by the oracle on all host cores."""
    import time

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    w = WL.make("c1", seed=0)
    niter = args.c1_steps
    out = {"workload": f"c1: {describe(w)}", "steps": niter}
    spec = {}
    for name, prec in (("mixed", capi.OCN_PREC_MIXED), ("fp64", capi.OCN_PREC_FP64)):
        ctx = capi.Context(w, precision=prec, device=local)
        ctx.haydock(niter)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ra, ia, rb, done = ctx.haydock(niter)
        spec[name] = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, args.ne, w.gam0)
        dt = time.perf_counter() - t0
        ctx.close()
        out[name] = {"value": niter / dt, "unit": UNIT, "spectra_per_s": 1.0 / dt}
    cores = os.cpu_count() or 1
    P = O.OracleProblem(w, nthreads=cores)
    t0 = time.perf_counter()
    rc, ora, oia, orb, odone = P.haydock(niter)
    so = O.write_core(ora, oia, orb, odone, w.kpref, w.el, w.eh, args.ne, w.gam0)
    dt = time.perf_counter() - t0
    out["cpu_oracle"] = {"value": niter / dt, "unit": UNIT, "spectra_per_s": 1.0 / dt, "cores": cores,
                         "kind": "port"}
    for name in ("mixed", "fp64"):
        out[name]["spectral_error_vs_oracle"] = float(np.linalg.norm(spec[name][:, 2] - so[:, 2]) /
                                                      np.linalg.norm(so[:, 2]))
    return out


def run_valence(args, torch, capi, WL, local):
    """Valence BSE (exchange + screened direct + pair energies) on the v2 case:
    Haydock H*psi/s of both precisions, the spectral error of the mixed run, the
    direct term's kernel rate, and the oracle's H*psi time estimated from the
    exchange part plus a timed y-slab of the direct term (scaled to all y)."""
    import dataclasses
    import time

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    dev = f"cuda:{local}"
    xm = args.valence_xmesh
    w = WL.make_val("v2", seed=0, device=dev, xmesh=(xm, xm, xm))
    niter = args.valence_steps
    nk, nx, nv = w.nk, w.nx, w.nv
    out = {"workload": f"v2: k-mesh {'x'.join(map(str, w.kmesh))}, x-mesh {'x'.join(map(str, w.xmesh))}, "
                       f"{w.nc} conduction + {nv} valence bands, exchange + screened direct",
           "steps": niter}
    d0 = torch.tensor(np.concatenate([w.psi_r, w.psi_i]), device=dev)
    spec = {}
    for name, prec in (("mixed", capi.OCN_PREC_MIXED), ("fp64", capi.OCN_PREC_FP64)):
        ctx = capi.ValContext(w, precision=prec, device=local)
        ctx.haydock_dev(3, d0.data_ptr())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ra, ia, rb, done = ctx.haydock_dev(niter, d0.data_ptr())
        dt = time.perf_counter() - t0
        # the direct term alone: H psi with and without it, CUDA events on the context stream
        st = torch.cuda.ExternalStream(ctx.stream)
        hx = torch.empty_like(d0)
        ms = {}
        for key, flags in (("all", (1, 1, 1)), ("no_direct", (1, 1, 0))):
            reps = 5 if name == "mixed" else 2
            ctx.apply_H_dev(d0.data_ptr(), hx.data_ptr(), flags=flags)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                ctx.apply_H_dev(d0.data_ptr(), hx.data_ptr(), flags=flags)
            e1.record(st)
            torch.cuda.synchronize()
            ms[key] = e0.elapsed_time(e1) / reps
        ctx.close()
        spec[name] = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, args.ne, w.gam0)
        direct_ms = ms["all"] - ms["no_direct"]
        # algorithmic work of the direct term per H psi: T build and B sums
        # (8 nv nk flops each per (x, y)), two k-mesh FFTs (5 nk log2 nk each),
        # the ladder product (2 nk); ladder bytes nx^2 nk in the term's precision
        flops = nx * nx * (16.0 * nv * nk + 10.0 * nk * math.log2(nk) + 2.0 * nk)
        lad_bytes = nx * nx * nk * (4 if name == "mixed" else 8)
        out[name] = {"value": niter / dt, "unit": UNIT, "ms_per_hpsi": dt * 1e3 / niter,
                     "hpsi_ms_events": ms["all"], "direct_term_ms": direct_ms,
                     "direct_term_tflops": flops / (direct_ms * 1e-3) / 1e12,
                     "direct_term_ladder_gbs": lad_bytes / (direct_ms * 1e-3) / 1e9}
    out["spectral_error_mixed_vs_fp64"] = float(np.linalg.norm(spec["mixed"][:, 2] - spec["fp64"][:, 2]) /
                                                np.linalg.norm(spec["fp64"][:, 2]))
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    # CPU: the oracle's exchange + energies on the whole problem, and the direct
    # term on ny_s of the nx y-points (scaled by nx / ny_s), OpenMP over x on all
    # host cores
    a = w.device_arrays
    wh = dataclasses.replace(w, conr=a["conr"].cpu().numpy(), coni=a["coni"].cpu().numpy(),
                             valr=a["valr"].cpu().numpy(), vali=a["vali"].cpu().numpy(), ladder=None)
    ny_s = 16
    slab = a["ladder"].reshape(nx, nx * nk)[:ny_s].cpu().numpy().reshape(-1)
    P = O.OracleVal(wh, bande=1, bflag=1, lflag=0)
    t0 = time.perf_counter()
    P.act(w.psi_r, w.psi_i)
    t_x = time.perf_counter() - t0
    t0 = time.perf_counter()
    P.ladder_slab(w.psi_r, w.psi_i, 0, ny_s, slab)
    t_s = time.perf_counter() - t0
    t_hpsi = t_x + t_s * nx / ny_s
    out["cpu_oracle"] = {"value": 1.0 / t_hpsi, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": f"exchange + energies on the whole case ({t_x:.2f} s) and the direct term "
                                   f"on {ny_s} of {nx} y-points ({t_s:.2f} s), scaled to all y"}
    out["speedup_mixed_vs_cpu_oracle"] = out["mixed"]["value"] / out["cpu_oracle"]["value"]
    del a, w
    torch.cuda.empty_cache()
    return out


def run_nonherm(args, torch, capi, w, local):
    """Two-sided Lanczos (ocn_haydock_nonherm) on the main workload made
    non-Hermitian by a band lifetime Sigma'' ~ U(0.005, 0.05) Ha: H*psi/s (two
    actions per step, H and H^dagger) of both precisions and the spectral error."""
    import dataclasses
    import time

    rng = np.random.default_rng(77)
    wn = dataclasses.replace(w, ei=rng.uniform(0.005, 0.05, w.npsi))
    niter = args.nonherm_steps
    out = {"steps": niter, "sigma2_ha": [0.005, 0.05]}
    spec = {}
    for name, prec in (("mixed", capi.OCN_PREC_MIXED), ("fp64", capi.OCN_PREC_FP64)):
        # two vectors per context: the mixed path applies H and H^dagger as one block
        ctx = capi.Context(wn, precision=prec, device=local, nvec=2)
        ctx.haydock_nonherm(3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        co, done = ctx.haydock_nonherm(niter)
        dt = time.perf_counter() - t0
        ctx.close()
        spec[name] = capi.spectrum_cf_bc(*co, done, wn.kpref, wn.el, wn.eh, args.ne, wn.gam0)
        out[name] = {"value": 2 * niter / dt, "unit": UNIT, "ms_per_step": dt * 1e3 / niter}
    out["spectral_error_mixed_vs_fp64"] = float(np.linalg.norm(spec["mixed"][:, 2] - spec["fp64"][:, 2]) /
                                                np.linalg.norm(spec["fp64"][:, 2]))
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def run_multiplet(args, torch, capi, WL, local, dev):
    """c3: Haydock with the multiplet (tcgen05 projector contractions) and
    spin-orbit terms; H*psi/s of both precisions and the spectral error."""
    import time

    w = WL.make("c3", seed=0)
    niter = args.multiplet_steps
    out = {"workload": f"c3: {describe(w)}, multiplet l=0..3 x 8 projectors + spin-orbit", "steps": niter}
    spec = {}
    for name, prec in (("mixed", capi.OCN_PREC_MIXED), ("fp64", capi.OCN_PREC_FP64)):
        ctx = capi.Context(w, precision=prec, device=local)
        ctx.haydock(9)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ra, ia, rb, done = ctx.haydock(niter)
        dt = time.perf_counter() - t0
        ctx.timing(True)
        ctx.timing_reset()
        ctx.haydock(30)
        kt = ctx.timing_read()
        ctx.close()
        spec[name] = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, args.ne, w.gam0)
        out[name] = {"value": niter / dt, "unit": UNIT, "ms_per_hpsi": dt * 1e3 / niter, "kernel_ms_30_steps": kt}
    out["spectral_error_mixed_vs_fp64"] = float(np.linalg.norm(spec["mixed"][:, 2] - spec["fp64"][:, 2]) /
                                                np.linalg.norm(spec["fp64"][:, 2]))
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def run_batch(args, torch, capi, WL, local, dev, niter: int = 500, nv: int = 3):
    """Batched uneven instances: autotuned tiles per instance, one batched run
    (ocn_haydock_batch) against the same instances run one after another."""
    import time

    ctxs, bufs, shapes, tuned = [], [], [], []
    t0 = time.perf_counter()
    for i in range(args.batch):
        w = WL.batch_instance(i, u2_device=dev)
        ctx = capi.Context(w, precision=capi.OCN_PREC_MIXED, device=local, nvec=nv)
        w.ur = w.ui = None  # the context holds its own copy
        rng = np.random.default_rng(500 + i)
        d = torch.empty(2 * w.npsi * nv, dtype=torch.float64, device=dev)
        for v in range(nv):
            r = w.psi_r if v == 0 else rng.standard_normal(w.npsi)
            im = w.psi_i if v == 0 else rng.standard_normal(w.npsi)
            s = np.sqrt(np.sum(r * r + im * im))
            d[2 * v * w.npsi:(2 * v + 1) * w.npsi].copy_(torch.from_numpy(r / s))
            d[(2 * v + 1) * w.npsi:(2 * v + 2) * w.npsi].copy_(torch.from_numpy(im / s))
        default_tiles = ctx.tiles()
        ms_best, best = ctx.autotune(nv=nv, reps=3)
        tuned.append({"tiles": list(best), "default": list(default_tiles), "lr_ms": ms_best,
                      "default_lr_ms": ctx.last_tune_current_ms})
        ctxs.append(ctx)
        bufs.append(d)
        shapes.append({"nb": w.nb, "kmesh": w.kmesh[0], "xmesh": w.xmesh[0], "na": w.na})
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    ptrs = [d.data_ptr() for d in bufs]
    nvs = [nv] * len(ctxs)
    capi.haydock_batch(ctxs, ptrs, nvs, 30)  # warm-up
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    capi.haydock_batch(ctxs, ptrs, nvs, niter)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for c, p in zip(ctxs, ptrs):
        c.haydock_block_dev(niter, nv, p)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    total = len(ctxs) * nv * niter
    cmp64 = None
    m = min(args.batch_fp64, len(ctxs))
    if m > 0:
        # The same first m instances through both precisions for fp64_steps
        # Lanczos steps: mixed as one batched launch, FP64 one context after
        # another (its kernels are FP64-pipe bound, batching would not change
        # that); spectra compared chain by chain.
        fp64_steps = 100
        mres = capi.haydock_batch(ctxs[:m], ptrs[:m], nvs[:m], fp64_steps)  # warm-up of this subset
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        mres = capi.haydock_batch(ctxs[:m], ptrs[:m], nvs[:m], fp64_steps)
        torch.cuda.synchronize()
        t5 = time.perf_counter()
        err, t64 = 0.0, 0.0
        for i in range(m):
            w = WL.batch_instance(i, u2_device=dev)
            c64 = capi.Context(w, precision=capi.OCN_PREC_FP64, device=local, nvec=nv)
            w.ur = w.ui = None
            c64.haydock_block_dev(3, nv, ptrs[i])  # warm-up
            torch.cuda.synchronize()
            t6 = time.perf_counter()
            ra, ia, rb, _ = c64.haydock_block_dev(fp64_steps, nv, ptrs[i])
            torch.cuda.synchronize()
            t64 += time.perf_counter() - t6
            c64.close()
            for v in range(nv):
                s64 = capi.spectrum_cf(ra[v], ia[v], rb[v], fp64_steps, w.kpref, w.el, w.eh, 1000, w.gam0)
                smx = capi.spectrum_cf(mres[i][0][v], mres[i][1][v], mres[i][2][v], fp64_steps, w.kpref,
                                       w.el, w.eh, 1000, w.gam0)
                err = max(err, float(np.linalg.norm(smx[:, 2] - s64[:, 2]) / np.linalg.norm(s64[:, 2])))
        sub = m * nv * fp64_steps
        cmp64 = {"instances": m, "lanczos_steps": fp64_steps, "mixed_batched_value": sub / (t5 - t4),
                 "fp64_value": sub / t64, "speedup_mixed_vs_fp64": (t64 / (t5 - t4)),
                 "max_spectral_error_mixed_vs_fp64": err}
    for c in ctxs:
        c.close()
    torch.cuda.empty_cache()
    return {"instances": len(ctxs), "chains_each": nv, "lanczos_steps": niter,
            "value": total / (t2 - t1), "unit": UNIT, "ms": (t2 - t1) * 1e3,
            "sequential_value": total / (t3 - t2), "sequential_ms": (t3 - t2) * 1e3,
            "fp64_subset": cmp64, "setup_s": setup_s, "shapes": shapes, "tiles": tuned}


def oracle_check(args, ctx, w, torch, capi):
    """The FP64 oracle's Haydock run of the main workload on the host cores and
    the mixed GPU path's spectrum (same steps) against it."""
    import time

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    nst = args.oracle_steps
    ra, ia, rb, done = ctx.haydock(nst)
    sg = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, args.ne, w.gam0)
    t0 = time.perf_counter()
    P = O.OracleProblem(w)
    rc, ora, oia, orb, odone = P.haydock(nst)
    t1 = time.perf_counter()
    so = O.write_core(ora, oia, orb, nst, w.kpref, w.el, w.eh, args.ne, w.gam0)
    err = float(np.linalg.norm(sg[:, 2] - so[:, 2]) / np.linalg.norm(so[:, 2]))
    return {"steps": nst, "oracle_rc": int(rc), "oracle_s": t1 - t0, "cores": os.cpu_count(),
            "spectral_error_mixed_vs_oracle": err,
            "first10_a_rel_mixed": float(np.max(np.abs(ra[:10] - ora[:10]) / np.abs(ora[:10]))),
            "_spectrum": so}


def run_gmres(args, torch, capi, w, prec, local):
    """GMRES over the energy window: the lanes run and the single sweep."""
    from ocean_gb300 import workloads as WL2

    energies = np.linspace(w.el, w.eh, args.gmres_omega) * WL2.HARTREE2EV
    lanes = max(1, args.gmres_lanes)
    dev = f"cuda:{local}"
    gctx = capi.Context(w, precision=prec, device=local, nvec=lanes if prec == capi.OCN_PREC_MIXED else 1)
    stream = torch.cuda.ExternalStream(gctx.stream, device=dev)
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    out = {"omega_points": int(args.gmres_omega), "tolerance_g2": 1e-6, "depth": 80}

    def timed(nl, es):
        gctx.set_gmres_lanes(nl)
        gctx.gmres(es[:2], depth=80, tol=1e-6, max_restarts=100)  # warm-up
        l1 = gctx.launches
        torch.cuda.synchronize()
        g0.record(stream)
        ore, oim, rel, its = gctx.gmres(es, depth=80, tol=1e-6, max_restarts=100)
        g1.record(stream)
        torch.cuda.synchronize()
        return g0.elapsed_time(g1), ore, oim, rel, its, gctx.launches - l1

    try:
        main_im = None
        for tag, nl in (("lanes", lanes), ("single_sweep", 1)):
            gms, ore, oim, rel, its, nlaunch = timed(nl, energies)
            out[tag] = {"lanes": nl, "ms": gms, "spectra_per_s": 1000.0 / gms, "inner_iterations": int(its.sum()),
                        "gpu_launches": nlaunch,
                        "hpsi_per_s": (int(its.sum()) + 2 * args.gmres_omega) / (gms / 1000.0),
                        "max_rel_error": float(np.max(np.abs(rel)))}
            if main_im is None:
                main_im = oim
            else:
                out[tag]["max_rel_diff_vs_lanes_im"] = float(np.max(np.abs(oim - main_im) / np.abs(main_im)))
        out["ms"] = out["lanes"]["ms"]
        out["spectra_per_s"] = out["lanes"]["spectra_per_s"]
        if args.gmres_fp64_omega > 0 and prec == capi.OCN_PREC_MIXED:
            # every k-th energy (recycling still applies at this spacing), solved here
            # and again by the FP64 path with the same lanes
            step = max(1, len(energies) // args.gmres_fp64_omega)
            idx = np.arange(0, len(energies), step)[:args.gmres_fp64_omega]
            sub_e = energies[idx]
            nl = min(lanes, len(sub_e))
            gms, sre, sim, _, sits, _ = timed(nl, sub_e)
            out["fp64_subset"] = {"energies_ev": sub_e, "which": f"every {step}th of the {len(energies)}",
                                  "lanes": nl, "mixed_ms": gms, "mixed_re": sre, "mixed_im": sim,
                                  "mixed_iterations": int(sits.sum())}
    finally:
        gctx.close()
    return out


def run_ours(args, ws, rank, local, pg):
    import torch

    from ocean_gb300 import build as B
    from ocean_gb300 import capi
    from ocean_gb300 import workloads as WL

    B.build()
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    prec = capi.OCN_PREC_FP64 if args.precision == "fp64" else capi.OCN_PREC_MIXED
    w = WL.make(args.workload, seed=rank)
    ctx = capi.Context(w, precision=prec, device=local)
    niter, ne = args.niter, args.ne
    n = w.npsi
    d_psi = torch.empty(2 * n, dtype=torch.float64, device=dev)
    d_psi[:n].copy_(torch.from_numpy(w.psi_r))
    d_psi[n:].copy_(torch.from_numpy(w.psi_i))
    torch.cuda.synchronize()
    pr_ptr = d_psi.data_ptr()
    pi_ptr = pr_ptr + 8 * n
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    tiles = None
    if prec == capi.OCN_PREC_MIXED and args.autotune:
        # the library's tile autotuner (CUDA events on the context stream), before any timing
        tune_ms, best = ctx.autotune(nv=1, reps=3)
        tiles = {"tiles": list(best), "lr_ms": tune_ms, "default_lr_ms": ctx.last_tune_current_ms}

    _device_steps(ctx, w, niter, ne, pr_ptr, pi_ptr, args.warmup, stream, torch)
    # ---- timed region (inputs resident in HBM, no instrumentation)
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    l0 = ctx.launches
    dev_ms, spec_main = _device_steps(ctx, w, niter, ne, pr_ptr, pi_ptr, args.steps, stream, torch)
    if pg is not None:
        pg.barrier()
    clocks = sampler.stop()
    launches = ctx.launches - l0
    # ---- one instrumented step: CUDA events around every timed kernel on the
    #      library's stream (event-record nodes inside the captured graph)
    ctx.timing(True)
    ctx.timing_reset()
    _device_steps(ctx, w, niter, ne, pr_ptr, pi_ptr, 1, stream, torch)
    kt = ctx.timing_read()
    ctx.timing(False)
    value, dev_ms = replica_rate(pg, ws, dev_ms, niter * args.steps, dev)

    # ---- e2e: pinned host psi0 -> ocn_haydock -> coefficients + spectrum back
    h_psi = torch.empty(2 * n, dtype=torch.float64).pin_memory()
    h_psi[:n].copy_(torch.from_numpy(w.psi_r))
    h_psi[n:].copy_(torch.from_numpy(w.psi_i))
    hr = h_psi[:n].numpy()
    hi = h_psi[n:].numpy()
    ctx.haydock(niter, hr, hi)
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ra, ia, rb, done = ctx.haydock(niter, hr, hi)
        capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, ne, w.gam0)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    e2e_value, e2e_ms = replica_rate(pg, ws, e2e_ms, niter * args.steps, dev)

    # ---- oracle check: the FP64 oracle's own Haydock run on the same input, and
    #      the spectral error of the mixed path against it (column Spect(0))
    orc = None
    if rank == 0 and args.oracle_steps > 0:
        orc = oracle_check(args, ctx, w, torch, capi)
    ctx.close()

    # ---- GMRES leg: 200 energies across the spectrum, tol 1e-6 on |g|^2, depth 80,
    #      in energy lanes (one block action per round) and as the single sweep
    gm = None
    if rank == 0 and args.gmres_omega > 0:
        gm = run_gmres(args, torch, capi, w, prec, local)

    # ---- adjoint leg: d(spectrum)/d(W scale, W(r) table, Gamma, scissor) through
    #      GmresSpectrum, 400 energies at Gamma = 0.3 eV on the same sizes
    adj = None
    if rank == 0 and args.adjoint_omega > 0:
        import time

        from ocean_gb300 import adjoint

        gam = 0.3 * WL.EV2HARTREE
        energies = np.linspace(w.el, w.eh, args.adjoint_omega) * WL.HARTREE2EV
        prob = adjoint.GmresProblem(w, energies, precision=prec, device=local, depth=80, tol=1e-6,
                                    max_restarts=100)
        pt = [torch.tensor(w.interaction_scale, dtype=torch.float64, requires_grad=True),
              torch.tensor(w.ptab, dtype=torch.float64, requires_grad=True),
              torch.tensor(gam, dtype=torch.float64, requires_grad=True),
              torch.tensor(0.0, dtype=torch.float64, requires_grad=True)]
        l2 = prob.ctx.launches
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ore, oim = adjoint.gmres_spectrum(prob, *pt)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        oim.sum().backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        adj = {"omega_points": int(args.adjoint_omega), "gamma_ev": 0.3, "tolerance_g2": 1e-6, "depth": 80,
               "forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
               "backward_over_forward": (t2 - t1) / (t1 - t0),
               "gpu_launches": prob.ctx.launches - l2,
               "loss": "sum over energies of out_im (the eps2-like column)",
               "grad": {"scale": float(pt[0].grad), "ptab_norm": float(pt[1].grad.norm()),
                        "gamma": float(pt[2].grad), "scissor": float(pt[3].grad)}}
        prob.close()

    # ---- small-case leg (the CPU-runnable configuration): GPU precisions and the
    #      oracle's whole Haydock run on all host cores
    small = None
    if rank == 0 and args.c1_steps > 0:
        small = run_small(args, torch, capi, WL, local)

    # ---- multiplet leg: 2p edge with multiplet and spin-orbit terms (6^3 k, 64 bands,
    #      10^3 x-mesh, 128 projectors), mixed precision against the FP64 path
    mlt = None
    if rank == 0 and args.multiplet_steps > 0 and prec == capi.OCN_PREC_MIXED:
        mlt = run_multiplet(args, torch, capi, WL, local, dev)

    # ---- non-Hermitian leg: two-sided Lanczos on the main workload with a band lifetime
    nh = None
    if rank == 0 and args.nonherm_steps > 0 and prec == capi.OCN_PREC_MIXED:
        nh = run_nonherm(args, torch, capi, w, local)

    # ---- valence leg: exchange + screened direct terms on the v2 case, both precisions
    val = None
    if rank == 0 and args.valence_steps > 0 and prec == capi.OCN_PREC_MIXED:
        val = run_valence(args, torch, capi, WL, local)

    # ---- batched leg: independent uneven instances (k-mesh n^3, n in {4,5,6,8};
    #      bands U{24..128}; 1s or 2p; x-mesh 8^3..12^3), 3 polarisations each,
    #      500 Lanczos steps, all advanced by one graph launch per 3 steps
    bat = None
    if rank == 0 and args.batch > 0 and prec == capi.OCN_PREC_MIXED:
        bat = run_batch(args, torch, capi, WL, local, dev)

    # ---- block leg: nb chains (polarisations of one site) in lockstep, psi0 in HBM
    blk = None
    if rank == 0 and args.block > 1 and prec == capi.OCN_PREC_MIXED:
        nvb = args.block
        cb = capi.Context(w, precision=prec, device=local, nvec=nvb)
        rng = np.random.default_rng(1000 + rank)
        d_blk = torch.empty(2 * n * nvb, dtype=torch.float64, device=dev)
        for v in range(nvb):
            r = w.psi_r if v == 0 else rng.standard_normal(n)
            i = w.psi_i if v == 0 else rng.standard_normal(n)
            nrm = np.sqrt(np.sum(r * r + i * i))
            d_blk[2 * v * n:(2 * v + 1) * n].copy_(torch.from_numpy(r / nrm))
            d_blk[(2 * v + 1) * n:(2 * v + 2) * n].copy_(torch.from_numpy(i / nrm))
        torch.cuda.synchronize()
        sb = torch.cuda.ExternalStream(cb.stream, device=dev)
        if args.autotune:
            cb.autotune(nv=nvb, reps=3)
        cb.haydock_block_dev(niter, nvb, d_blk.data_ptr())  # warm-up (graph capture)
        b0 = torch.cuda.Event(enable_timing=True)
        b1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        b0.record(sb)
        for _ in range(args.steps):
            ra, ia, rb, done = cb.haydock_block_dev(niter, nvb, d_blk.data_ptr())
            for v in range(nvb):
                capi.spectrum_cf(ra[v], ia[v], rb[v], int(done[v]), w.kpref, w.el, w.eh, ne, w.gam0)
        b1.record(sb)
        torch.cuda.synchronize()
        bms = b0.elapsed_time(b1)
        cb.close()
        blk = {"chains": nvb, "value": nvb * niter * args.steps / (bms / 1000.0), "unit": UNIT,
               "ms_per_step": bms / args.steps,
               "spectra_per_s": nvb * args.steps / (bms / 1000.0)}

    if rank != 0:
        return
    # ---- the project's own FP64 GPU path on the same input: speed and the
    #      spectral error of the mixed path against it (column Spect(0))
    fp64 = None
    if prec == capi.OCN_PREC_MIXED and not args.no_fp64_compare:
        c64 = capi.Context(w, precision=capi.OCN_PREC_FP64, device=local)
        s64 = torch.cuda.ExternalStream(c64.stream, device=dev)
        c64.haydock_dev(50, pr_ptr, pi_ptr)
        ms64, spec64 = _device_steps(c64, w, niter, ne, pr_ptr, pi_ptr, 1, s64, torch)
        err = float(np.linalg.norm(spec_main[:, 2] - spec64[:, 2]) / np.linalg.norm(spec64[:, 2]))
        fp64 = {"value": niter / (ms64 / 1000.0), "unit": UNIT, "ms_per_step": ms64,
                "spectral_error_mixed_vs_fp64": err,
                "speedup_mixed_vs_fp64": value / ws / (niter / (ms64 / 1000.0))}
        if gm is not None and "fp64_subset" in gm:
            sub = gm.pop("fp64_subset")
            c64.set_gmres_lanes(sub["lanes"])
            h0 = torch.cuda.Event(enable_timing=True)
            h1 = torch.cuda.Event(enable_timing=True)
            h0.record(s64)
            re64, im64, _, its64 = c64.gmres(sub["energies_ev"], depth=80, tol=1e-6, max_restarts=100)
            h1.record(s64)
            torch.cuda.synchronize()
            ms_g64 = h0.elapsed_time(h1)
            # out_im is the absorption (1 - kpref Re F is out_re): both columns compared,
            # as a 2-norm over the energies and energy by energy
            e_im = float(np.linalg.norm(sub["mixed_im"] - im64) / np.linalg.norm(im64))
            e_re = float(np.linalg.norm(sub["mixed_re"] - re64) / np.linalg.norm(re64))
            m_im = float(np.max(np.abs(sub["mixed_im"] - im64) / np.abs(im64)))
            m_re = float(np.max(np.abs(sub["mixed_re"] - re64) / np.abs(re64)))
            gm["fp64_subset"] = {"omega_points": len(sub["energies_ev"]), "lanes": sub["lanes"],
                                 "energies": sub["which"], "mixed_ms": sub["mixed_ms"],
                                 "fp64_ms": ms_g64, "speedup_mixed_vs_fp64": ms_g64 / sub["mixed_ms"],
                                 "mixed_iterations": sub["mixed_iterations"], "fp64_iterations": int(its64.sum()),
                                 "spectral_error_im": e_im, "spectral_error_re": e_re,
                                 "max_rel_error_im_per_energy": m_im, "max_rel_error_re_per_energy": m_re}
        if orc is not None:
            ra, ia, rb, done = c64.haydock_dev(orc["steps"], pr_ptr, pi_ptr)
            s64o = capi.spectrum_cf(ra, ia, rb, done, w.kpref, w.el, w.eh, ne, w.gam0)
            so = orc["_spectrum"]
            orc["spectral_error_fp64_vs_oracle"] = float(np.linalg.norm(s64o[:, 2] - so[:, 2]) /
                                                         np.linalg.norm(so[:, 2]))
        c64.close()
    if orc is not None:
        orc.pop("_spectrum", None)
    if gm is not None and "mixed_re" in gm.get("fp64_subset", {}):
        gm.pop("fp64_subset")  # no FP64 run to compare with
    # dominant kernel and its roofline
    hbm, bf16, src = measured_peaks()
    lr_classes = {k: v for k, v in kt.items() if v[0] > 0 and k.startswith("lr_") and k != "lr_prep"}
    dom = max(lr_classes, key=lambda k: lr_classes[k][1]) if lr_classes else None
    roof = None
    if dom:
        cnt, ms = lr_classes[dom]
        per_launch_s = ms / cnt / 1000.0
        bytes_pl = algorithmic_bytes(w, dom, args.precision)
        achieved = bytes_pl / per_launch_s / 1e9
        tr = traffic_summary().get(f"k_lr_tc:{dom}:{args.workload}") if args.precision == "mixed" else None
        total_ms = sum(x[1] for x in kt.values())
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": f"{src} hbm_gbs (copy bandwidth)",
                "traffic": tr, "algorithmic_bytes_per_launch": bytes_pl,
                "avg_launch_ms": ms / cnt,
                "kernel_share": {k: round(v[1] / max(1e-9, total_ms), 4) for k, v in kt.items() if v[0] > 0}}
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(w)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "bf16x2-split+f32 (contractions), f32x2 double-float (Lanczos vectors), f64 (coefficients)",
            "data": "synthetic (seeded; u2 QR-orthonormal complex Gaussian, U(0,30) eV bands, "
                    "erf(r/0.5A)/(4r) W table)",
            "config": {"workload": f"{args.workload}: {describe(w)}, "
                                   f"{niter} Lanczos iterations + {ne + 1}-point spectrum per step",
                       "precision": args.precision, "parallelism": f"replicas x{ws}",
                       "l2": "inputs larger than L2 (u2 %.2f GB per contraction operand)" % (
                           w.nb * w.nk * w.nx * (16 if args.precision == 'fp64' else 8) / 1e9)},
            "spectra_per_s": args.steps * ws / (dev_ms / 1000.0),
            "fp64_gpu": fp64, "oracle_check": orc, "gmres": gm, "block_haydock": blk, "adjoint": adj, "batch": bat,
            "multiplet": mlt, "nonherm": nh, "valence": val, "c1": small, "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * n * 8,
                    "d2h_bytes_per_step": 3 * (niter + 1) * 8 + (ne + 1) * 9 * 8},
            "gpu_launches": launches, "clocks": clocks, "kernel_ms": kt, "tiles": tiles}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
    elif args.valence_only:
        import torch

        from ocean_gb300 import capi
        from ocean_gb300 import workloads as WL

        capi.load()
        if rank == 0:
            print(json.dumps({"valence": run_valence(args, torch, capi, WL, local)}), flush=True)
    else:
        run_ours(args, ws, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
