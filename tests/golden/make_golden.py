"""Extract the continued-fraction known-answer vectors from the reference's own
example results (EXAMPLE/Cu_TwoPhoton/Results) into a small fixture.

For each of the 7 photon files:
  abslanc_Cu.0001_1s_0P : N, kpref, a_0..a_N, b_1..b_N and the N+1 tridiagonal
                          eigenvalues written by redtrid/write_lanczos
                          (OCEAN2/OCEAN_haydock.f90:2273-2358)
  absspct_Cu.0001_1s_0P : write_core output (OCEAN_haydock.f90:1801-1894); every
                          10th row (plus the last) of the 5001 is kept.
Text fixtures (verbatim bytes, for the byte-compatibility tests of the writers):
  cu_abslanc_01.txt       : abslanc_Cu.0001_1s_01 whole
  cu_absspct_01_rows.txt  : absspct_Cu.0001_1s_01, its two header records and
                            the same kept rows
Run from the repository root: python tests/golden/make_golden.py <reference_root>
(the root of an OCEAN v3.2.1 source tree).
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py <reference_root>")
REF = sys.argv[1]
RES = os.path.join(REF, "EXAMPLE", "Cu_TwoPhoton", "Results")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cu_twophoton_kat.npz")


def read_lanc(path):
    with open(path) as f:
        lines = f.read().split("\n")
    n_str, kpref_str = lines[0].split()
    n = int(n_str)
    ra = np.zeros(n + 1)
    rb = np.zeros(n + 1)
    ra[0] = float(lines[1].split()[0])
    for i in range(1, n + 1):
        a, b = lines[1 + i].split()
        ra[i] = float(a)
        rb[i] = float(b)
    eig = []
    for line in lines[n + 2:]:
        parts = line.split()
        if len(parts) == 3:
            eig.append(float(parts[2]))
    return n, float(kpref_str), ra, rb, np.array(eig)


def read_spct(path):
    rows = []
    header = None
    with open(path) as f:
        for line in f:
            if line.lstrip().startswith("#"):
                if "iter=" in line:
                    header = line
                continue
            rows.append([float(v) for v in line.split()])
    arr = np.array(rows)
    vol = float(header.split("vol=")[1])
    return arr, vol


def main():
    data = {}
    for p in range(1, 8):
        n, kpref, ra, rb, eig = read_lanc(os.path.join(RES, f"abslanc_Cu.0001_1s_0{p}"))
        spct, vol = read_spct(os.path.join(RES, f"absspct_Cu.0001_1s_0{p}"))
        keep = np.unique(np.concatenate([np.arange(0, len(spct), 10), [len(spct) - 1]]))
        data[f"p{p}_n"] = np.array(n)
        data[f"p{p}_kpref"] = np.array(kpref)
        data[f"p{p}_real_a"] = ra
        data[f"p{p}_real_b"] = rb
        data[f"p{p}_eig"] = eig
        data[f"p{p}_rows"] = keep
        data[f"p{p}_spct"] = spct[keep]
        data[f"p{p}_vol"] = np.array(vol)
        data[f"p{p}_nrows"] = np.array(len(spct))
    # run parameters from EXAMPLE/Cu_TwoPhoton/Cu.in: bse.core.broaden 1.245 eV,
    # cnbse.spect_range {5000 -30 70}; ebase = 0 (CNBSE/cnbse.pl:879)
    data["gam0_ev"] = np.array(1.245)
    data["ne"] = np.array(5000)
    data["el_ev"] = np.array(-30.0)
    data["eh_ev"] = np.array(70.0)
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
    here = os.path.dirname(OUT)
    with open(os.path.join(RES, "abslanc_Cu.0001_1s_01"), "rb") as f:
        lanc = f.read()
    with open(os.path.join(here, "cu_abslanc_01.txt"), "wb") as f:
        f.write(lanc)
    with open(os.path.join(RES, "absspct_Cu.0001_1s_01"), "rb") as f:
        lines = f.read().split(b"\n")
    body = [l for l in lines[2:] if l]
    keep = np.unique(np.concatenate([np.arange(0, len(body), 10), [len(body) - 1]]))
    with open(os.path.join(here, "cu_absspct_01_rows.txt"), "wb") as f:
        f.write(b"\n".join(lines[:2] + [body[i] for i in keep]) + b"\n")


if __name__ == "__main__":
    main()
