"""The OCEAN pipeline's input files for this path, read as ocean.x reads them
(CPU): u2.dat (OCEAN_bloch.f90:515-575), rpottrim (long_range.f90:1689-1698),
wvfcninfo (OCEAN_energies.f90:629-689), cksc / parcksc (OCEAN_multiplet.f90:
414-481) and cmel<l> (:489-500).  The reference ships none of these files, so
each test writes one in the format the reader code above expects (sequential
unformatted records framed by 4-byte lengths, as gfortran writes them; stream
files without frames; list-directed text) and checks every value read back."""
import struct

import numpy as np
import pytest

from ocean_gb300 import capi


@pytest.fixture(scope="module")
def lib(lib_built):
    return capi.load(lib_built)


def _rec(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _write_u2dat(path, vals, nx, ny, nz, nkpts, nspn, nband_file, first, nbd):
    """vals(s, iq, band, ix, iy, iz) -> (ur, ui); bands outside the window get
    records of other lengths, which a reader must skip by their frames."""
    out = bytearray()
    for s in range(nspn):
        for iq in range(nkpts):
            f0 = first[iq + nkpts * s]
            for b in range(nband_file):
                for ix in range(nx):
                    for iy in range(ny):
                        for iz in range(nz):
                            if f0 <= b < f0 + nbd:
                                ur, ui = vals(s, iq, b, ix, iy, iz)
                                out += _rec(struct.pack("<3i2d", ix + 1, iy + 1, iz + 1, ur, ui))
                            else:
                                out += _rec(struct.pack("<3i", 7, 7, 7) + b"\0" * (8 * (b % 3)))
    with open(path, "wb") as f:
        f.write(bytes(out))


def test_u2dat_window_and_layout(lib, tmp_path):
    nx, ny, nz, nkpts, nspn, nband_file, nbd = 2, 3, 2, 3, 2, 5, 2
    first = [0, 1, 2, 1, 3, 0]  # per (k-point, spin), k fastest
    rng = np.random.default_rng(4)
    table = rng.standard_normal((nspn, nkpts, nband_file, nx, ny, nz, 2))
    p = str(tmp_path / "u2.dat")
    _write_u2dat(p, lambda s, q, b, x, y, z: table[s, q, b, x, y, z], nx, ny, nz, nkpts, nspn, nband_file, first, nbd)
    re, im = capi.read_u2dat(p, nx, ny, nz, nkpts, nspn, nband_file, first, nbd)
    for s in range(nspn):
        for q in range(nkpts):
            f0 = first[q + nkpts * s]
            for b in range(nbd):
                for ix in range(nx):
                    for iy in range(ny):
                        for iz in range(nz):
                            x = ix + nx * (iy + ny * iz)
                            assert re[s, x, q, b] == table[s, q, f0 + b, ix, iy, iz, 0]
                            assert im[s, x, q, b] == table[s, q, f0 + b, ix, iy, iz, 1]


def test_u2dat_one_window_and_malformed_files(lib, tmp_path):
    nx, ny, nz, nkpts, nband_file, nbd = 2, 2, 2, 2, 3, 2
    p = str(tmp_path / "u2.dat")
    _write_u2dat(p, lambda s, q, b, x, y, z: (q + 0.5 * b, x - y + 0.25 * z), nx, ny, nz, nkpts, 1, nband_file,
                 [1, 1], nbd)
    re, im = capi.read_u2dat(p, nx, ny, nz, nkpts, 1, nband_file, 1, nbd)
    assert re[0, 0, 1, 0] == 1.5 and re[0, 0, 0, 1] == 1.0 and im[0, 7, 0, 0] == 0.25
    data = open(p, "rb").read()
    with open(p, "wb") as f:
        f.write(data[:-40])  # truncated
    with pytest.raises(capi.OcnError):
        capi.read_u2dat(p, nx, ny, nz, nkpts, 1, nband_file, 1, nbd)
    bad = bytearray(data)
    # the first k-point's band 0 is 8 skipped 20-byte records; the trailing length
    # of the first data record (at 160 + 4 + 28) no longer matches its leading one
    bad[160 + 4 + 28] ^= 1
    with open(p, "wb") as f:
        f.write(bytes(bad))
    with pytest.raises(capi.OcnError):
        capi.read_u2dat(p, nx, ny, nz, nkpts, 1, nband_file, 1, nbd)
    with pytest.raises(capi.OcnError):  # window beyond the file's bands
        capi.read_u2dat(p, nx, ny, nz, nkpts, 1, nband_file, 2, nbd)


def test_rpottrim(lib, tmp_path):
    p = tmp_path / capi.input_filename("rpottrim", "Cu", 1, n=2, l=1)
    assert p.name == "rpottrim.zCu0001_n02l01"
    r = np.linspace(0.1, 6.3, 64)
    pv = np.exp(-r) / r
    p.write_text("rpottrim   64\n" + "".join(f"  {a:.16E}  {b:.16E}\n" for a, b in zip(pv, r)).replace("E", "D"))
    ptab, rtab = capi.read_rpottrim(str(p))
    assert np.array_equal(ptab, pv) and np.array_equal(rtab, r)


@pytest.mark.parametrize("nspn", [1, 2])
def test_energy_file(lib, tmp_path, nspn):
    nbd, nq = 7, 5
    e = np.random.default_rng(nspn).uniform(-1, 2, (nspn, nq, nbd))
    head = struct.pack("<3i", nbd, nq, nspn) if nspn == 2 else struct.pack("<2i", nbd, nq)
    p = tmp_path / capi.input_filename("energies", "", 0)
    assert p.name == "wvfcninfo"
    p.write_bytes(_rec(head) + _rec(e.astype("<f8").tobytes()))
    assert np.array_equal(capi.read_energies(str(p), nspn), e)


def test_cks_both_formats_and_the_mpc_order(lib, tmp_path):
    lmin, lmax, nproj = 0, 2, [2, 1, 3]
    nptot = sum((2 * l + 1) * nproj[l - lmin] for l in range(lmin, lmax + 1))
    nb, nk, nspn, nbd_file = 4, 3, 1, 6
    rng = np.random.default_rng(9)
    pc = rng.standard_normal((nspn, nk, nbd_file, nptot)) + 1j * rng.standard_normal((nspn, nk, nbd_file, nptot))
    par = tmp_path / capi.input_filename("parcks", "Cu", 3)
    assert par.name == "parcksc.Cu0003"
    par.write_bytes(struct.pack("<3i", 0, nbd_file * nk, 0) + pc.astype("<c16").tobytes())
    pr, pi = capi.read_cks(str(par), True, nptot, nb, nk, nspn)
    assert np.array_equal(pr, pc.real[:, :, :nb]) and np.array_equal(pi, pc.imag[:, :, :nb])
    leg = tmp_path / capi.input_filename("cks", "Cu", 3)
    assert leg.name == "cksc.Cu0003"
    sub = pc[:, :, :nb]
    leg.write_bytes(_rec(b"head") + _rec(b"more") + _rec(np.ascontiguousarray(sub.real).tobytes())
                    + _rec(np.ascontiguousarray(sub.imag).tobytes()))
    qr, qi = capi.read_cks(str(leg), False, nptot, nb, nk, nspn)
    assert np.array_equal(qr, pr) and np.array_equal(qi, pi)
    mr, mi = capi.cks_to_mpc(lmin, lmax, nproj, qr, qi)
    # OCEAN_multiplet.f90:466-481, restated
    for s in range(nspn):
        for k in range(nk):
            for b in range(nb):
                ip = 0
                for l in range(lmin, lmax + 1):
                    for m in range(-l, l + 1):
                        for nu in range(nproj[l - lmin]):
                            assert mr[s, l - lmin, m + lmax, nu, k, b] == qr[s, k, b, ip]
                            assert mi[s, l - lmin, m + lmax, nu, k, b] == qi[s, k, b, ip]
                            ip += 1
    assert np.count_nonzero(mr) == nspn * nk * nb * nptot


def test_cmel_and_names(lib, tmp_path):
    p = tmp_path / capi.input_filename("cmel", "", 0, l=2)
    assert p.name == "cmel2"
    vals = np.arange(1, 10) * 0.125
    p.write_text("  1.25d-1 2.5d-1,3.75d-1\n 0.5 0.625 0.75\n  0.875\n 1.0D0 1.125\n")
    m = capi.read_cmel(str(p), 3)
    assert np.array_equal(m.ravel(), vals)  # m[nu] is column nu of mpm(:, :, l)
    assert capi.input_filename("cks", "Ti", 12, calc_type="XES") == "cksv.Ti0012"
    assert capi.input_filename("energies", "", 0, calc_type="VAL") == "wvfvainfo"
    with pytest.raises(capi.OcnError):
        capi.input_filename("cmel", "", 0, l=10)


def test_u2dat_feeds_the_library_layout(lib, tmp_path):
    """A workload's Bloch functions written as u2.dat (one occupied band before
    the window, two above it) come back as exactly the arrays ocn_set_bloch
    takes: u[s][x][k][n] with x = ix + nx*(iy + ny*iz)."""
    from ocean_gb300 import workloads as WL

    w = WL.make("tiny", seed=3)
    nx, ny, nz = w.xmesh
    nb, nk = w.nb, w.nk
    ur = w.ur.reshape(w.nspn, nx * ny * nz, nk, nb)
    ui = w.ui.reshape(w.nspn, nx * ny * nz, nk, nb)

    def vals(s, q, b, ix, iy, iz):
        x = ix + nx * (iy + ny * iz)
        return ur[s, x, q, b - 1], ui[s, x, q, b - 1]

    p = str(tmp_path / "u2.dat")
    _write_u2dat(p, vals, nx, ny, nz, nk, w.nspn, nb + 3, [1] * (nk * w.nspn), nb)
    re, im = capi.read_u2dat(p, nx, ny, nz, nk, w.nspn, nb + 3, 1, nb)
    assert np.array_equal(re.ravel(), w.ur) and np.array_equal(im.ravel(), w.ui)


# ---- valence run files

def test_val_u2_stream_file_layout_and_band_window(lib_built, tmp_path):
    """val.u2.dat / con.u2.dat (load_single_prefixu2dat): x1 fastest in the file,
    x3 fastest in the arrays; bands outside the window skipped; spins outer."""
    capi.load(lib_built)
    rng = np.random.default_rng(3)
    xm, nk, nspn, fb0, fb1 = (2, 3, 4), 5, 2, 1, 6
    nx = int(np.prod(xm))
    data = rng.standard_normal((nspn, nk, fb1 - fb0 + 1, nx)) + 1j * rng.standard_normal((nspn, nk, fb1 - fb0 + 1, nx))
    path = str(tmp_path / "con.u2.dat")
    data.astype(np.complex128).tofile(path)  # stream access: no record markers
    lo, nb = 3, 3
    re, im = capi.read_val_u2(path, xm, nk, nspn, fb0, fb1, lo, nb)
    got = (re + 1j * im).reshape(nspn, nk, nb, nx)
    for s in range(nspn):
        for k in range(nk):
            for b in range(nb):
                f = data[s, k, b + lo - fb0].reshape(xm[2], xm[1], xm[0])  # (iz, iy, ix), x1 fastest
                want = np.transpose(f, (2, 1, 0)).reshape(-1)             # x3 fastest
                assert np.array_equal(got[s, k, b], want)
    with open(str(tmp_path / "short"), "wb") as fh:
        fh.write(data.astype(np.complex128).tobytes()[:-16])
    with pytest.raises(capi.OcnError):
        capi.read_val_u2(str(tmp_path / "short"), xm, nk, nspn, fb0, fb1, lo, nb)


def test_val_pair_energies_blocks(lib_built):
    capi.load(lib_built)
    rng = np.random.default_rng(4)
    nk, nspn = 4, 2
    ec = rng.uniform(0, 1, (nspn, nk, 10))   # (spin, k, band): Fortran e(band, k, spin)
    ev = rng.uniform(-1, 0, (nspn, nk, 7))
    nc, nv, clo, vlo = 3, 2, 5, 4
    out = capi.val_pair_energies(nc, nv, nk, nspn, 2, ec.reshape(-1), 10, clo, ev.reshape(-1), 7, vlo)
    out = out.reshape(4, nk, nv, nc)
    for i in range(2):
        for j in range(2):
            want = ec[j][:, None, clo - 1:clo - 1 + nc] - ev[i][:, vlo - 1:vlo - 1 + nv, None]
            assert np.array_equal(out[i * 2 + j], want)


def test_read_haydockconv(tmp_path, lib_built):
    """haydockconv.ipt holds the early-exit threshold and spacing, read
    list-directed (OCEAN_system.f90:452-458)."""
    from ocean_gb300 import capi

    capi.load(lib_built)
    p = tmp_path / "haydockconv.ipt"
    p.write_text("  1.0d-3   5\n")
    assert capi.read_haydockconv(str(p)) == (1.0e-3, 5)
    p.write_text("0.02, 10 ! threshold, spacing\n")
    assert capi.read_haydockconv(str(p)) == (0.02, 10)
    p.write_text("0.02\n")
    with pytest.raises(capi.OcnError):
        capi.read_haydockconv(str(p))


def test_u2par_new_format_layout_and_window(lib, tmp_path):
    """u2par.dat (load_new_u2, OCEAN_bloch.f90:697-996): raw complex(DP), each
    (k-point, spin) block width(3) bands long, ivh2 bands skipped, iz fastest
    within a band; lands as re_bloch_state(band, k, x, spin), x = ix + nx(iy + ny iz)."""
    xm, nk, nspn, width3, nbd = (2, 3, 4), 3, 2, 6, 3
    nx, ny, nz = xm
    first = [0, 1, 2, 3, 1, 0]  # per (k-point, spin), k fastest
    rng = np.random.default_rng(8)
    data = rng.standard_normal((nspn, nk, width3, nx, ny, nz)) + 1j * rng.standard_normal((nspn, nk, width3, nx, ny, nz))
    p = str(tmp_path / "u2par.dat")
    data.astype(np.complex128).tofile(p)  # C order (..., ix, iy, iz): iz fastest, as u2_buf(iz, iy, ix, band)
    re, im = capi.read_u2par(p, xm, nk, nspn, width3, first, nbd)
    for s in range(nspn):
        for q in range(nk):
            f0 = first[q + nk * s]
            for b in range(nbd):
                for ix in range(nx):
                    for iy in range(ny):
                        for iz in range(nz):
                            x = ix + nx * (iy + ny * iz)
                            assert re[s, x, q, b] == data[s, q, f0 + b, ix, iy, iz].real
                            assert im[s, x, q, b] == data[s, q, f0 + b, ix, iy, iz].imag
    with pytest.raises(capi.OcnError):  # window beyond width(3)
        capi.read_u2par(p, xm, nk, nspn, width3, 4, nbd)
    with open(str(tmp_path / "short"), "wb") as fh:
        fh.write(data.astype(np.complex128).tobytes()[:-16])
    with pytest.raises(capi.OcnError):  # the last block's window reaches the (cut) end of the file
        capi.read_u2par(str(tmp_path / "short"), xm, nk, nspn, width3, width3 - nbd, nbd)


def test_run_directory_formats_feed_the_library_layout(lib, tmp_path):
    """A workload's Bloch functions written in each of the three formats the
    core run reads (u2.dat 'old', u2par.dat 'new' with bloch_type and
    obf_control, con.u2.dat 'par' which wins whenever it exists) come back
    through load_bloch_states as exactly the arrays ocn_set_bloch takes."""
    from ocean_gb300 import workloads as WL

    w = WL.make("tiny", seed=5)
    nx, ny, nz = w.xmesh
    nxyz, nb, nk = nx * ny * nz, w.nb, w.nk
    u = (w.ur + 1j * w.ui).reshape(w.nspn, nxyz, nk, nb)  # [s][x][k][n]
    xyz = [(ix, iy, iz) for ix in range(nx) for iy in range(ny) for iz in range(nz)]
    # 'old'
    d_old = tmp_path / "old"
    d_old.mkdir()

    def vals(s, q, b, ix, iy, iz):
        v = u[s, ix + nx * (iy + ny * iz), q, b - 1]
        return v.real, v.imag

    _write_u2dat(str(d_old / "u2.dat"), vals, nx, ny, nz, nk, w.nspn, nb + 2, [1] * (nk * w.nspn), nb)
    fmt, re, im = capi.load_bloch_states(str(d_old), w.xmesh, nk, w.nspn, nb, first=1, bands_in_file=nb + 2)
    assert fmt == "old" and np.array_equal(re.ravel(), w.ur) and np.array_equal(im.ravel(), w.ui)
    # 'new': two occupied bands skipped, width(3) = nb + 3
    d_new = tmp_path / "new"
    d_new.mkdir()
    (d_new / "bloch_type").write_text("new\n")
    (d_new / "obf_control").write_text(f"1\n1\n{nb + 3}\n")
    blk = np.zeros((w.nspn, nk, nb + 3, nx, ny, nz), dtype=np.complex128)
    for s in range(w.nspn):
        for q in range(nk):
            for (ix, iy, iz) in xyz:
                blk[s, q, 2:2 + nb, ix, iy, iz] = u[s, ix + nx * (iy + ny * iz), q, :]
    blk.tofile(str(d_new / "u2par.dat"))
    fmt, re, im = capi.load_bloch_states(str(d_new), w.xmesh, nk, w.nspn, nb, first=2)
    assert fmt == "new" and np.array_equal(re.ravel(), w.ur) and np.array_equal(im.ravel(), w.ui)
    # 'par': con.u2.dat present (bloch_type says 'new' and is overridden), two extra bands per k
    (d_new / "con.u2.dat").write_bytes(b"")
    par = np.zeros((w.nspn, nk, nb + 2, nxyz), dtype=np.complex128)
    par[:, :, :nb, :] = np.transpose(u, (0, 2, 3, 1))
    par.tofile(str(d_new / "con.u2.dat"))
    fmt, re, im = capi.load_bloch_states(str(d_new), w.xmesh, nk, w.nspn, nb, bands_in_file=nb + 2)
    assert fmt == "par" and np.array_equal(re.ravel(), w.ur) and np.array_equal(im.ravel(), w.ui)
    with pytest.raises(capi.OcnError):  # file shorter than bands_in_file promises
        capi.load_bloch_states(str(d_new), w.xmesh, nk, w.nspn, nb, bands_in_file=nb + 3)
