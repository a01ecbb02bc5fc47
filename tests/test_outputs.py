"""The ASCII output writers (diskflux, flux.f90:23-121, and output.F90:166-503)
through hc3d_write_outputs, fed the tallies of an oracle run: file set,
formats and normalisation.  CPU only."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d

LSUN = 3.839e33
NAMES = ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums", "ti", "tq", "tu", "tv", "ti2", "tq2", "tu2",
         "tv2", "numt", "image_i", "image_q", "image_u", "image_v")


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def test_writers_from_oracle_tallies(O, model_factory, tmp_path):
    m = model_factory("tiny")
    n = 3000
    p = m.run_params(np=n, iter=2, ipeel=1)
    r = O.run(m, p)
    T = hc3d.Tallies()
    keep = []
    for k in NAMES:
        a = np.asfortranarray(r[k])
        keep.append(a)
        setattr(T, k, a.ctypes.data_as(C.POINTER(C.c_int64)))
    T.stokes_scale, T.square_scale, T.path_scale = r["stokes_scale"], r["square_scale"], r["path_scale"]
    td = np.asfortranarray(m.tdust)
    out = tmp_path / "out"
    out.mkdir()
    rc = hc3d.lib().hc3d_write_outputs(m._h, C.byref(p), C.byref(T), td.ctypes.data_as(hc3d.dp),
                                       td.ctypes.data_as(hc3d.dp), str(out).encode())
    assert rc == 0
    nf, nmu, nph, nap, npeel, nx = p.nfreq, p.nmu, p.nph, p.nap, p.npeel, p.nxhst
    # the file set of output.F90
    assert len(list(out.glob("flux*.dat"))) == 8
    assert len(list(out.glob("peel_flux*.dat"))) == 8 * npeel
    assert len(list(out.glob("e_ALL_*_img.dat"))) == 4 * npeel
    assert len(list(out.glob("tmidplane*.dat"))) == 4 and len(list(out.glob("tave*.dat"))) == 4
    # flux.dat: list-directed dimensions, the column header, rows (F10.4, 8(2X, ES11.4))
    lines = (out / "flux.dat").read_text().splitlines()
    assert lines[0].split()[:4] == [str(nf), str(nph), str(nmu), str(nap)]
    assert lines[1].startswith("# Lambda         I          I_err         Q/I       (Q/I)_err")
    assert len(lines) == 2 + nf * nmu * nph * nap
    row = lines[2]
    assert len(row) == 10 + 8 * 13 and row[10:12] == "  "
    # normalisation (flux.f90): F = sum I / (np / nmu / nph / (L/Lsun)) / dnu-bin width
    rnorm = n / nmu / nph / (m.info.ltot / LSUN)
    nurat = p.numax / p.numin
    nunorm = nurat ** (0.5 / nf) - nurat ** (-0.5 / nf)
    si = r["si"][..., 0] / r["stokes_scale"]
    vals = np.array([[float(v) for v in l.split()] for l in lines[2:]])
    got = vals[:, 1].reshape(nmu, nf)  # rows: mu outer, frequency inner (nph = nap = 1)
    want = si[:, :, 0, 0].T / rnorm / nunorm
    np.testing.assert_allclose(got, want, rtol=6e-5, atol=0)
    wav = 1.2398 / (p.numin * nurat ** ((np.arange(1, nf + 1) - 0.5) / nf))
    np.testing.assert_allclose(vals[:nf, 0], wav, atol=6e-5)
    # images: nx rows of nx values, each ES11.4 and a blank
    img = (out / f"e_ALL_{m.thete[0] * 180 / np.pi:.1f}_{m.phie[0] * 180 / np.pi:.1f}_I_img.dat".replace(" ", ""))
    rows = img.read_text().splitlines()
    assert len(rows) == nx and all(len(x) == 12 * nx for x in rows)
    # tmidplane: the temperatures of the midplane row, in K
    tm = (out / "tmidplane1.dat").read_text().splitlines()
    it = (m.shape4[1] + 1) // 2
    tcol = np.array([float(l.split()[4]) for l in tm[2:]])
    np.testing.assert_allclose(tcol, td[:-1, it - 1, 0, 0] * 11605.0, rtol=0, atol=6e-6)


def test_writer_rejects_missing_arrays(model_factory, tmp_path):
    m = model_factory("tiny")
    p = m.run_params(np=10, ipeel=1)
    T = hc3d.Tallies()
    T.stokes_scale = T.square_scale = T.path_scale = 1.0
    td = np.asfortranarray(m.tdust)
    rc = hc3d.lib().hc3d_write_outputs(m._h, C.byref(p), C.byref(T), td.ctypes.data_as(hc3d.dp),
                                       td.ctypes.data_as(hc3d.dp), str(tmp_path).encode())
    assert rc == -1


def _read_unf(path):
    """Fortran unformatted sequential records (4-byte length markers)."""
    raw = path.read_bytes()
    recs, i = [], 0
    while i < len(raw):
        n = int(np.frombuffer(raw[i:i + 4], dtype="<i4")[0])
        recs.append(raw[i + 4:i + 4 + n])
        assert int(np.frombuffer(raw[i + 4 + n:i + 8 + n], dtype="<i4")[0]) == n
        i += 8 + n
    return recs


def test_grid_unf_files(model_factory, tmp_path):
    """output_grid (output.F90:38-150): header record, cell-centre radii in AU,
    polar and azimuthal centres, then the array over the cells."""
    m = model_factory("tiny3d")
    nrg, ntg, npg, ndg = m.shape4
    path = tmp_path / "darr.unf"
    d = np.asfortranarray(m.densarr)
    assert hc3d.lib().hc3d_write_grid_unf(m._h, str(path).encode(), ndg, d.ctypes.data_as(hc3d.dp), None) == 0
    recs = _read_unf(path)
    assert len(recs) == 5
    assert list(np.frombuffer(recs[0], dtype="<i4")) == [nrg - 1, ntg - 1, npg - 1, ndg]
    rave = np.sqrt(m.rarr[:-1] * m.rarr[1:])
    np.testing.assert_allclose(np.frombuffer(recs[1], dtype="<f8") * m.info.autors, rave, rtol=1e-12)
    assert len(np.frombuffer(recs[2], dtype="<f8")) == ntg - 1
    np.testing.assert_allclose(np.frombuffer(recs[3], dtype="<f8"), 0.5 * (m.phiarr[:-1] + m.phiarr[1:]), rtol=1e-15)
    body = np.frombuffer(recs[4], dtype="<f8").reshape((nrg - 1, ntg - 1, npg - 1, ndg), order="F")
    np.testing.assert_array_equal(body, m.densarr[:-1, :-1, :-1, :])
    # an integer grid (lastdim 1)
    k = np.asfortranarray(np.arange(nrg * ntg * npg, dtype=np.int32).reshape((nrg, ntg, npg), order="F"))
    path = tmp_path / "killed_001.unf"
    assert hc3d.lib().hc3d_write_grid_unf(m._h, str(path).encode(), 1, None,
                                          k.ctypes.data_as(hc3d.i32p)) == 0
    recs = _read_unf(path)
    got = np.frombuffer(recs[4], dtype="<i4").reshape((nrg - 1, ntg - 1, npg - 1), order="F")
    np.testing.assert_array_equal(got, k[:-1, :-1, :-1])
    # exactly one array
    assert hc3d.lib().hc3d_write_grid_unf(m._h, str(path).encode(), 1, None, None) == -1
