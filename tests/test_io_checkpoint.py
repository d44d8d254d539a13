"""The reference's file formats and checkpoint/restart.

.dat cases follow the reference's own io tests (test/io_test.f90): bounds
(1:9, 0:10, 1:11), values (i+1)(j+2)(k+3), round trip through save/load,
and the three bound-mismatch codes of load_data_into_array."""
import numpy as np
import pytest

from tpls_gb300.io import (OPTION_FILE_NOT_FOUND_ERR, OPTION_FORMAT_ERR, load_data, load_data_into_array,
                           load_options, params_from_options, save_data)

B = (1, 9, 0, 10, 1, 11)


def _sample():
    lx, ly, mx, my, nx, ny = B
    i = np.arange(lx, ly + 1)[:, None, None]
    j = np.arange(mx, my + 1)[None, :, None]
    k = np.arange(nx, ny + 1)[None, None, :]
    return np.asfortranarray(((i + 1) * (j + 2) * (k + 3)).astype(np.float64))


def test_dat_round_trip(tmp_path):
    f = tmp_path / "a.dat"
    d = _sample()
    save_data(f, "tpls_io test file", d, B)
    text = f.read_text().splitlines()
    assert text[0].strip() == "DATA: tpls_io test file"
    assert [int(t) for t in text[2].split()] == list(B)
    assert len(text) == 3 + d.size
    got, bounds, ierr = load_data(f)
    assert ierr == 0 and bounds == B and np.array_equal(got, d)
    got2, ierr2 = load_data_into_array(f, B)
    assert ierr2 == 0 and np.array_equal(got2, d)


def test_dat_bounds_mismatch_codes(tmp_path):
    f = tmp_path / "a.dat"
    save_data(f, "x", _sample(), B)
    assert load_data_into_array(f, (0, 9, 0, 10, 1, 11))[1] == 1
    assert load_data_into_array(f, (1, 9, 1, 10, 1, 11))[1] == 2
    assert load_data_into_array(f, (1, 9, 0, 10, 1, 12))[1] == 3


def test_dat_reads_fortran_d_exponents_and_short_files(tmp_path):
    f = tmp_path / "b.dat"
    f.write_text(" DATA: x\n DIMENSIONS: Lmin Lmax Mmin Mmax Nmin Nmax\n 1 2 1 1 1 1\n  0.5D+00\n  -1.25D+01\n")
    d, b, ierr = load_data(f)
    assert ierr == 0 and d.ravel().tolist() == [0.5, -12.5]
    g = tmp_path / "c.dat"
    g.write_text(" DATA: x\n DIMENSIONS: Lmin Lmax Mmin Mmax Nmin Nmax\n 1 3 1 1 1 1\n 1.0\n")
    assert load_data(g)[2] == 1


def test_options_and_params(tmp_path):
    f = tmp_path / "tpls_config.opt"
    f.write_text("# run options\nmaxl 257\nmaxm 129\nmaxn 193\n\nre 200.0\nmu_minus 2.0\nmu_plus 1.0\n"
                 "height 0.5\nscap 1.0\ndt 0.0001\nsmooth_width_scale 1.5\nmom_u 30\nmom_v 30\nmom_w 30\n"
                 "levelset 10\n")
    opts, ierr = load_options(f)
    assert ierr == 0 and opts["re"] == "200.0" and len(opts) == 14
    nx, ny, nz, p = params_from_options(opts)
    assert (nx, ny, nz) == (256, 128, 192)
    assert p.dx == p.dy == p.dz == 1.0 / 192 and p.smooth_width == 1.5 / 192 and p.dt == 1e-4
    assert load_options(tmp_path / "missing.opt")[1] == OPTION_FILE_NOT_FOUND_ERR
    bad = tmp_path / "bad.opt"
    bad.write_text("re 100\nlonelytoken\n")
    assert load_options(bad)[1] == OPTION_FORMAT_ERR


@pytest.mark.gpu
def test_checkpoint_restart_is_bit_identical(tmp_path):
    from tpls_gb300.api import STATE_FIELDS, TplsGpu
    from tpls_gb300.channel import make_case
    from tpls_gb300.checkpoint import load_checkpoint, save_checkpoint
    params, uin, st = make_case("A", nx=32, ny=16, nz=24)
    a = TplsGpu(32, 16, 24, params, uin)
    a.set_state(st)
    a.step(5)
    b = TplsGpu(32, 16, 24, params, uin)
    b.set_state(st)
    b.step(2)
    save_checkpoint(b, tmp_path / "ck.npz")
    b.close()
    c = load_checkpoint(tmp_path / "ck.npz")
    assert c.stats()["steps_done"] == 2  # the step count continues
    c.step(3)
    sa, sc = a.get_state(), c.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sa[k], sc[k]), k
    assert c.stats()["steps_done"] == 5
    a.close()
    c.close()


def test_checkpoint_file_holds_the_whole_state(tmp_path):
    """A checkpoint written from a channel mid-run holds everything a restart
    needs: restoring the file into a fresh channel and stepping on gives the
    uninterrupted run bit for bit (checked on the CPU oracle, which has the
    same field interface as the GPU context)."""
    import json

    from oracle.oracle import Oracle
    from tpls_gb300.api import Params
    from tpls_gb300.channel import make_case
    from tpls_gb300.checkpoint import save_checkpoint
    params, uin, st = make_case("A", nx=12, ny=6, nz=8)
    a = Oracle(12, 6, 8, params, uin)
    a.set_state(st)
    a.step(2)
    f = tmp_path / "ck.npz"
    save_checkpoint(a, f)
    z = np.load(f, allow_pickle=False)
    assert list(z["grid"]) == [12, 6, 8] and np.array_equal(z["u_inlet"], uin)
    meta = json.loads(str(z["params"]))
    assert Params(**meta) == params
    b = Oracle(12, 6, 8, Params(**meta), z["u_inlet"])
    b.set_state({k[2:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("f_")})
    a.step(2)
    b.step(2)
    for k, v in a.get_state().items():
        assert np.array_equal(v, b.get_field(k)), k


# ---- the reference's backup format (io.F90:647-791) -------------------------

_BK_NAMES = ["u2", "v2", "w2", "conv0_u", "conv1_u", "conv0_v", "conv1_v", "conv0_w", "conv1_w", "pres_old",
             "pres", "phi", "conv0_phi", "conv1_phi"]


def _bk_shapes(nx, ny, nz):
    uv, w, p = (nx + 2, ny + 2, nz), (nx + 2, ny + 2, nz + 1), (nx + 2, ny + 2, nz + 2)
    return {"u2": uv, "v2": uv, "w2": w, "conv0_u": uv, "conv1_u": uv, "conv0_v": uv, "conv1_v": uv,
            "conv0_w": w, "conv1_w": w, "pres_old": p, "pres": p, "phi": p, "conv0_phi": p, "conv1_phi": p}


def _bk_call(fn, arrays, nx, ny, nz, path):
    import ctypes as C
    dp = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrays]
    l, m, n = C.c_int(nx + 1), C.c_int(ny + 1), C.c_int(nz + 1)
    return fn(*dp, C.byref(l), C.byref(m), C.byref(n), str(path).encode())


def test_reference_backup_layout_and_round_trip(tmp_path):
    """tpls_write_backup writes backup_channel's records (i fastest; u, v, w
    blocks of three values, phi block of three, pres block of two) with 17
    significant digits, and tpls_read_backup restores them bit for bit."""
    from tpls_gb300.api import load_library
    lib = load_library()
    nx, ny, nz = 5, 3, 4
    rng = np.random.default_rng(3)
    sh = _bk_shapes(nx, ny, nz)
    arrs = {k: np.asfortranarray(rng.normal(size=sh[k]) * 10.0 ** rng.integers(-8, 8)) for k in _BK_NAMES}
    f = tmp_path / "fieldbackup0.dat"
    assert _bk_call(lib.tpls_write_backup, [arrs[k] for k in _BK_NAMES], nx, ny, nz, f) == 0
    lines = f.read_text().splitlines()
    nuv, nw, np_ = (nx + 2) * (ny + 2) * nz, (nx + 2) * (ny + 2) * (nz + 1), (nx + 2) * (ny + 2) * (nz + 2)
    assert len(lines) == 2 * nuv + nw + 2 * np_
    rows = [[float(t) for t in ln.split()] for ln in lines]
    # record c of the u block: u2, conv0_u, conv1_u at Fortran position c
    c = 17
    assert rows[c] == [arrs["u2"].ravel(order="F")[c], arrs["conv0_u"].ravel(order="F")[c],
                       arrs["conv1_u"].ravel(order="F")[c]]
    last = rows[-1]
    assert last == [arrs["pres"].ravel(order="F")[-1], arrs["pres_old"].ravel(order="F")[-1]]
    back = {k: np.zeros(sh[k], order="F") for k in _BK_NAMES}
    assert _bk_call(lib.tpls_read_backup, [back[k] for k in _BK_NAMES], nx, ny, nz, f) == 0
    for k in _BK_NAMES:
        assert np.array_equal(back[k], arrs[k]), k


def test_reference_backup_reads_fortran_list_directed_forms(tmp_path):
    """A file in the forms a Fortran list-directed write or a hand edit
    produces (D exponents, comma separators, r*value repeats) reads like the
    reference's dataload_channel would; a short or missing file is
    TPLS_ERR_IO (6)."""
    from tpls_gb300.api import load_library
    lib = load_library()
    nx, ny, nz = 2, 2, 3
    sh = _bk_shapes(nx, ny, nz)
    nuv, nw, np_ = 4 * 4 * nz, 4 * 4 * (nz + 1), 4 * 4 * (nz + 2)
    parts = ["   1.0000000000000000       0.50000000000000000      -2.5000000000000000D-002"]
    parts += ["%d*0.0" % (3 * nuv - 3)]
    parts += ["1.5E+00, 2, 3"] * nuv
    parts += ["  -7.0D0  8.0  9.0"] * nw
    parts += ["4.0 5.0 6.0"] * np_
    parts += ["1.0D+01 2.0d+01"] * np_
    f = tmp_path / "ref.dat"
    f.write_text("\n".join(parts) + "\n")
    back = {k: np.full(sh[k], np.nan, order="F") for k in _BK_NAMES}
    assert _bk_call(lib.tpls_read_backup, [back[k] for k in _BK_NAMES], nx, ny, nz, f) == 0
    u = back["u2"].ravel(order="F")
    assert u[0] == 1.0 and back["conv0_u"].ravel(order="F")[0] == 0.5
    assert back["conv1_u"].ravel(order="F")[0] == -0.025 and u[1] == 0.0
    assert np.all(back["v2"] == 1.5) and np.all(back["conv1_v"] == 3.0) and np.all(back["w2"] == -7.0)
    assert np.all(back["phi"] == 4.0) and np.all(back["pres"] == 10.0) and np.all(back["pres_old"] == 20.0)
    short = tmp_path / "short.dat"
    short.write_text("\n".join(parts[:-5]) + "\n")
    assert _bk_call(lib.tpls_read_backup, [back[k] for k in _BK_NAMES], nx, ny, nz, short) == 6
    assert _bk_call(lib.tpls_read_backup, [back[k] for k in _BK_NAMES], nx, ny, nz, tmp_path / "none.dat") == 6


@pytest.mark.gpu
def test_reference_backup_restart_is_bit_identical(tmp_path):
    """Backup after 2 steps (the reference's file plus the CSF companion),
    restart a fresh context from it, 3 more steps: bit-identical to 5
    uninterrupted steps, with the step count carried over."""
    from tpls_gb300.api import STATE_FIELDS, TplsGpu
    from tpls_gb300.channel import make_case
    from tpls_gb300.checkpoint import backup_channel, csf_companion, dataload_channel
    nx, ny, nz = 32, 16, 24
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    a = TplsGpu(nx, ny, nz, params, uin)
    a.set_state(st)
    a.step(5)
    b = TplsGpu(nx, ny, nz, params, uin)
    b.set_state(st)
    b.step(2)
    f = tmp_path / "fieldbackup0.dat"
    backup_channel(b, f)
    assert (tmp_path / "fieldbackup0_csf.dat").exists() and csf_companion(f).endswith("fieldbackup0_csf.dat")
    b.close()
    c = TplsGpu(nx, ny, nz, params, uin)
    dataload_channel(c, f, steps_done=2)
    c.step(3)
    sa, sc = a.get_state(), c.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sa[k], sc[k]), k
    assert c.stats()["steps_done"] == 5
    a.close()
    c.close()
