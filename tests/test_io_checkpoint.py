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
    c.step(3)
    sa, sc = a.get_state(), c.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sa[k], sc[k]), k
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
