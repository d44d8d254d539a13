"""Option files, option accessors and the point-file formats of the
reference's driver, checked on the cases of the reference's own tests
(test/options_utils_test.f90 and test/io_test.f90: the same option names,
values, error codes, grid bounds l=9 m=5 n=5, cell sizes 0.1/0.2/0.3 and
values (i+1)(j+2)(k+3))."""
import io as _io

import numpy as np
import pytest

from tpls_gb300 import io as tio


def _opts(pairs):
    o = {}
    for k, v in pairs:
        tio.put_option(o, k, v)
    return o


def test_has_option():
    o = _opts([("option1", "value1"), ("option2", "value2"), ("option3", "value3")])
    assert tio.has_option(o, "option1") and tio.has_option(o, "option2") and tio.has_option(o, "option3")
    assert not tio.has_option(o, "option4")


def test_get_option_by_type():
    o = _opts([("string", "blah"), ("int", "2"), ("double", "3.45"), ("logical", "true")])
    assert tio.get_option(o, "string") == ("blah", 0)
    assert tio.get_string_option(o, "string") == ("blah", 0)
    assert tio.get_typed_option(o, "string", str) == ("blah", 0)
    assert tio.get_option(o, "int") == ("2", 0)
    assert tio.get_integer_option(o, "int") == (2, 0)
    assert tio.get_typed_option(o, "int", int) == (2, 0)
    v, e = tio.get_double_option(o, "double")
    assert e == 0 and abs(v - 3.45) < 0.01
    assert tio.get_typed_option(o, "double", float)[0] == v
    assert tio.get_logical_option(o, "logical") == (True, 0)
    assert tio.get_typed_option(o, "logical", bool) == (True, 0)


def test_get_no_such_option():
    o = _opts([("option", "value")])
    for get in (tio.get_option, tio.get_string_option, tio.get_integer_option, tio.get_double_option,
                tio.get_logical_option):
        assert get(o, "blah") == (None, tio.OPTION_NOT_FOUND_ERR)
    for kind in (str, int, float, bool):
        assert tio.get_typed_option(o, "blah", kind)[1] == tio.OPTION_NOT_FOUND_ERR
    assert tio.OPTION_NOT_FOUND_ERR == 100


def _add_test_options(o):
    tio.put_string_option(o, "string", "blah")
    tio.put_integer_option(o, "int", 2)
    tio.put_double_option(o, "double", 3.45)
    tio.put_logical_option(o, "logical", True)
    tio.put_option(o, "option", "value")


def _add_typed_test_options(o):
    tio.put_typed_option(o, "string_type", "blah_type")
    tio.put_typed_option(o, "int_type", 6)
    tio.put_typed_option(o, "double_type", 7.89)
    tio.put_typed_option(o, "logical_type", False)


def _check_test_options(o):
    assert tio.get_typed_option(o, "string", str) == ("blah", 0)
    assert tio.get_typed_option(o, "int", int) == (2, 0)
    v, e = tio.get_typed_option(o, "double", float)
    assert e == 0 and abs(v - 3.45) < 0.01
    assert tio.get_typed_option(o, "logical", bool) == (True, 0)


def _check_typed_test_options(o):
    assert tio.get_typed_option(o, "string_type", str) == ("blah_type", 0)
    assert tio.get_typed_option(o, "int_type", int) == (6, 0)
    v, e = tio.get_typed_option(o, "double_type", float)
    assert e == 0 and abs(v - 7.89) < 0.01
    assert tio.get_typed_option(o, "logical_type", bool) == (False, 0)


def test_put_option_typed_and_untyped():
    o = {}
    _add_test_options(o)
    _add_typed_test_options(o)
    assert len(o) == 9
    _check_test_options(o)
    _check_typed_test_options(o)
    # the edit descriptors of the typed putters: I10, F20.10, L1
    assert o["int"] == "         2" and o["double"] == "        3.4500000000" and o["logical"] == "T"
    assert o["logical_type"] == "F"


def test_multiple_put_option_overwrites_in_place():
    o = {}
    tio.put_option(o, "key", "blah")
    assert len(o) == 1 and tio.get_option(o, "key") == ("blah", 0)
    tio.put_option(o, "key_two", "two_blah")
    assert len(o) == 2 and tio.get_option(o, "key_two") == ("two_blah", 0)
    tio.put_option(o, "key", "tpls")
    assert len(o) == 2 and tio.get_option(o, "key") == ("tpls", 0)
    tio.put_option(o, "key", "dim")
    assert len(o) == 2 and tio.get_option(o, "key") == ("dim", 0)
    tio.put_option(o, "key_two", "69")
    assert len(o) == 2 and tio.get_option(o, "key_two") == ("69", 0)
    tio.put_option(o, "key_3", "This is another value")
    assert len(o) == 3 and tio.get_option(o, "key_3") == ("This is another value", 0)
    assert list(o) == ["key", "key_two", "key_3"]


HEADER = ["options_utils_test header", "Automatically created by options_utils_test", "Options now follow..."]


def test_save_and_load_options(tmp_path):
    f = tmp_path / "test_options_utils.tmp"
    o = {}
    _add_test_options(o)
    _add_typed_test_options(o)
    tio.save_options(f, o, HEADER)
    lines = f.read_text().splitlines()
    assert lines[:3] == ["# " + h for h in HEADER] and lines[3] == "string blah"
    got, ierr = tio.load_options(f)
    assert ierr == 0 and len(got) == 9
    _check_test_options(got)
    _check_typed_test_options(got)


def test_save_append_load_options(tmp_path):
    f = tmp_path / "test_options_utils.tmp"
    a, b = {}, {}
    _add_test_options(a)
    tio.save_options(f, a, HEADER)
    _add_typed_test_options(b)
    tio.append_options(f, b)
    got, ierr = tio.load_options(f)
    assert ierr == 0 and len(got) == 9
    _check_test_options(got)
    _check_typed_test_options(got)


def test_load_options_not_found(tmp_path):
    assert tio.load_options(tmp_path / "blah.tmp") == ({}, tio.OPTION_FILE_NOT_FOUND_ERR)
    assert tio.OPTION_FILE_NOT_FOUND_ERR == 103


def test_load_options_format_error(tmp_path):
    f = tmp_path / "test_options_utils.tmp"
    f.write_text("# Comment\n# Comment\n# Comment\nkey value\ninteger 123\nk v\ninvalidvalue\n")
    opts, ierr = tio.load_options(f)
    assert ierr == tio.OPTION_FORMAT_ERR == 101
    assert opts == {"key": "value", "integer": "123", "k": "v"}


def test_load_duplicates_keep_the_last_value(tmp_path):
    f = tmp_path / "test_options_utils.tmp"
    f.write_text("key 123\nkey 456\nkey 789\nkey abc\nkey check\n")
    opts, ierr = tio.load_options(f)
    assert ierr == 0 and len(opts) == 1 and tio.get_option(opts, "key") == ("check", 0)


def test_load_options_line_rules(tmp_path):
    """Split at the first space only (a tab does not separate), leading
    blanks of a value kept, indented comments and blank lines skipped, names
    cut to 20 characters, values to 60, lines to 80."""
    f = tmp_path / "rules.opt"
    long_name = "n" * 25
    f.write_text("   # indented comment\n\n   \nre   200.0\n" + f"{long_name} 1\n" + "v " + "x" * 70 + "\n")
    opts, ierr = tio.load_options(f)
    assert ierr == 0
    assert opts["re"] == "  200.0" and tio.get_double_option(opts, "re") == (200.0, 0)
    assert opts["n" * 20] == "1"
    assert opts["v"] == "x" * 60
    g = tmp_path / "tab.opt"
    g.write_text("key\tvalue\n")
    assert tio.load_options(g)[1] == tio.OPTION_FORMAT_ERR


def test_list_directed_values():
    o = _opts([("i", " 7 8"), ("d", "1.5d-3"), ("e", "2,5"), ("bad_i", "2.5"), ("bad_d", "abc"),
               ("l1", ".false."), ("l2", "Tremendous"), ("bad_l", "yes")])
    assert tio.get_integer_option(o, "i") == (7, 0)
    assert tio.get_double_option(o, "d") == (1.5e-3, 0)
    assert tio.get_double_option(o, "e") == (2.0, 0)
    assert tio.get_integer_option(o, "bad_i") == (None, tio.OPTION_INVALID_ERR)
    assert tio.get_double_option(o, "bad_d") == (None, tio.OPTION_INVALID_ERR)
    assert tio.get_logical_option(o, "l1") == (False, 0)
    assert tio.get_logical_option(o, "l2") == (True, 0)
    assert tio.get_logical_option(o, "bad_l") == (None, tio.OPTION_INVALID_ERR)


def test_typed_putter_overflow_fields():
    o = {}
    tio.put_integer_option(o, "big", 12345678901)
    tio.put_double_option(o, "huge", 1e12)
    assert o["big"] == "*" * 10 and o["huge"] == "*" * 20


def test_command_line_options():
    assert tio.get_command_line_options(["-n", "5", "-v"]) == {"-n": "5", "-v": ""}
    # a flag after a flag still waiting for its value is dropped, as in the reference
    assert tio.get_command_line_options(["-a", "-b", "1"]) == {"-a": "1"}
    assert tio.get_command_line_options(["stray", "-x", "y"]) == {"-x": "y"}


def test_option_messages_and_print():
    assert tio.missing_option_message("maxl") == "Error: Missing value: maxl"
    assert tio.invalid_option_message("re", 3, "positive") == "Error: Invalid value: re      3 positive"
    assert tio.invalid_option_message("dt", 0.5, "x") == "Error: Invalid value: dt         0.5000000000 x"
    assert tio.invalid_option_message("flag", True, "L") == "Error: Invalid value: flag T L"
    assert tio.invalid_option_message("idm", "abc", "lsm|dim") == "Error: Invalid value: idm abc lsm|dim"
    buf = _io.StringIO()
    tio.print_options({"a": "1", "b": "two"}, file=buf)
    assert buf.getvalue() == "a 1\nb two\n"


# ---- point files (io_test.f90) ---------------------------------------------

L, M, N = 9, 5, 5
DX, DY, DZ = 0.1, 0.2, 0.3


def _out_data(l, m, n):
    i = np.arange(l + 1)[:, None, None]
    j = np.arange(m + 1)[None, :, None]
    k = np.arange(n + 1)[None, None, :]
    return ((i + 1) * (j + 2) * (k + 3)).astype(np.float64)


def test_channel_output_and_input_phi_round_trip(tmp_path):
    f = tmp_path / "test_tpls_io.tmp"
    d = _out_data(L, M, N)
    tio.channel_output_phi(d, L, M, N, DX, DY, DZ, f)
    lines = f.read_text().splitlines()
    assert lines[0] == ' VARIABLES="X ","Y ","Z ","Phi"'
    assert lines[1].split()[:2] == ["ZONE", 'T="Floor",']
    assert len(lines) == 2 + (L - 1) * (M - 1) * (N - 1)
    x, y, z, v = (float(t) for t in lines[2].split())
    assert (x, y, z, v) == (DX / 2 + DX * 1, DY / 2, DZ / 2, d[2, 0, 1])
    got, ierr = tio.channel_input_phi(f, L, M, N)
    assert ierr == 0
    for k in range(N - 1):
        for j in range(M - 1):
            for i in range(1, L):
                assert got[i + 1, j, k + 1] == d[i + 1, j, k + 1]


def test_channel_input_phi_layouts(tmp_path):
    """Four items per row, across records if need be, the rest of a record
    skipped; a short file reports ierr 1."""
    f = tmp_path / "p.tmp"
    f.write_text("h1\nh2\n 0.1 0.2 0.3 1.5D0 99 99\n 0.1 0.2\n 0.3 -2.5\n")
    got, ierr = tio.channel_input_phi(f, 2, 2, 3)   # (l-1)(m-1)(n-1) = 2 rows
    assert ierr == 0 and got[2, 0, 1] == 1.5 and got[2, 0, 2] == -2.5
    got, ierr = tio.channel_input_phi(f, 2, 2, 4)   # 3 rows expected
    assert ierr == 1


def test_channel_output_uvw(tmp_path):
    f = tmp_path / "test_tpls_io.tmp"
    d = _out_data(L, M, N)
    tio.channel_output_uvw(d, d, d, d, L, M, N, DX, DY, DZ, f)
    lines = f.read_text().splitlines()
    assert lines[0] == ' VARIABLES="X ","Y ","Z ","U","V","W","P"'
    assert len(lines) == 2 + (L - 1) * (M - 1) * (N - 1)
    row = [float(t) for t in lines[2].split()]   # i = 1, j = 0, k = 0
    assert row == [DX / 2 + DX, DY / 2, DZ / 2, (d[1, 0, 0] + d[2, 0, 0]) / 2, (d[1, 0, 0] + d[1, 1, 0]) / 2,
                   (d[1, 0, 0] + d[1, 0, 1]) / 2, d[1, 0, 1]]


def test_channel_output2d(tmp_path):
    f = tmp_path / "test_tpls_io.tmp"
    d = _out_data(L, M, N)
    tio.channel_output2d(d, d, d, d, d, d, L, M, N, DX, DY, DZ, f)
    lines = f.read_text().splitlines()
    assert lines[0] == ' VARIABLES="X ","Z ","U","V","W","P","fi","Viscosity"'
    assert len(lines) == 2 + (L - 1) * (N - 1)
    j = (M - 1) // 2
    row = [float(t) for t in lines[2].split()]   # i = 1, k = 0
    assert row[:2] == [DX / 2 + DX, DZ / 2]
    assert row[5:] == [d[1, j, 1], d[2, j, 1], d[1, j, 1]]


def test_row_to_grid_traversal():
    l, m, n = 9, 5, 4
    row = 1
    for k in range(n + 1):
        for j in range(m + 1):
            for i in range(l + 1):
                assert tio.row_to_grid(0, l, 0, m, 0, n, row) == (i, j, k)
                row += 1


def test_filepath_and_backup_info(tmp_path):
    assert tio.get_filepath("out  ", "phi.dat ") == "out/phi.dat"
    f = tmp_path / "info.txt"
    tio.save_backup_info(f, 0, 9, 0, 5, 0, 5, 1, 2, 3)
    lines = f.read_text().splitlines()
    assert [int(t) for t in lines[1].split()] == [0, 9, 0, 5, 0, 5]
    assert [int(t) for t in lines[3].split()] == [1, 2, 3]


@pytest.mark.parametrize("value", [0.0, -1.25, 1e-300, 123456.789])
def test_point_rows_round_trip_exactly(tmp_path, value):
    f = tmp_path / "one.tmp"
    phi = np.zeros((3, 3, 3))
    phi[2, 0, 1] = value
    tio.channel_output_phi(phi, 2, 2, 2, DX, DY, DZ, f)
    got, ierr = tio.channel_input_phi(f, 2, 2, 2)
    assert ierr == 0 and got[2, 0, 1] == value
