"""C-ABI library checks that need no GPU: the shared library loads, exports
every function include/tpls_gpu.h declares, and its host-only entries
(status strings, argument validation before any device call, the 1-D base
profile) behave as documented."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from tpls_gb300.api import LIB_PATH, Params, base_profile, load_library
from tpls_gb300.channel import make_case

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"//[^\n]*|/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tpls_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("tpls_gpu_create", "tpls_step", "tpls_pressure_solve", "tpls_do_sor_u",
              "tpls_get_difference_noalloc", "tpls_exchange2d"):
        assert n in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    assert LIB_PATH.exists(), "build the library first"
    lib = C.CDLL(str(LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    lib = load_library()
    for code, text in ((0, b"ok"), (1, b"bad argument"), (3, b"call sequence"), (-3, b"DIVERGED_ITS"),
                       (5, b"")):
        s = lib.tpls_status_string(code)
        assert s is not None and text in s


def test_create_rejects_bad_arguments_before_device_work():
    """Argument checks run before the first CUDA call, so they hold on a
    machine without a GPU."""
    lib = load_library()
    params, uin, _ = make_case("A")
    cp = params.to_c()
    out = C.c_void_p()
    uin = np.ascontiguousarray(uin)
    up = uin.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.tpls_gpu_create(2, 32, 48, C.byref(cp), up, C.byref(out)) == 1   # nx < 4
    assert lib.tpls_gpu_create(64, 32, 48, None, up, C.byref(out)) == 1
    bad = Params(**{**params.__dict__, "dt": 0.0}).to_c()
    assert lib.tpls_gpu_create(64, 32, 48, C.byref(bad), up, C.byref(out)) == 1
    badp = Params(**{**params.__dict__, "precision": 7}).to_c()
    assert lib.tpls_gpu_create(64, 32, 48, C.byref(badp), up, C.byref(out)) == 1
    # the diffuse-interface method: FP64 form only, with epn > 0 and Pe > 0
    dparams, _, _ = make_case("A", idm="dim")
    for change in ({"precision": 1}, {"epn": 0.0}, {"pe": 0.0}, {"max_iteration_dim": -1}, {"idm": 2}):
        bd = Params(**{**dparams.__dict__, **change}).to_c()
        assert lib.tpls_gpu_create(64, 32, 48, C.byref(bd), up, C.byref(out)) == 1, change
    assert not out.value


def test_base_profile_matches_oracle_recurrence():
    """tpls_base_profile (host code in the library) against a numpy
    restatement of twophase_initialisation_wave.F90:79-122."""
    nz, dz, re_, dpdl, mm, mp, h, sw = 24, 1.0 / 24, 100.0, -1.0, 2.0, 1.0, 0.5, 1.5 * 2 * np.pi / 64
    u = base_profile(nz, dz, re_, dpdl, mm, mp, h, sw)
    pi = float(np.float32(3.14159265359))
    n = nz + 1
    z = dz * np.arange(n + 1) - dz / 2.0
    ph = z - h
    hv = np.where(ph < -sw, 0.0, np.where(ph > sw, 1.0, 0.5 + ph / (2 * sw) + np.sin(pi * ph / sw) / (2 * pi)))
    visc = (mp * hv + mm * (1.0 - hv)) / re_
    ref = np.zeros(n - 1)
    for _ in range(10000):
        for k in range(n - 1):
            umz = -2.0 * ref[0] + ref[1] / 3.0 if k == 0 else ref[k - 1]
            upz = -2.0 * ref[n - 2] + ref[n - 3] / 3.0 if k == n - 2 else ref[k + 1]
            mmk = (visc[k] + visc[k + 1]) / 2.0
            mpk = (visc[k + 2] + visc[k + 1]) / 2.0
            diag = (mpk + mmk) / (dz * dz)
            ref[k] = (1.0 / diag) * (((mpk * upz + mmk * umz) / (dz * dz)) - dpdl)
    assert np.max(np.abs(u - ref[:nz])) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("cls_name,c_name", [("TplsParams", "tpls_params"),
                                             ("TplsStats", "tpls_stats")])
def test_ctypes_structs_match_header_layout(tmp_path, cls_name, c_name):
    """The Python mirrors of the header's structs have the C compiler's size and
    field offsets (a drifted mirror would pass garbage to every entry point)."""
    import shutil
    import subprocess
    import tpls_gb300.api as api
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cls = getattr(api, cls_name)
    lines = [f'printf("size %zu\\n", sizeof({c_name}));']
    for f, _ in cls._fields_:
        lines.append(f'printf("{f} %zu\\n", offsetof({c_name}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"tpls_gpu.h\"\n"
                   "int main(void) {\n" + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = dict(line.split() for line in out.splitlines())
    assert int(got["size"]) == C.sizeof(cls)
    for f, _ in cls._fields_:
        assert int(got[f]) == getattr(cls, f).offset, f


def test_base_profile_matches_oracle_restatement():
    """The library's tpls_base_profile and the oracle's restatement of
    twophase_initialisation_wave.F90:79-122 agree bit for bit (both host
    code, same operation order), on cubic cells and on the 2*pi x pi x 1
    channel's smoothing width."""
    from oracle.oracle import base_profile as orc_profile
    for nz, sw in ((48, 1.5 / 48), (23, 1.5 * 2 * np.pi / 37)):
        args = (nz, 1.0 / nz, 200.0, -1.0, 2.0, 1.0, 0.5, sw)
        np.testing.assert_array_equal(base_profile(*args), orc_profile(*args))


def test_missing_native_library_fails_loudly(tmp_path, monkeypatch):
    """No CPU fallback: without the built library the loader and the context
    constructor raise instead of computing anything."""
    import tpls_gb300.api as api
    with pytest.raises(api.TplsError, match="not found"):
        api.load_library(tmp_path / "missing.so")
    params, uin, _ = make_case("A", nx=8, ny=4, nz=6)   # uses the library: before removing it
    monkeypatch.setattr(api, "LIB_PATH", tmp_path / "missing.so")
    monkeypatch.setattr(api, "_lib", None)
    with pytest.raises(api.TplsError, match="not found"):
        api.TplsGpu(8, 4, 6, params, uin)
