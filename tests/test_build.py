"""Host-side build bookkeeping (no GPU): the source digest that names the
build an ncu capture was taken of ignores comments and layout but not code,
and the bench reads a committed capture's figures only for the build they
were taken of."""
from pathlib import Path

import pytest

from tpls_gb300 import build


def test_code_only_drops_comments_and_layout_but_keeps_literals():
    src = 'int a = 1; // one\n/* block\n comment */ const char *s = "x // y /* z */";\n\n\tchar q = \'/\';\n'
    assert build._code_only(src) == 'int a = 1; const char *s = "x // y /* z */"; char q = \'/\'; '
    assert build._code_only("a  =\n b;\n") == build._code_only("a = b; // note\n")
    assert build._code_only("a = b;") != build._code_only("a = c;")
    assert build._code_only('s = "a\\"//b";') == 's = "a\\"//b";'


def test_source_digest_follows_code_not_comments(tmp_path, monkeypatch):
    csrc = tmp_path / "csrc"
    inc = tmp_path / "include"
    csrc.mkdir()
    inc.mkdir()
    (inc / "tpls_gpu.h").write_text("int f(void);\n")
    k = csrc / "k.cu"
    monkeypatch.setattr(build, "CSRC", csrc)
    monkeypatch.setattr(build, "ROOT", tmp_path)
    k.write_text("__global__ void k(int *x) { x[0] = 1; }\n")
    d0 = build.source_digest()
    k.write_text("// the kernel\n__global__ void k(int *x) {\n  x[0] = 1;  /* one */\n}\n")
    assert build.source_digest() == d0
    k.write_text("__global__ void k(int *x) { x[0] = 2; }\n")
    assert build.source_digest() != d0
    assert len(d0) == 12


def test_bench_reads_capture_figures_with_their_build(tmp_path, monkeypatch):
    bench = pytest.importorskip("bench")
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "kernels_x.md").write_text(
        "text\n\n    traffic k_sor_odd_seg 256x128x192-fp64: 265000000 build abcdef012345\n"
        "    fp64pipe k_sor_odd_seg 192x96x144-fp64: 64 build abcdef012345\n")
    monkeypatch.setattr(bench, "ROOT", Path(tmp_path))
    monkeypatch.setattr(build, "source_digest", lambda: "abcdef012345")
    t = bench._profile_figure("traffic", "k_sor_odd_seg", "256x128x192-fp64")
    assert t["value"] == 265000000 and t["current"] and t["workload"] == "256x128x192-fp64"
    assert bench._profile_figure("traffic", "k_sor_odd_seg", "512x256x256-mixed") is None
    f = bench._profile_figure("fp64pipe", "k_sor_odd_seg", None)
    assert f["value"] == 64 and f["workload"] == "192x96x144-fp64"
    monkeypatch.setattr(build, "source_digest", lambda: "000000000000")
    assert not bench._profile_figure("traffic", "k_sor_odd_seg", "256x128x192-fp64")["current"]
