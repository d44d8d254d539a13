"""Build the in-tree native libraries.

* ``tpls_gb300/_lib/libtpls_gb300.so`` -- the CUDA (sm_103a) kernels and the
  C ABI of ``include/tpls_gpu.h``; one nvcc process per translation unit, run
  in parallel, then one link step.
* ``oracle/_build/liboracle.so`` -- the CPU restatement used as the parity
  oracle and CPU baseline (test infrastructure; built here only so tests and
  the bench find it).

Neither uses cmake; both finish in well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "tpls_gb300" / "csrc"
LIBDIR = ROOT / "tpls_gb300" / "_lib"
OBJDIR = ROOT / "tpls_gb300" / "_build"
LIB = LIBDIR / "libtpls_gb300.so"
ORACLE_SRC = ROOT / "oracle" / "tpls_oracle.c"
ORACLE_LIB = ROOT / "oracle" / "_build" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tpls_gb300")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("TPLS_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)


def _code_only(text: str) -> str:
    """C/C++ source with its comments removed (string and character
    literals kept) and every run of white space outside literals made one
    space, so a comment or layout edit does not change the digest."""
    out, i, n = [], 0, len(text)
    while i < n:
        ch = text[i]
        if ch in "\"'":
            j = i + 1
            while j < n and text[j] != ch:
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        elif ch.isspace():
            j = i
            while j < n and text[j].isspace():
                j += 1
            if out and out[-1] != " ":
                out.append(" ")
            i = j
        else:
            out.append(ch)
            i += 1
    return "".join(out)


def source_digest() -> str:
    """12 hex digits of SHA-256 over the CUDA sources and headers (their
    code, comments removed) and the build flags: names the build an ncu
    capture was taken of."""
    import hashlib
    h = hashlib.sha256(" ".join(ARCH + NVCC_FLAGS[:-1]).encode())
    files = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))
    for f in files + [ROOT / "include" / "tpls_gpu.h"]:
        h.update(f.name.encode())
        h.update(_code_only(f.read_text()).encode())
    return h.hexdigest()[:12]


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_cuda(force: bool = False, ptxas_verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OBJDIR.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    units = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "tpls_gpu.h"]
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []

    def compile_one(cu: Path) -> Path:
        obj = OBJDIR / (cu.stem + ".o")
        if force or _stale(obj, [cu] + headers):
            _run([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(cu), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(units))) as ex:
        objs = list(ex.map(compile_one, units))
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    srcs = [ORACLE_SRC, ORACLE_SRC.with_suffix(".h"), ROOT / "include" / "tpls_gpu.h"]
    if force or _stale(ORACLE_LIB, srcs):
        cc = shutil.which("gcc") or "cc"
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run([cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
              "-o", str(tmp), str(ORACLE_SRC), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_cuda(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
