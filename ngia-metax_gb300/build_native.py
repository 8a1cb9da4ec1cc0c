"""Build recipe of the native library and command-line tools.

Outputs (git-ignored) go to ``ngia-metax_gb300/_build/``:

* ``libngia.so``   C ABI of include/ngia.h: CUDA kernels for sm_103a + host code
* ``cluster``      drop-in for the reference ``cluster`` program
* ``makeDB``       drop-in for the reference ``makeDB`` tool
* ``ngia_synth``   seeded synthetic FASTA generator

Translation units compile in parallel; nothing is rebuilt when the sources
are older than the outputs.  Only nvcc and g++ are needed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
OUT = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")

CU_SOURCES = ["csrc/filter.cu", "csrc/align.cu", "csrc/api.cu", "csrc/probe.cu", "csrc/noalloc.cu", "csrc/batch.cu", "csrc/serve.cu", "csrc/checkpoint.cu", "csrc/tune.cu", "csrc/spec.cu", "csrc/pool.cu"]
CPP_SOURCES = ["host/errors.cpp", "host/synth.cpp", "host/dbformat.cpp"]
TOOLS = {"cluster": "host/cluster_main.cpp", "makeDB": "host/makedb_main.cpp", "ngia_synth": "host/synth_main.cpp"}

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return list((PKG / "csrc").glob("*.cuh")) + list((PKG / "csrc").glob("*.h")) + \
        list((PKG / "host").glob("*.h")) + [ROOT / "include" / "ngia.h"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _compile(src: str, verbose_ptxas: bool = False) -> Path:
    s = PKG / src
    o = OUT / (Path(src).stem + (".cu.o" if src.endswith(".cu") else ".o"))
    if _stale(o, [s] + _headers()) or verbose_ptxas:
        if src.endswith(".cu"):
            extra = ["-Xptxas", "-v"] if verbose_ptxas else []
            _run([NVCC] + NVFLAGS + extra + ["-c", str(s), "-o", str(o)])
        else:
            _run([CXX] + CXXFLAGS + ["-c", str(s), "-o", str(o)])
    return o


def build(jobs: int | None = None, verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    lib = OUT / "libngia.so"
    if _stale(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs] +
             ["-cudart", "static", "-Xcompiler", "-pthread"])
    for name, src in TOOLS.items():
        exe = OUT / name
        s = PKG / src
        if _stale(exe, [s, lib] + _headers()):
            _run([CXX] + CXXFLAGS + [str(s), "-o", str(exe), f"-L{OUT}", "-lngia",
                  "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}")
    return lib


def ptxas_report() -> str:
    """Registers / spills / shared memory of every kernel (nvcc -Xptxas -v)."""
    OUT.mkdir(parents=True, exist_ok=True)
    lines = []
    for src in CU_SOURCES:
        s = PKG / src
        r = subprocess.run([NVCC] + NVFLAGS + ["-Xptxas", "-v", "-c", str(s), "-o", os.devnull],
                           capture_output=True, text=True)
        lines.append(r.stderr)
    return "\n".join(lines)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report())
    else:
        build(verbose=True)
