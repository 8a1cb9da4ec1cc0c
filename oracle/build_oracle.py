"""Build recipe of the CPU oracle (test infrastructure) and of the reference's
own makeDB tool.

* ``oracle/_build/liboracle.so`` and ``oracle/_build/ngia_oracle``: the C
  restatement of the reference clustering (gcc, OpenMP, -ffp-contract=off).
* ``oracle/_build/libsynth.so``: the seeded workload generator
  (ngia-metax_gb300/host/synth.cpp, the same source the product library
  carries) on its own, so that the timed CPU reference arm builds its inputs
  without loading the product library.
* ``oracle/_ref/makeDB``: the reference makeDB compiled from its single
  source file where it lies (``makeDB/src/makeDB.cpp`` of the reference
  tree, with its own cmdline.h / timer.h headers), exactly as its Makefile
  line ``g++ -fopenmp src/makeDB.cpp`` does.  Built only when the reference
  tree is present (it is not on GPU hosts); used to pin the database format.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("NGIA_REFERENCE_DIR", "/root/reference"))
CC = os.environ.get("CC", "gcc")
CXX = os.environ.get("CXX", "g++")
CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-std=gnu11", "-Wall"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    return not target.exists() or any(d.stat().st_mtime > target.stat().st_mtime for d in deps)


def build_oracle() -> Path:
    OUT.mkdir(exist_ok=True)
    src = [HERE / "ngia_oracle.c"]
    hdr = [HERE / "ngia_oracle.h"]
    lib = OUT / "liboracle.so"
    if _stale(lib, src + hdr):
        _run([CC] + CFLAGS + ["-fPIC", "-shared", str(src[0]), "-o", str(lib), "-lm"])
    exe = OUT / "ngia_oracle"
    if _stale(exe, src + hdr + [HERE / "oracle_main.c"]):
        _run([CC] + CFLAGS + [str(HERE / "oracle_main.c"), str(src[0]), "-o", str(exe), "-lm"])
    gen_src = [ROOT / "ngia-metax_gb300" / "host" / f for f in ("synth.cpp", "errors.cpp")]
    gen = OUT / "libsynth.so"
    if _stale(gen, gen_src + list((ROOT / "ngia-metax_gb300" / "host").glob("*.h")) + [ROOT / "include" / "ngia.h"]):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-Wl,-Bsymbolic"] +
             [str(x) for x in gen_src] + ["-o", str(gen)])
    nofma = OUT / "liboracle_nofma.so"  # separately rounded band shift (fixture search only)
    if _stale(nofma, src + hdr):
        _run([CC] + CFLAGS + ["-DORA_BAND_NOFMA", "-fPIC", "-shared", str(src[0]), "-o", str(nofma), "-lm"])
    return lib


def build_ref() -> Path | None:
    """Reference makeDB from its own source file; None when the tree is absent."""
    src = REFERENCE / "makeDB" / "src" / "makeDB.cpp"
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    exe = REF_OUT / "makeDB"
    if not exe.exists():
        _run([CXX, "-O2", "-fopenmp", str(src), "-o", str(exe)])
    return exe


def stage_ref_program() -> None:
    """Copies the reference's CUDA clustering sources into baseline/_ref
    (the git-ignored directory that travels to GPU hosts) when the reference
    tree is present and they are not staged yet; see ref_cluster.py."""
    if not (REFERENCE / "CUDA" / "signalNode" / "src" / "func.cu").exists():
        return
    import sys

    if str(HERE.parent) not in sys.path:
        sys.path.insert(0, str(HERE.parent))
    from oracle import ref_cluster

    if not (ref_cluster.STAGE / "src" / "func.cu").exists():
        ref_cluster.stage()


def build() -> None:
    build_oracle()
    build_ref()
    stage_ref_program()


if __name__ == "__main__":
    build()
    print("oracle built:", OUT)
