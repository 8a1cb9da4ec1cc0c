"""Runs the reference's own CUDA clustering program (CUDA/signalNode) to
produce golden outputs.  Test infrastructure.

    python oracle/ref_cluster.py stage        # where the reference tree exists
    python oracle/ref_cluster.py run OUTDIR   # on a GPU host

`stage` copies the program's five source files (cluster.cpp, func.cu,
func.h, cmdline.h, timer.h) unchanged into baseline/_ref/signalNode/ — the
git-ignored directory that carries the reference install to GPU hosts.
`run` compiles them there with nvcc for sm_103a exactly as the reference
Makefile line does (nvcc src/cluster.cpp src/func.cu -o cluster), adding only
-gencode and `-include oracle/ref_copykind.h`, builds each golden fixture's
database with the makeDB drop-in (byte-identical to the reference makeDB, see
manifest.json), runs the reference on every parameter set twice, and copies
cluster.txt / represent.fasta to OUTDIR/<fixture>/<tag>/ (flagging any run
whose two outputs differ).
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
STAGE = ROOT / "baseline" / "_ref" / "signalNode"
REFERENCE = Path(os.environ.get("NGIA_REFERENCE_DIR", "/root/reference"))
FILES = ["cluster.cpp", "func.cu", "func.h", "cmdline.h", "timer.h"]


def stage() -> None:
    src = REFERENCE / "CUDA" / "signalNode" / "src"
    (STAGE / "src").mkdir(parents=True, exist_ok=True)
    for f in FILES:
        shutil.copyfile(src / f, STAGE / "src" / f)
    print("staged", STAGE)


def build() -> Path:
    exe = STAGE / "cluster"
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-include", str(HERE / "ref_copykind.h"),
           str(STAGE / "src" / "cluster.cpp"), str(STAGE / "src" / "func.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise SystemExit("reference build failed:\n" + r.stderr)
    return exe


def run(outdir: str) -> None:
    sys.path.insert(0, str(ROOT / "ngia-metax_gb300"))
    import ngia

    exe = build()
    golden = ROOT / "tests" / "golden"
    manifest = json.loads((golden / "manifest.json").read_text())
    out = Path(outdir)
    report = {}
    for name, m in manifest.items():
        dbdir = out / "_db" / name
        dbdir.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(golden / f"{name}.fasta", dbdir / "in.fasta")
        ngia.makedb(str(dbdir / "in.fasta"), str(dbdir), m["type"])
        for s, w, p in m["params"]:
            tag = f"s{s}_w{w}_p{p}"
            runs = []
            for k in range(2):
                od = out / name / tag / f"run{k}"
                od.mkdir(parents=True, exist_ok=True)
                t0 = time.time()
                r = subprocess.run([str(exe), "-i", str(dbdir), "-o", str(od), "-w", str(w), "-s", str(s), "-p",
                                    str(p)], capture_output=True, text=True, timeout=600)
                runs.append((r.returncode, time.time() - t0, (od / "cluster.txt").read_bytes() if
                             (od / "cluster.txt").exists() else b""))
            same = runs[0][2] == runs[1][2]
            final = out / name / tag
            for f in ("cluster.txt", "represent.fasta"):
                shutil.copyfile(final / "run0" / f, final / f)
            report[f"{name}/{tag}"] = {"rc": [r[0] for r in runs], "seconds": [round(r[1], 3) for r in runs],
                                       "deterministic": same}
    (out / "report.json").write_text(json.dumps(report, indent=1) + "\n")
    print(json.dumps(report, indent=1))


if __name__ == "__main__":
    if sys.argv[1] == "stage":
        stage()
    elif sys.argv[1] == "run":
        run(sys.argv[2])
