"""Runs the reference's own CUDA clustering program (CUDA/signalNode) to
produce golden outputs.  Test infrastructure.

    python oracle/ref_cluster.py stage        # where the reference tree exists
    python oracle/ref_cluster.py run OUTDIR [FIXTURE ...]   # on a GPU host

`stage` copies the program's five source files (cluster.cpp, func.cu,
func.h, cmdline.h, timer.h) unchanged into baseline/_ref/signalNode/ — the
git-ignored directory that carries the reference install to GPU hosts.
`compare OUTDIR --workload W` runs the reference and the drop-in `cluster`
on one generated workload, times both and byte-compares their outputs.

`run` compiles them there with nvcc for sm_103a exactly as the reference
Makefile line does (nvcc src/cluster.cpp src/func.cu -o cluster), adding only
-gencode and `-include oracle/ref_copykind.h`, builds each golden fixture's
database with the makeDB drop-in (byte-identical to the reference makeDB, see
manifest.json), runs the reference on every parameter set twice, and copies
cluster.txt / represent.fasta to OUTDIR/<fixture>/<tag>/ (flagging any run
whose two outputs differ).  For a generated fixture (manifest "generated")
the FASTA is written from its generator first and the outputs are recorded
as md5s in OUTDIR/<fixture>/<tag>/outputs.json.

The reference tree is read where this build container mounts it
(NGIA_REFERENCE_DIR overrides the location); only `stage` reads it.
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
    srcs = [STAGE / "src" / f for f in FILES] + [HERE / "ref_copykind.h"]
    if exe.exists() and all(s.stat().st_mtime <= exe.stat().st_mtime for s in srcs):
        return exe
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-include", str(HERE / "ref_copykind.h"),
           str(STAGE / "src" / "cluster.cpp"), str(STAGE / "src" / "func.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise SystemExit("reference build failed:\n" + r.stderr)
    return exe


def _md5(path: Path) -> str:
    import hashlib

    return hashlib.md5(path.read_bytes()).hexdigest()


def run(outdir: str, only: list[str] | None = None) -> None:
    sys.path.insert(0, str(ROOT / "ngia-metax_gb300"))
    sys.path.insert(0, str(ROOT))
    import ngia
    from tests.golden.make_golden import fixture_fasta

    exe = build()
    golden = ROOT / "tests" / "golden"
    manifest = json.loads((golden / "manifest.json").read_text())
    out = Path(outdir)
    report = {}
    for name, m in manifest.items():
        if only and name not in only:
            continue
        dbdir = out / "_db" / name
        dbdir.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(fixture_fasta(name, m, dbdir), dbdir / "in.fasta")
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
            if m.get("generated"):
                n_clusters = sum(1 for ln in (final / "run0" / "cluster.txt").read_bytes().splitlines()
                                 if not ln.startswith(b" "))
                (final / "outputs.json").write_text(json.dumps(
                    {f: _md5(final / "run0" / f) for f in ("cluster.txt", "represent.fasta")} |
                    {"clusters": n_clusters}, indent=1) + "\n")
            else:
                for f in ("cluster.txt", "represent.fasta"):
                    shutil.copyfile(final / "run0" / f, final / f)
            for k in range(2):
                shutil.rmtree(final / f"run{k}", ignore_errors=True)
            report[f"{name}/{tag}"] = {"rc": [r[0] for r in runs], "seconds": [round(r[1], 3) for r in runs],
                                       "deterministic": same}
    (out / "report.json").write_text(json.dumps(report, indent=1) + "\n")
    print(json.dumps(report, indent=1))


def compare(outdir: str, workload: str, similarity: float, word: int, n_seqs: int = 0, seed: int = 1,
            timeout: int = 1200, quiet: bool = False) -> dict:
    """Generates a workload, runs the reference `cluster` and the drop-in
    `cluster` on the same database, times both (wall clock, including their
    own database loading and result writing) and byte-compares the outputs."""
    sys.path.insert(0, str(ROOT / "ngia-metax_gb300"))
    import ngia

    t_build = time.time()
    exe = build()
    t_build = time.time() - t_build
    out = Path(outdir)
    dbdir, o_ref, o_new = out / "db", out / "ref", out / "ours"
    for d in (dbdir, o_ref, o_new):
        d.mkdir(parents=True, exist_ok=True)
    cfg = dict(ngia.CONFIGS[workload])
    if n_seqs:
        cfg["n_seqs"] = n_seqs
    seqs = ngia.synth(**cfg, seed=seed)
    ngia.write_fasta(str(dbdir / "in.fasta"), seqs, seqs.off, width=80)
    seqs.close()
    ngia.makedb(str(dbdir / "in.fasta"), str(dbdir), cfg["type"])
    args = ["-i", str(dbdir), "-w", str(word), "-s", str(similarity)]
    res = {"workload": workload, "n_seqs": cfg["n_seqs"], "similarity": similarity, "word": word,
           "reference_build_s": round(t_build, 1),
           "timing": "wall clock of each whole program (CUDA start-up, database load, clustering, result files)"}
    for name, cmd, od in (("reference", [str(exe)], o_ref),
                          ("ours", [str(ROOT / "ngia-metax_gb300" / "_build" / "cluster")], o_new)):
        t0 = time.time()
        try:
            r = subprocess.run(cmd + args + ["-o", str(od)], capture_output=True, text=True, timeout=timeout)
            res[name] = {"rc": r.returncode, "seconds": round(time.time() - t0, 3),
                         "clusters": next((ln.split("\t")[1] for ln in r.stdout.splitlines()
                                           if ln.startswith("Cluster:")), None)}
        except subprocess.TimeoutExpired:
            res[name] = {"rc": None, "seconds": timeout, "timeout": True}
    same = all((o_ref / f).exists() and (o_ref / f).read_bytes() == (o_new / f).read_bytes()
               for f in ("cluster.txt", "represent.fasta"))
    res["outputs_identical"] = same
    shutil.rmtree(dbdir, ignore_errors=True)
    (out / "compare.json").write_text(json.dumps(res, indent=1) + "\n")
    if not quiet:
        print(json.dumps(res))
    return res


if __name__ == "__main__":
    if sys.argv[1] == "stage":
        stage()
    elif sys.argv[1] == "run":
        run(sys.argv[2], sys.argv[3:] or None)
    elif sys.argv[1] == "compare":
        import argparse

        ap = argparse.ArgumentParser()
        ap.add_argument("cmd")
        ap.add_argument("outdir")
        ap.add_argument("--workload", default="dna_small")
        ap.add_argument("--similarity", type=float, default=0.85)
        ap.add_argument("--word", type=int, default=5)
        ap.add_argument("--n-seqs", type=int, default=0)
        ap.add_argument("--timeout", type=int, default=1200)
        a = ap.parse_args()
        compare(a.outdir, a.workload, a.similarity, a.word, a.n_seqs, timeout=a.timeout)
