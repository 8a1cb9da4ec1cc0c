"""Generates the golden fixtures under tests/golden/.

Run here (where the reference tree exists):
    python tests/golden/make_golden.py fasta
writes the small FASTA fixtures and manifest.json with, per fixture, the md5
of the data.bin that the reference makeDB tool (built from its own source by
oracle/build_oracle.py into oracle/_ref/makeDB) produces.

The reference's clustering program only runs on a GPU; its outputs for every
(fixture, parameter set) of the manifest are produced on a GPU host by
oracle/ref_cluster.py and committed under tests/golden/ref/<fixture>/<tag>/
(cluster.txt, represent.fasta).  `python tests/golden/make_golden.py check`
re-verifies the checksums.

Fixtures of kind "q1" (tests/golden/q1_fixture.py) are too large to commit
as FASTA; their bytes come from a seeded generator and the manifest pins
their md5 (`fasta_md5`) beside the data.bin md5.  For them the reference's
outputs are committed as md5s (tests/golden/ref/<fixture>/<tag>/outputs.json).
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "ngia-metax_gb300"))
sys.path.insert(0, str(ROOT))

import ngia  # noqa: E402
from tests.golden import q1_fixture  # noqa: E402

# (name, type, generator args, edits, parameter sets [s, w, p])
FIXTURES = [
    ("dna_a", 0, dict(type=0, n_seqs=300, n_ancestors=6, len_a=500.0, len_b=60.0, len_min=300, len_max=700,
                      subst_max=0.2, indel_max=3, seed=101),
     "plain", [(0.85, 5, 0), (0.9, 8, 0), (0.95, 8, 0), (0.8, 5, 0), (0.99, 8, 0), (0.9, 6, 1)]),
    ("dna_noisy", 0, dict(type=0, n_seqs=260, n_ancestors=5, len_a=420.0, len_b=80.0, len_min=200, len_max=700,
                          subst_max=0.15, indel_max=3, seed=202),
     "noisy", [(0.85, 5, 0), (0.9, 7, 0), (0.7, 4, 0)]),
    ("prot_a", 1, dict(type=1, len_dist=1, n_seqs=240, n_ancestors=8, len_a=180.0, len_b=0.6, len_min=20,
                       len_max=1200, subst_max=0.5, indel_max=5, seed=303),
     "plain", [(0.9, 3, 0), (0.5, 2, 0), (0.7, 3, 0), (0.45, 3, 0)]),
    ("dna_q1", 0, None, "q1", q1_fixture.PARAMS),
]


def fixture_fasta(name: str, m: dict, workdir: Path) -> Path:
    """Path of a fixture's FASTA: the committed file, or for a generated
    fixture a fresh copy written into workdir and checked against its md5."""
    if m.get("generated") != "q1":
        return HERE / f"{name}.fasta"
    fa = Path(workdir) / f"{name}.fasta"
    facts = q1_fixture.write(fa)
    if facts["fasta_md5"] != m["fasta_md5"]:
        raise RuntimeError(f"{name}: generated FASTA md5 {facts['fasta_md5']} != manifest {m['fasta_md5']}")
    return fa


def _noisy(seqs: list[bytes], seed: int) -> list[bytes]:
    """Lower case runs, non-ACGT characters, records of net length < 16."""
    rng = np.random.default_rng(seed)
    out = []
    for s in seqs:
        b = bytearray(s)
        r = rng.random()
        if r < 0.3:
            for _ in range(int(rng.integers(1, 20))):
                b.insert(int(rng.integers(0, len(b) + 1)), b"NRYKM"[int(rng.integers(0, 5))])
        elif r < 0.45:
            a = int(rng.integers(0, len(b)))
            b[a:a + 60] = b[a:a + 60].lower()
        out.append(bytes(b))
    for k in range(12):
        core = bytes(b"ACGTU"[int(i)] for i in rng.integers(0, 5, int(rng.integers(0, 15))))
        out.insert(int(rng.integers(0, len(out))), b"N" * int(rng.integers(0, 400)) + core)
    return out


def _write_fasta(path: Path, seqs: list[bytes], crlf_every: int = 0) -> None:
    with open(path, "wb") as f:
        for i, s in enumerate(seqs):
            nl = b"\r\n" if crlf_every and i % crlf_every == 0 else b"\n"
            f.write(b">s%d desc%d" % (i, i % 7) + nl)
            for p in range(0, len(s), 61):
                f.write(s[p:p + 61] + nl)


def md5(path: Path) -> str:
    return hashlib.md5(path.read_bytes()).hexdigest()


def tag(s: float, w: int, p: int) -> str:
    return f"s{s}_w{w}_p{p}"


def make_fasta(only: list[str] | None = None) -> None:
    ref_makedb = ROOT / "oracle" / "_ref" / "makeDB"
    if not ref_makedb.exists():
        raise SystemExit("oracle/_ref/makeDB missing: run oracle/build_oracle.py where the reference tree exists")
    path = HERE / "manifest.json"
    manifest = json.loads(path.read_text()) if only and path.exists() else {}
    for name, typ, gen, kind, params in FIXTURES:
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            extra = {}
            if kind == "q1":
                fa = Path(td) / f"{name}.fasta"
                extra = {"generated": "q1", "fasta_md5": q1_fixture.write(fa)["fasta_md5"]}
            else:
                seq, off = ngia.synth(**gen)
                seqs = seq.all_bytes()
                if kind == "noisy":
                    seqs = _noisy(seqs, gen["seed"])
                fa = HERE / f"{name}.fasta"
                _write_fasta(fa, seqs, crlf_every=5 if kind == "noisy" else 0)
            out = Path(td) / "db"
            out.mkdir()
            subprocess.run([str(ref_makedb), "-i", str(fa), "-o", str(out), "-t", str(typ)], check=True,
                           capture_output=True)
            manifest[name] = {"type": typ, **extra, "data_bin_md5": md5(out / "data.bin"),
                              "params": [list(p) for p in params]}
    path.write_text(json.dumps(manifest, indent=1) + "\n")
    print("wrote", ", ".join(manifest))


def check() -> None:
    manifest = json.loads((HERE / "manifest.json").read_text())
    for name, m in manifest.items():
        with tempfile.TemporaryDirectory() as td:
            ngia.makedb(str(fixture_fasta(name, m, Path(td))), td, m["type"])
            assert md5(Path(td) / "data.bin") == m["data_bin_md5"], name
    print("ok")


if __name__ == "__main__":
    cmd = sys.argv[1] if len(sys.argv) > 1 else "check"
    if cmd == "fasta":
        make_fasta(sys.argv[2:] or None)
    else:
        check()
