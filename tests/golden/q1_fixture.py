"""The `dna_q1` golden fixture: a database on which the reference's
short-word kernel returns whole threads while its job list is longer than the
kernel's 16,384 threads (CUDA/signalNode/src/func.cu:375 and the grid of
func.h:8-9, <<<128,128>>> with a grid-stride loop).

Thread t of that kernel tests the jobs at list positions t, t+16384, ...; at
its first job of net length < 16 it leaves the kernel, so every later job of
that thread passes the short-word test untested and goes on to the alignment.
The fixture is built so that this changes the clustering:

* record R (25 residues, composition A7 C6 G6 T6) sorts first and is the
  first representative;
* every other record has raw length 16 and a composition inside R's, so all
  of them pass the composition test against R and the job list of the first
  iteration is R followed by the 16-residue records in FASTA order;
* 40 "short" records (15 bases and one N: net length 15) sit at list
  positions p in [1, 3600);
* at each position p + 16384 sits a record D made from R by deleting 9
  residues: D is a subsequence of R (banded LCS 16 >= ceil(16 * 0.9)), but
  fewer of its words occur in R than the short-word test needs (w = 5 and
  w = 4 at s = 0.9), so it joins R only because its thread left the kernel;
* 40 more such D records sit at other positions, where the test runs and
  rejects them;
* the rest are 400 families of 16-mers (a seed and copies with at most one
  substitution).

The records are produced by a 64-bit splitmix generator in plain Python, so
the FASTA bytes are the same on every machine; `manifest.json` holds their
md5 and that of the data.bin the reference makeDB writes for them.
"""
from __future__ import annotations

import hashlib

M64 = (1 << 64) - 1
N16 = 20000           # records of raw length 16
REF_THREADS = 16384   # BLOCK * WARP of the reference launches
N_SHORT = 40
N_CONTROL = 40
N_FAMILIES = 400
REP_COUNTS = {"A": 7, "C": 6, "G": 6, "T": 6}
PARAMS = [(0.9, 5, 0), (0.9, 4, 0)]


class _Rng:
    def __init__(self, seed: int):
        self.x = seed & M64

    def next(self) -> int:
        self.x = (self.x + 0x9E3779B97F4A7C15) & M64
        z = self.x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def below(self, n: int) -> int:
        return self.next() % n

    def shuffle(self, xs: list) -> None:
        for i in range(len(xs) - 1, 0, -1):
            j = self.below(i + 1)
            xs[i], xs[j] = xs[j], xs[i]


def _fits(s: bytes) -> bool:
    """Composition inside R's: the composition test against R passes."""
    return all(s.count(c.encode()) <= k for c, k in REP_COUNTS.items())


def _words(s: bytes, w: int) -> list[bytes]:
    return [s[i:i + w] for i in range(len(s) - w + 1)]


def word_count(rep: bytes, cand: bytes, w: int) -> int:
    """The reference's short-word count for an all-ACGT pair: occurrences of
    the candidate's w-mers (from position w-1 on) in the representative's
    w-mer set."""
    present = set(_words(rep, w))
    return sum(1 for x in _words(cand, w) if x in present)


def word_min(length: int, s: float, w: int) -> int:
    """(len - w + 1) - ceil(len * (1 - s)) * w with the reference's float
    arithmetic (func.cu:393-396)."""
    import numpy as np

    one_minus = np.float32(1.0) - np.float32(s)
    return (length - w + 1) - int(np.ceil(np.float32(length) * one_minus)) * w


def _random16(rng: _Rng) -> bytes:
    while True:
        s = bytes(b"ACGT"[rng.below(4)] for _ in range(16))
        if _fits(s):
            return s


def _derived(rng: _Rng, rep: bytes) -> bytes:
    """R with 9 residues deleted, rejected by the short-word test at every
    parameter set of PARAMS."""
    while True:
        idx = list(range(len(rep)))
        rng.shuffle(idx)
        d = bytes(rep[i] for i in sorted(idx[:16]))
        if all(word_count(rep, d, w) < word_min(16, s, w) for s, w, _ in PARAMS):
            return d


def records() -> tuple[list[bytes], dict]:
    """(sequences in FASTA order, layout facts for the tests)."""
    rng = _Rng(0x51F0_2024)
    pool = list(b"A" * 7 + b"C" * 6 + b"G" * 6 + b"T" * 6)
    rng.shuffle(pool)
    rep = bytes(pool)

    seeds = [_random16(rng) for _ in range(N_FAMILIES)]
    body: list[bytes] = []
    while len(body) < N16:
        s = bytearray(seeds[rng.below(N_FAMILIES)])
        if rng.below(2):
            s[rng.below(16)] = b"ACGT"[rng.below(4)]
        if _fits(bytes(s)):
            body.append(bytes(s))

    # list positions (1-based: position 0 is R) of the short records
    short_pos = sorted(set(1 + rng.below(3599) for _ in range(N_SHORT * 2)))[:N_SHORT]
    while len(short_pos) < N_SHORT:
        short_pos = sorted(set(short_pos + [1 + rng.below(3599)]))[:N_SHORT]
    skipped_pos = [p + REF_THREADS for p in short_pos]
    taken = set(short_pos) | set(skipped_pos)
    control_pos: list[int] = []
    while len(control_pos) < N_CONTROL:
        p = 1 + rng.below(N16)
        if p not in taken:
            taken.add(p)
            control_pos.append(p)
    control_pos.sort()

    for k, p in enumerate(short_pos):
        if k % 2 == 0:  # a 15-residue subsequence of R: joins R by the alignment
            idx = list(range(len(rep)))
            rng.shuffle(idx)
            core = bytes(rep[i] for i in sorted(idx[:15]))
        else:
            while True:
                core = bytes(b"ACGT"[rng.below(4)] for _ in range(15))
                if _fits(core):
                    break
        at = rng.below(16)
        body[p - 1] = core[:at] + b"N" + core[at:]
    for p in skipped_pos + control_pos:
        body[p - 1] = _derived(rng, rep)

    seqs = body[:N16 // 2] + [rep] + body[N16 // 2:]
    facts = {"rep_fasta_index": N16 // 2, "short_pos": short_pos, "skipped_pos": skipped_pos,
             "control_pos": control_pos}
    return seqs, facts


def fasta_bytes(seqs: list[bytes]) -> bytes:
    out = bytearray()
    for i, s in enumerate(seqs):
        out += b">q%d\n" % i + s + b"\n"
    return bytes(out)


def write(path) -> dict:
    seqs, facts = records()
    data = fasta_bytes(seqs)
    with open(path, "wb") as f:
        f.write(data)
    facts["fasta_md5"] = hashlib.md5(data).hexdigest()
    return facts

