"""Shared test inputs: seeded synthetic databases, including crafted edge
records (non-alphabet characters, net length < 16, very long records)."""
from __future__ import annotations

import numpy as np

import ngia


def seqs_to_db(db_type: int, seqs: list[bytes]) -> "ngia.DB":
    off = np.zeros(len(seqs) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    return ngia.DB.pack(db_type, b"".join(seqs), off)


def split(seq, off: np.ndarray) -> list[bytes]:
    if isinstance(seq, ngia.Seqs):
        return seq.all_bytes()
    return [bytes(seq[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def family_db(db_type: int = 0, n: int = 400, anc: int = 8, seed: int = 1, **kw) -> "ngia.DB":
    if db_type == 0:
        args = dict(type=0, n_seqs=n, n_ancestors=anc, len_a=600.0, len_b=80.0, len_min=300, len_max=900,
                    subst_max=0.2, indel_max=3, seed=seed)
    else:
        args = dict(type=1, len_dist=1, n_seqs=n, n_ancestors=anc, len_a=200.0, len_b=0.5, len_min=20,
                    len_max=1500, subst_max=0.5, indel_max=5, seed=seed)
    args.update(kw)
    seq, off = ngia.synth(**args)
    return ngia.DB.pack(db_type, seq, off)


def noisy_db(db_type: int, n: int, seed: int, short_records: int = 0, long_records: int = 0) -> "ngia.DB":
    """Family sequences with scattered non-alphabet characters (net < raw),
    plus optional records of net length < 16 and records longer than 4096."""
    rng = np.random.default_rng(seed)
    seq, off = ngia.synth(**(dict(type=0, n_seqs=n, n_ancestors=max(2, n // 40), len_a=600.0, len_b=80.0,
                                  len_min=300, len_max=900, seed=seed) if db_type == 0 else
                             dict(type=1, len_dist=1, n_seqs=n, n_ancestors=max(2, n // 40), len_a=200.0,
                                  len_b=0.5, len_min=20, len_max=1500, subst_max=0.5, indel_max=5, seed=seed)))
    out = []
    junk = b"NNRYX" if db_type == 0 else b"#@1"
    for s in split(seq, off):
        b = bytearray(s)
        if rng.random() < 0.5:
            for _ in range(int(rng.integers(1, 12))):
                b.insert(int(rng.integers(0, len(b) + 1)), junk[int(rng.integers(0, len(junk)))])
        if rng.random() < 0.2:
            b = b.lower() if rng.random() < 0.5 else b
        out.append(bytes(b))
    alpha = b"ACGT" if db_type == 0 else b"ACDEFGHIKLMNPQRSTVWY"
    for k in range(short_records):
        L = int(rng.integers(0, 15))
        core = bytes(alpha[int(i)] for i in rng.integers(0, len(alpha), L))
        pad = b"N" * int(rng.integers(0, 700)) if db_type == 0 else b"#" * int(rng.integers(0, 700))
        out.insert(int(rng.integers(0, len(out) + 1)), pad + core)
    for k in range(long_records):
        L = int(rng.integers(4200, 6000))
        out.append(bytes(alpha[int(i)] for i in rng.integers(0, len(alpha), L)))
    return seqs_to_db(db_type, out)
