"""CPU: the protein residue-code stream the loader builds for the short-word
test (k_codes in csrc/filter.cu) holds every w-mer of a record in 5w
contiguous bits, last residue lowest, so that one funnel shift of two stream
words reads it (codes_word).  This restates that layout and extraction and
checks the word counts they give against the oracle's short-word count
(func.cu:376-396: the rolling word over the candidate, counted from position
w-1 when the representative holds it), for whole blocks, ragged last blocks
and records of more than 32 blocks (the warp form's history hand-over)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests.helpers import family_db

M32 = 0xFFFFFFFF
HW = 30  # protein header words: length, net length, 28 residue counts


def _codes(words: np.ndarray, off: int) -> list[int]:
    """Residue codes of a record from its five bit planes (plane p = bit p)."""
    net = int(words[off + 1])
    pl = words[off + HW:]
    return [sum(((int(pl[5 * (q >> 5) + p]) >> (q & 31)) & 1) << p for p in range(5)) for q in range(net)]


def _stream(codes: list[int]) -> list[int]:
    """Five words per 32-residue block; residue j's code in bits 155-5j ..
    159-5j of the block's 160-bit value, word 0 its top 32 bits."""
    out = []
    for b in range((len(codes) + 31) // 32):
        v = 0
        for j in range(32):
            q = 32 * b + j
            v |= (codes[q] if q < len(codes) else 0) << (155 - 5 * j)
        out += [(v >> (32 * (4 - k))) & M32 for k in range(5)]
    return out


def _word(st: list[int], prev: int, j: int) -> int:
    """The 32 bits ending 5(j+1) bits below the top of the block (one funnel
    shift of two stream words, the previous block's last word above)."""
    e = 5 * (j + 1)
    k = (e - 1) >> 5
    hi = st[k - 1] if k else prev
    return (((hi << 32) | st[k]) >> (32 * (k + 1) - e)) & M32


def _count(cand: list[int], present: set[int], w: int, warp: bool) -> int:
    """Short-word count from the stream: every position with a zero history
    before the record, minus the first w-1 positions (as the kernels do);
    warp=True hands the history over in rounds of 32 blocks."""
    mask = (1 << (5 * w)) - 1
    s = _stream(cand)
    n = len(cand)
    nb = (n + 31) // 32
    tot = 0
    prev = 0
    step = 32 if warp else 1
    for b0 in range(0, nb, step):
        lasts = [s[5 * b + 4] for b in range(b0, min(nb, b0 + step))]
        for i, b in enumerate(range(b0, min(nb, b0 + step))):
            p = prev if i == 0 else lasts[i - 1]
            st = s[5 * b:5 * b + 5]
            tot += sum((_word(st, p, j) & mask) in present for j in range(min(32, n - 32 * b)))
        prev = lasts[-1]
    head = min(w - 1, n)
    tot -= sum((_word(s[0:5], 0, j) & mask) in present for j in range(head))
    return tot


def _rep_words(rep: list[int], w: int) -> set[int]:
    mask = (1 << (5 * w)) - 1
    word, out = 0, set()
    for q, c in enumerate(rep):
        word = ((word << 5) | c) & mask
        if q >= w - 1:
            out.add(word)
    return out


@pytest.mark.parametrize("w", [2, 3])
def test_code_stream_word_count_matches_oracle(w):
    db = family_db(1, n=60, anc=3, seed=71, len_a=900.0, len_b=0.8, len_min=20, len_max=3000, subst_max=0.2)
    words, off = db.words, db.rec_off
    s = 0.7 if w == 2 else 0.9
    checked = 0
    lengths = set()
    for rep in range(0, 6):
        rc = _codes(words, int(off[rep]))
        present = _rep_words(rc, w)
        for cand in range(rep + 1, db.n, 3):
            o = oracle.pair(words, off, 1, s, w, rep, cand)
            if o[1] < 0:  # composition test failed: the oracle counts no words
                continue
            cc = _codes(words, int(off[cand]))
            got = _count(cc, present, w, warp=False)
            assert got == o[1], (rep, cand, len(cc))
            if len(cc) > 32 * 32:
                assert _count(cc, present, w, warp=True) == o[1]
            lengths.add(len(cc))
            checked += 1
    assert checked >= 20
    assert any(n % 32 for n in lengths) and max(lengths) > 32 * 32
