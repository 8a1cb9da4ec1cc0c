"""The allocation-free scoring entry point (ngia_rep_scores_noalloc) against
the regular pair-score entry point.

Some callers cannot allocate device memory — their device memory belongs to
another allocator or pool, or their loop cannot afford cudaMalloc/cudaFree —
so they hand the library inputs and outputs that already live on the device.
This test plays such a caller: torch owns every device buffer, the library
only reads and writes them.  Scores must equal the oracle's banded-LCS score
of every pair and those of ngia_pair_scores (integer scores: exact), on two
calls in a row (the fixed working array keeps the previous call's contents,
which must not leak into the next).  A 60,000-residue representative makes
the rows so long that the array holds fewer rows than there are queries:
threads then take several queries each, the grid-stride path."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import noisy_db, seqs_to_db

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("db_type,s,w", [(0, 0.85, 5), (0, 0.95, 8), (1, 0.9, 3)])
def test_noalloc_scores_match_pair_scores(cuda_device, db_type, s, w):
    torch = pytest.importorskip("torch")
    db = noisy_db(db_type, 300, seed=91 + db_type, long_records=2)
    p = ngia.params_clamp(db_type, s, w, 0)
    words = torch.from_numpy(np.ascontiguousarray(db.words).view(np.int32)).cuda()
    with ngia.Context(db) as ctx:
        for rep in (0, 1, db.n // 2):
            cands = np.arange(db.n, dtype=np.int32)
            expect = ctx.pair_scores(p, rep, cands)[:, 2]
            ora = _oracle_scores(db, p, rep, cands)
            assert np.array_equal(expect, ora)
            offs = torch.from_numpy(db.rec_off[cands].astype(np.int64)).cuda()
            out = torch.full((db.n,), -7, dtype=torch.int32, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            for call in range(2):
                ngia.rep_scores_noalloc(words.data_ptr(), int(db.rec_off[rep]), offs.data_ptr(), db.n, db_type,
                                        p.similarity, out.data_ptr(), stream)
                torch.cuda.synchronize()
                got = out.cpu().numpy()
                bad = np.flatnonzero(got != expect)
                assert bad.size == 0, (call, rep, int(bad[0]), int(got[bad[0]]), int(expect[bad[0]]))
                out.fill_(-7)


def _oracle_scores(db, p, rep, cands):
    return np.array([oracle.pair(db.words, db.rec_off, db.type, p.similarity, p.word_length, rep, int(c))[2]
                     for c in cands], dtype=np.int32)


def _noalloc(torch, db, p, rep, n_calls=2):
    words = torch.from_numpy(np.ascontiguousarray(db.words).view(np.int32)).cuda()
    offs = torch.from_numpy(db.rec_off.astype(np.int64)).cuda()
    out = torch.full((db.n,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    res = []
    for call in range(n_calls):
        ngia.rep_scores_noalloc(words.data_ptr(), int(db.rec_off[rep]), offs.data_ptr(), db.n, db.type,
                                p.similarity, out.data_ptr(), stream)
        torch.cuda.synchronize()
        res.append(out.cpu().numpy().copy())
        out.fill_(-7)
    return res


def test_noalloc_long_representative_threads_take_several_queries(cuda_device):
    """60,000-residue representative: 1,875 words per row, so the 4 MiB
    array holds rows for 559 threads and the grid has 512 lanes for 2,500
    queries (each thread scores up to five of them, one after the other)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    rep = bytes(b"ACGT"[int(i)] for i in rng.integers(0, 4, 60000))
    seqs = [rep]
    for k in range(2500):
        L = int(rng.integers(40, 120))
        if k % 2:  # a mutated window of the representative: high scores
            a = int(rng.integers(0, len(rep) - L))
            b = bytearray(rep[a:a + L])
            for _ in range(int(rng.integers(0, 6))):
                b[int(rng.integers(0, L))] = b"ACGT"[int(rng.integers(0, 4))]
            seqs.append(bytes(b))
        else:
            seqs.append(bytes(b"ACGT"[int(i)] for i in rng.integers(0, 4, L)))
    db = seqs_to_db(0, seqs)
    assert db.read_len[0] == 60000 and db.n == 2501
    p = ngia.params_clamp(0, 0.8, 5, 0)
    got = _noalloc(torch, db, p, 0)
    cands = np.arange(db.n, dtype=np.int32)
    ora = _oracle_scores(db, p, 0, cands)
    for call, g in enumerate(got):
        bad = np.flatnonzero(g != ora)
        assert bad.size == 0, (call, int(bad[0]), int(g[bad[0]]), int(ora[bad[0]]))
    assert (ora[1:] >= 40).sum() > 1000  # the mutated windows score high


def test_noalloc_rejects_bad_arguments(cuda_device):
    with pytest.raises(ngia.NgiaError) as e:
        ngia.rep_scores_noalloc(0, 0, 0, 1, 0, 0.9, 0)
    assert e.value.code == -1
