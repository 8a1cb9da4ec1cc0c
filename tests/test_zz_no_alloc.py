"""The allocation-free scoring entry point (ngia_rep_scores_noalloc) against
the regular pair-score entry point.

Some callers cannot allocate device memory — their device memory belongs to
another allocator or pool, or their loop cannot afford cudaMalloc/cudaFree —
so they hand the library inputs and outputs that already live on the device.
This test plays such a caller: torch owns every device buffer, the library
only reads and writes them.  Scores must equal those of ngia_pair_scores
(integer scores: exact), on two calls in a row (the fixed working array keeps
the previous call's contents, which must not leak into the next)."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from tests.helpers import noisy_db

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


def test_noalloc_rejects_bad_arguments(cuda_device):
    with pytest.raises(ngia.NgiaError) as e:
        ngia.rep_scores_noalloc(0, 0, 0, 1, 0, 0.9, 0)
    assert e.value.code == -1
