"""GPU: the pooled batch form (NGIA_MODE_POOL).  The jobs of one record type
share every launch of a round: one filter over all their unclustered
sequences, and per length bucket one alignment launch whose CTAs take chunks
of pairs from any job.  Each job must still get exactly the oracle's
clustering: jobs of very different sizes and lengths, records longer than
2,048 residues (the filter's warp-wide short-word count) and wider than 128
blocks (the global-ring bucket), both test orders, and a job with records of
net length < 16 that keeps its own loop while precise is 0 and joins the pool
when precise is 1."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db, noisy_db

pytestmark = pytest.mark.gpu


def _check(dbs, params, cls, ids, st, max_iters=0):
    iters = 0
    for k, (db, p, cl, ident) in enumerate(zip(dbs, params, cls, ids)):
        ocl, oid, ost = oracle.cluster(db.words, db.rec_off, db.type, p.similarity, p.word_length, p.precise,
                                       max_iters=max_iters)
        assert np.array_equal(cl, ocl), f"job {k}: assignment differs"
        assert np.array_equal(ident, oid), f"job {k}: scores differ"
        iters += ost["iterations"]
    assert st["iterations"] == iters


def _mixed():
    specs = [  # type, kind, n, ancestors, s, w
        (0, "fam", 900, 12, 0.85, 5), (0, "fam", 40, 2, 0.9, 5), (0, "long", 160, 0, 0.85, 5),
        (0, "fam", 500, 10, 0.95, 5), (0, "short", 300, 0, 0.9, 5), (1, "fam", 400, 10, 0.9, 3),
        (1, "fam", 70, 3, 0.5, 2), (0, "fam", 1, 1, 0.85, 5), (1, "long", 120, 0, 0.9, 3),
        (0, "fam", 2000, 30, 0.8, 4), (1, "fam", 250, 6, 0.95, 3), (0, "fam", 333, 5, 0.99, 6),
        (0, "long", 100, 0, 0.95, 5),
    ]
    dbs, params = [], []
    for k, (t, kind, n, anc, s, w) in enumerate(specs):
        seed = 900 + k
        if kind == "fam":
            db = family_db(t, n=n, anc=anc, seed=seed)
        elif kind == "long":
            db = noisy_db(t, n, seed=seed, long_records=8)
        else:
            db = noisy_db(t, n, seed=seed, short_records=7)
        dbs.append(db)
        params.append(ngia.params_clamp(t, s, w, 0))
    return dbs, params


def test_pool_matches_oracle_on_mixed_jobs(cuda_device):
    dbs, params = _mixed()
    with ngia.Batch(dbs) as b:
        cls, ids, st = b.run(params, ngia.MODE_POOL)
        _check(dbs, params, cls, ids, st)
        # a second run reuses the captured graph
        cls, ids, st = b.run(params, ngia.MODE_POOL)
        _check(dbs, params, cls, ids, st)


def test_pool_rebuilds_when_a_job_changes_its_loop(cuda_device):
    dbs, params = _mixed()
    with ngia.Batch(dbs) as b:
        cls, ids, st = b.run(params, ngia.MODE_POOL)
        _check(dbs, params, cls, ids, st)
        # precise 1: the job with short records joins its pool; other similarities
        params2 = [ngia.params_clamp(db.type, 0.9 if db.type == 0 else 0.5, 5 if db.type == 0 else 2, 1)
                   for db in dbs]
        cls, ids, st = b.run(params2, ngia.MODE_POOL)
        _check(dbs, params2, cls, ids, st)


def test_pool_sampled_iterations(cuda_device):
    dbs, params = _mixed()
    with ngia.Batch(dbs) as b:
        cls, ids, st = b.run(params, ngia.MODE_POOL, max_iters=7)
    _check(dbs, params, cls, ids, st, max_iters=7)


def test_speculative_batch_matches_oracle_on_mixed_jobs(cuda_device, monkeypatch):
    """The speculative batch form on the same jobs, with fewer worker threads
    than jobs (each worker clusters several jobs in turn)."""
    monkeypatch.setenv("NGIA_BATCH_WORKERS", "3")
    dbs, params = _mixed()
    with ngia.Batch(dbs) as b:
        cls, ids, st = b.run(params, ngia.MODE_SPEC)
    _check(dbs, params, cls, ids, st)
