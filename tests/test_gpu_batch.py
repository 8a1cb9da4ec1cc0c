"""GPU: a batch of independent jobs (mixed DNA / protein, sizes and
similarities) clustered in one CUDA graph launch (a loop per job, or the
pooled rounds shared by the jobs of a record type), with every job's
speculative driver on host worker threads, and one after the other with the
plain driver, gives every job exactly the oracle's clustering."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db, noisy_db

pytestmark = pytest.mark.gpu


def _jobs():
    specs = [(0, 300, 6, 0.8, 5), (1, 200, 6, 0.9, 3), (0, 120, 3, 0.95, 8), (0, 450, 9, 0.9, 6),
             (1, 260, 8, 0.5, 2), (0, 60, 2, 0.85, 5)]
    dbs, params = [], []
    for k, (t, n, anc, s, w) in enumerate(specs):
        dbs.append(family_db(t, n=n, anc=anc, seed=500 + k) if k != 3 else noisy_db(0, n, seed=503,
                                                                                    short_records=6))
        params.append(ngia.params_clamp(t, s, w, 0))
    return dbs, params


@pytest.mark.parametrize("mode", [ngia.MODE_GRAPH, ngia.MODE_POOL, ngia.MODE_SPEC, ngia.MODE_PLAIN])
def test_batch_matches_oracle_per_job(cuda_device, mode):
    dbs, params = _jobs()
    with ngia.Batch(dbs) as b:
        cls, ids, st = b.run(params, mode)
    iters = 0
    for db, p, cl, ident in zip(dbs, params, cls, ids):
        ocl, oid, ost = oracle.cluster(db.words, db.rec_off, db.type, p.similarity, p.word_length, p.precise)
        assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)
        iters += ost["iterations"]
    assert st["iterations"] == iters


def test_batch_sampled_iterations_agree(cuda_device):
    dbs, params = _jobs()
    with ngia.Batch(dbs) as b:
        g = b.run(params, ngia.MODE_GRAPH, max_iters=5)
        q = b.run(params, ngia.MODE_POOL, max_iters=5)
        r = b.run(params, ngia.MODE_SPEC, max_iters=5)
        p = b.run(params, ngia.MODE_PLAIN, max_iters=5)
    for a, c, d, e in zip(g[0], p[0], q[0], r[0]):
        assert np.array_equal(a, c) and np.array_equal(a, d) and np.array_equal(a, e)
    assert g[2]["iterations"] == p[2]["iterations"] == q[2]["iterations"] == r[2]["iterations"] == 5 * len(dbs)


def test_batch_autotune_keeps_results(cuda_device):
    """The batch policy tuner (thread per pair, each job's default cut-off,
    each job's own per-bucket tuning), then the one-loop-per-job form under
    every policy: still the oracle's clustering per job."""
    dbs, params = _jobs()
    want = [oracle.cluster(db.words, db.rec_off, db.type, p.similarity, p.word_length, p.precise)[:2]
            for db, p in zip(dbs, params)]
    with ngia.Batch(dbs) as b:
        assert b.policy() == -1
        with pytest.raises(ngia.NgiaError):
            b.set_policy(ngia.POLICY_TUNED)  # needs the jobs' own tuning first
        tun = b.autotune(params, 2)
        assert len(tun) == len(dbs) and all(t["refill"] >= 1 and t["candidates"] == 3 for t in tun)
        chosen = b.policy()
        assert chosen in (ngia.POLICY_THREAD, ngia.POLICY_CUTOFF, ngia.POLICY_TUNED)
        for pol in (chosen, ngia.POLICY_THREAD, ngia.POLICY_CUTOFF, ngia.POLICY_TUNED):
            b.set_policy(pol)
            assert b.policy() == pol
            cls, ids, st = b.run(params, ngia.MODE_GRAPH)
            for (ocl, oid), cl, ident in zip(want, cls, ids):
                assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)
