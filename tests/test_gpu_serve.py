"""GPU: the serving path (ngia_serve_*) — batches assigned to a resident
representative set, leftovers clustered among themselves — against the
oracle's replay of the same batches (ora_assign), and every batch's result
identical alone and in a mix of batches running side by side."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import seqs_to_db, split

pytestmark = pytest.mark.gpu

GEN = {
    0: dict(type=0, len_a=600.0, len_b=80.0, len_min=300, len_max=900, subst_max=0.2, indel_max=3),
    1: dict(type=1, len_dist=1, len_a=200.0, len_b=0.5, len_min=20, len_max=1500, subst_max=0.5, indel_max=5),
}


def _workload(db_type: int, s: float, w: int, n_res: int, anc: int, sizes: list[int], seed: int):
    """Resident representatives (the clustering of n_res sequences, in
    creation order) and query batches drawn from the same ancestors beyond
    them, 10% of them from novel ancestors."""
    p = ngia.params_clamp(db_type, s, w, 0)
    total = n_res + sum(sizes)
    seq, off = ngia.synth(**GEN[db_type], n_seqs=total, n_ancestors=anc, novel_frac=0.1, seed=seed)
    seqs = split(seq, off)
    res_seq, res_off = ngia.synth(**GEN[db_type], n_seqs=n_res, n_ancestors=anc, seed=seed)
    res_db = ngia.DB.pack(db_type, res_seq, res_off)
    cl, _, _ = oracle.cluster(res_db.words, res_db.rec_off, db_type, p.similarity, p.word_length, p.precise)
    reps = ngia.Records.subset(res_db, np.flatnonzero(cl == np.arange(res_db.n)))
    batches, k = [], n_res
    for m in sizes:
        batches.append(seqs_to_db(db_type, seqs[k:k + m]))
        k += m
    return p, reps, batches


def _expected(p, reps, b):
    return oracle.assign(reps.words, reps.rec_off, b.words, b.rec_off, b.type, p.similarity, p.word_length,
                         p.precise)


@pytest.mark.parametrize("db_type,s,w", [(0, 0.9, 5), (0, 0.95, 5), (1, 0.9, 3)])
def test_serve_matches_oracle_alone_and_mixed(cuda_device, db_type, s, w):
    sizes = [1, 7, 64, 250, 33, 400, 2, 120, 17, 90]
    p, reps, batches = _workload(db_type, s, w, 500 if db_type == 0 else 400, 10, sizes, seed=81 + db_type)
    exp = [_expected(p, reps, b) for b in batches]
    assert sum(int((e[0] >= 0).sum()) for e in exp) > 50  # queries do join resident representatives
    with ngia.Server(reps, p, slots=4, max_batch=512) as srv:
        assert srv.slots == 4
        # the mix: everything submitted at once, batches run side by side
        tickets = [srv.submit(b) for b in batches]
        mixed = [srv.wait(t) for t in tickets]
        # alone: one batch at a time
        alone = [srv.wait(srv.submit(b)) for b in batches]
    for b, e, m, a in zip(batches, exp, mixed, alone):
        assert np.array_equal(m[0], e[0]) and np.array_equal(m[1], e[1]), f"batch of {b.n}: mixed != oracle"
        assert np.array_equal(a[0], m[0]) and np.array_equal(a[1], m[1]), f"batch of {b.n}: alone != mixed"
        info = m[2]
        assert info["done"] == 1 and info["resident"] == int((e[0] >= 0).sum()) and info["new_reps"] == e[2]
    assert len({m[2]["slot"] for m in mixed}) > 1  # the mix did use several slots


def test_serve_poll_and_errors(cuda_device):
    p, reps, batches = _workload(0, 0.9, 5, 300, 6, [40, 5], seed=91)
    with ngia.Server(reps, p, slots=2, max_batch=64) as srv:
        t = srv.submit(batches[0])
        got = None
        for _ in range(10000):
            got = srv.poll(t, wait_ms=5)
            if got is not None:
                break
        assert got is not None
        e = _expected(p, reps, batches[0])
        assert np.array_equal(got[0], e[0]) and np.array_equal(got[1], e[1])
        with pytest.raises(ngia.NgiaError) as ex:  # a released ticket
            srv.poll(t)
        assert ex.value.code == -1
        big = _workload(0, 0.9, 5, 10, 6, [80], seed=92)[2][0]
        with pytest.raises(ngia.NgiaError) as ex:  # more records than a slot holds
            srv.submit(big)
        assert ex.value.code == -8
        prot = _workload(1, 0.9, 3, 10, 3, [5], seed=93)[2][0]
        with pytest.raises(ngia.NgiaError) as ex:  # another sequence type
            srv.submit(prot)
        assert ex.value.code == -1
        assert srv.wait(srv.submit(batches[1]))[2]["done"] == 1
