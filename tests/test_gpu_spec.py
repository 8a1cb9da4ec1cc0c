"""GPU: the speculative-round driver (NGIA_MODE_SPEC) — the next K
unclustered sequences as candidate representatives of one round, every pair
against them at once, the greedy order replayed on the device — against the
oracle's one-representative loop.  Bit-exact: representatives, memberships,
per-member scores, the number of representatives and of accepted pairs."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db, noisy_db

pytestmark = pytest.mark.gpu


def _check_spec(db, p):
    ocl, oid, ost = oracle.cluster(db.words, db.rec_off, db.type, p.similarity, p.word_length, p.precise)
    with ngia.Context(db) as ctx:
        cl, ident, st = ctx.cluster(p, ngia.MODE_SPEC)
    bad = np.flatnonzero((cl != ocl) | (ident != oid))
    assert bad.size == 0, (f"seq {bad[0]}: gpu ({cl[bad[0]]}, {ident[bad[0]]}) "
                           f"oracle ({ocl[bad[0]]}, {oid[bad[0]]})")
    assert st["iterations"] == ost["iterations"]
    assert st["members"] == ost["members"]
    return st


@pytest.mark.parametrize("s", [0.8, 0.85, 0.9, 0.95])
def test_spec_dna(cuda_device, s):
    _check_spec(family_db(0, n=500, anc=10, seed=int(s * 100)), ngia.params_clamp(0, s, 5, 0))


def test_spec_dna_noisy(cuda_device):
    _check_spec(noisy_db(0, 600, seed=9, long_records=2), ngia.params_clamp(0, 0.85, 5, 0))


def test_spec_dna_precise(cuda_device):
    _check_spec(family_db(0, n=400, anc=8, seed=21), ngia.params_clamp(0, 0.9, 6, 1))


@pytest.mark.parametrize("s,w", [(0.5, 2), (0.9, 3)])
def test_spec_protein(cuda_device, s, w):
    _check_spec(family_db(1, n=400, anc=10, seed=31), ngia.params_clamp(1, s, w, 0))


@pytest.mark.parametrize("db_type,s,w", [(0, 0.95, 5), (1, 0.9, 3)])
def test_spec_long_records_word_first(cuda_device, db_type, s, w):
    """Short-word test in the round filter (word-first order), records both
    sides of 2,048 residues and windows past the shared-memory rings."""
    if db_type == 0:
        db = family_db(0, n=160, anc=6, seed=61, len_a=2100.0, len_b=500.0, len_min=1200, len_max=6000,
                       subst_max=0.05)
    else:
        db = family_db(1, n=160, anc=6, seed=62, len_a=2000.0, len_b=0.6, len_min=200, len_max=9000,
                       subst_max=0.15)
    _check_spec(db, ngia.params_clamp(db_type, s, w, 0))


@pytest.mark.parametrize("precise", [0, 1])
def test_spec_short_records(cuda_device, precise):
    """Records of net length < 16 skip the short-word test.  Up to 16,384
    sequences (one job per thread of the reference's word kernel) that is a
    rule of the pair and the rounds run; beyond, a pair's test depends on its
    iteration's job list and the driver runs the plain loop (precise mode:
    no short-word test, rounds at any size)."""
    db = noisy_db(0, 500, seed=12, short_records=25)
    assert (db.words[db.rec_off + 1] < 16).any()
    _check_spec(db, ngia.params_clamp(0, 0.88, 7, precise))


@pytest.mark.parametrize("budget", ["1", "40", "300"])
def test_spec_plain_iterations_then_rounds(cuda_device, monkeypatch, budget):
    """Above the round budget the driver runs plain iterations, then rounds
    of K = budget / unclustered candidates."""
    monkeypatch.setenv("NGIA_SPEC_BUDGET", budget)
    _check_spec(family_db(0, n=400, anc=8, seed=71), ngia.params_clamp(0, 0.85, 5, 0))


def test_spec_stepwise_and_checkpoint(cuda_device, tmp_path):
    """Steps of at most 7 representatives; a run saved between rounds and
    resumed in another context, by the rounds or by the plain loop, ends as
    the uninterrupted run."""
    db = family_db(0, n=400, anc=8, seed=55)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    ck = tmp_path / "spec.ckpt"
    with ngia.Context(db) as ctx:
        full = ctx.cluster(p, ngia.MODE_GRAPH)
        ctx.begin(p, ngia.MODE_SPEC)
        last = 0
        for step in range(1000):
            done = ctx.step(7)
            it = ctx.stats()["iterations"]
            assert 0 < it - last <= 7 or done
            last = it
            if step == 3:
                ctx.save(ck)
            if done:
                break
        cl, ident, st = ctx.end()
        assert np.array_equal(cl, full[0]) and np.array_equal(ident, full[1])
        assert st["iterations"] == full[2]["iterations"]
    for mode in (ngia.MODE_SPEC, ngia.MODE_PLAIN):
        with ngia.Context(db) as ctx:
            ctx.resume(ck, mode)
            while not ctx.step(50):
                pass
            cl, ident, st = ctx.end()
        assert np.array_equal(cl, full[0]) and np.array_equal(ident, full[1])
        assert st["iterations"] == full[2]["iterations"]
