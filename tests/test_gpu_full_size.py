"""GPU parity at the benchmark's full sizes: the first greedy iterations of
the 1,000,000-sequence DNA workload and of the 200,000-sequence protein
workload against the oracle's same iterations (bit for bit: assignment,
scores and stage counts), plus size-independent properties of the state
they leave (every assigned sequence points at a representative; the
representatives are the first unclustered sequences in order)."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle

pytestmark = pytest.mark.gpu

ITERS = 2


@pytest.mark.parametrize("workload,s,w", [("dna_1m", 0.85, 5), ("protein_200k", 0.9, 5)])
def test_first_iterations_match_oracle(cuda_device, workload, s, w):
    cfg = dict(ngia.CONFIGS[workload])
    seqs = ngia.synth(**cfg, seed=1)
    db = ngia.DB.pack(cfg["type"], seqs, seqs.off)
    seqs.close()
    p = ngia.params_clamp(cfg["type"], s, w, 0)
    with ngia.Context(db) as ctx:
        runs = []
        for mode in (ngia.MODE_GRAPH, ngia.MODE_PLAIN):
            ctx.begin(p, mode)
            ctx.step(ITERS)
            runs.append(ctx.end())
    ocl, oid, ost = oracle.cluster(db.words, db.rec_off, cfg["type"], p.similarity, p.word_length, p.precise,
                                   max_iters=ITERS)
    for cl, ident, st in runs:
        assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)
        assert st["iterations"] == ost["iterations"] == ITERS
        assert st["candidates"] == ost["candidates"] and st["base_pass"] == ost["base_pass"]
        assert st["members"] == ost["members"]
    cl = runs[0][0]
    reps = np.flatnonzero(cl == np.arange(db.n))
    assert len(reps) == ITERS
    assigned = cl >= 0
    assert np.isin(cl[assigned], reps).all()
    # each representative is the first sequence not taken by an earlier one
    for k, r in enumerate(reps):
        earlier = np.isin(cl, reps[:k])
        assert r == int(np.flatnonzero(~earlier)[0])
