"""Measurement entry points: the composition filter's floor (an empty launch
and a read-only pass with the filter's grid) leaves the run untouched."""
from __future__ import annotations

import math

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db

pytestmark = pytest.mark.gpu


def test_filter_floor_is_positive_and_leaves_the_run_unchanged(cuda_device):
    db = family_db(0, n=3000, anc=30, seed=43)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    ocl, oid, _ = oracle.cluster(db.words, db.rec_off, 0, p.similarity, p.word_length, p.precise)
    with ngia.Context(db) as ctx:
        ctx.begin(p, ngia.MODE_PLAIN)
        ctx.step(3)
        launch_us, read_us = ctx.filter_floor()
        assert math.isfinite(launch_us) and math.isfinite(read_us)
        assert 0.0 < launch_us < 1e4 and 0.0 < read_us < 1e4
        ctx.step(0)
        cl, ident, _ = ctx.end()
    assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)


def test_filter_floor_needs_a_begun_dna_context(cuda_device):
    db = family_db(1, n=200, anc=5, seed=44)
    with ngia.Context(db) as ctx:
        with pytest.raises(ngia.NgiaError):
            ctx.filter_floor()  # not begun
        ctx.begin(ngia.params_clamp(1, 0.9, 5, 0), ngia.MODE_PLAIN)
        with pytest.raises(ngia.NgiaError):
            ctx.filter_floor()  # protein
