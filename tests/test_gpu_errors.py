"""The device-side error path, made to run without faulting the GPU.

Every staging wait of the alignment kernels is bounded: when it gives up,
the kernel records an error in the run state, lets its copy land and
returns; the iteration's later kernels see the error and do nothing, and the
host returns NGIA_E_DEVICE.  NGIA_WAIT_POLLS=0 (read at ngia_cluster_begin)
sets that poll limit to zero, so every such wait gives up at once.  The same
context must then cluster correctly once the variable is gone."""
from __future__ import annotations

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db

pytestmark = pytest.mark.gpu

NGIA_E_DEVICE = -6


@pytest.mark.parametrize("mode", [ngia.MODE_PLAIN, ngia.MODE_GRAPH])
def test_expired_wait_returns_device_error_and_context_recovers(cuda_device, monkeypatch, mode):
    db = family_db(0, n=300, anc=6, seed=41)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    ocl, oid, _ = oracle.cluster(db.words, db.rec_off, 0, p.similarity, p.word_length, p.precise)
    with ngia.Context(db) as ctx:
        monkeypatch.setenv("NGIA_WAIT_POLLS", "0")
        with pytest.raises(ngia.NgiaError) as e:
            ctx.cluster(p, mode)
        assert e.value.code == NGIA_E_DEVICE
        assert "device error 1" in str(e.value)  # the mbarrier-timeout code
        monkeypatch.delenv("NGIA_WAIT_POLLS")
        cl, ident, st = ctx.cluster(p, mode)
        assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)
        # and once more with the short limit, then normal again: no state leaks
        monkeypatch.setenv("NGIA_WAIT_POLLS", "0")
        with pytest.raises(ngia.NgiaError):
            ctx.cluster(p, mode)
        monkeypatch.delenv("NGIA_WAIT_POLLS")
        cl, ident, _ = ctx.cluster(p, mode)
        assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)
