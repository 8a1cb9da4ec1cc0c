"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on
the same seeded inputs.  Integer work, so the bar is bit-exact: composition
sums, short-word counts, band widths, banded-LCS scores, representatives,
memberships and per-member scores must all be identical."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import ngia
from oracle import oracle
from tests.helpers import family_db, noisy_db, seqs_to_db

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _oracle_pairs(db, p, rep, cands):
    return np.array([oracle.pair(db.words, db.rec_off, db.type, p.similarity, p.word_length, rep, int(c))[:4]
                     for c in cands], dtype=np.int32)


def _check_pairs(db, p, reps, rng, k=300):
    with ngia.Context(db) as ctx:
        for rep in reps:
            cands = rng.choice(db.n, size=min(k, db.n), replace=False).astype(np.int32)
            got = ctx.pair_scores(p, rep, cands)
            exp = _oracle_pairs(db, p, rep, cands)
            bad = np.flatnonzero((got != exp).any(axis=1))
            assert bad.size == 0, (f"rep {rep} cand {cands[bad[0]]}: gpu {got[bad[0]].tolist()} "
                                   f"oracle {exp[bad[0]].tolist()}")


def _check_cluster(db, p, modes=(ngia.MODE_PLAIN, ngia.MODE_GRAPH)):
    ocl, oid, ost = oracle.cluster(db.words, db.rec_off, db.type, p.similarity, p.word_length, p.precise)
    with ngia.Context(db) as ctx:
        for mode in modes:
            cl, ident, st = ctx.cluster(p, mode)
            bad = np.flatnonzero((cl != ocl) | (ident != oid))
            assert bad.size == 0, (f"mode {mode} seq {bad[0]}: gpu ({cl[bad[0]]}, {ident[bad[0]]}) "
                                   f"oracle ({ocl[bad[0]]}, {oid[bad[0]]})")
            assert st["iterations"] == ost["iterations"]
            if mode != ngia.MODE_SPEC:  # speculative rounds count their pairs apart
                assert st["candidates"] == ost["candidates"]
                assert st["base_pass"] == ost["base_pass"]
                assert st["members"] == ost["members"]
    return ost


@pytest.mark.parametrize("s", [0.5, 0.8, 0.85, 0.9, 0.95, 1.0])
def test_pair_scores_dna(cuda_device, s):
    db = noisy_db(0, 500, seed=3, long_records=3)
    p = ngia.params_clamp(0, s, 8, 0)
    rng = np.random.default_rng(5)
    reps = [0, 1, 2, 3, db.n // 2, db.n - 1]
    _check_pairs(db, p, reps, rng)


@pytest.mark.parametrize("s,w", [(0.5, 2), (0.7, 3), (0.9, 3)])
def test_pair_scores_protein(cuda_device, s, w):
    db = noisy_db(1, 400, seed=4, long_records=2)
    p = ngia.params_clamp(1, s, w, 0)
    rng = np.random.default_rng(6)
    _check_pairs(db, p, [0, 1, 2, 5, db.n // 3, db.n - 1], rng)


def test_pair_scores_band_rounding(cuda_device):
    """L1=113, L2=90, s=0.9: one fused multiply-add gives band 2, separate
    rounding would give band 1 (the reference's kernels are contracted)."""
    rng = np.random.default_rng(7)
    seqs = [bytes(b"ACGT"[int(i)] for i in rng.integers(0, 4, L)) for L in (113, 90, 90, 100, 64)]
    db = seqs_to_db(0, seqs)
    p = ngia.params_clamp(0, 0.9, 5, 0)
    with ngia.Context(db) as ctx:
        got = ctx.pair_scores(p, 0, np.arange(db.n, dtype=np.int32))
    exp = _oracle_pairs(db, p, 0, range(db.n))
    assert np.array_equal(got, exp)
    idx90 = [i for i in range(db.n) if db.read_len[i] == 90]
    assert all(got[i, 3] == 2 for i in idx90)


@pytest.mark.parametrize("s", [0.8, 0.85, 0.9, 0.95])
def test_cluster_dna(cuda_device, s):
    db = family_db(0, n=500, anc=10, seed=int(s * 100))
    p = ngia.params_clamp(0, s, 5, 0)
    _check_cluster(db, p)


def test_cluster_dna_noisy(cuda_device):
    db = noisy_db(0, 600, seed=9, long_records=2)
    _check_cluster(db, ngia.params_clamp(0, 0.85, 5, 0))


def test_cluster_dna_precise(cuda_device):
    db = family_db(0, n=400, anc=8, seed=21)
    _check_cluster(db, ngia.params_clamp(0, 0.9, 6, 1))


def test_cluster_short_records(cuda_device):
    """Records of net length < 16 make the reference's word kernel return a
    whole thread; the exact path reproduces which jobs skip the test."""
    db = noisy_db(0, 500, seed=12, short_records=25)
    assert (db.words[db.rec_off + 1] < 16).any()
    _check_cluster(db, ngia.params_clamp(0, 0.88, 7, 0))


@pytest.mark.parametrize("s,w", [(0.5, 2), (0.9, 3)])
def test_cluster_protein(cuda_device, s, w):
    db = family_db(1, n=400, anc=10, seed=31)
    _check_cluster(db, ngia.params_clamp(1, s, w, 0))


def test_cluster_protein_precise_forced(cuda_device):
    """Protein below s=0.5: the clamps force precise mode (func.cu:71), so
    the short-word test is off; every driver form against the oracle."""
    db = family_db(1, n=400, anc=10, seed=33)
    p = ngia.params_clamp(1, 0.45, 3, 0)
    assert p.precise == 1 and p.word_length == 2
    _check_cluster(db, p, modes=(ngia.MODE_PLAIN, ngia.MODE_GRAPH, ngia.MODE_SPEC))


@pytest.mark.parametrize("db_type,s,w", [(0, 0.95, 5), (0, 0.93, 8), (1, 0.9, 3), (1, 0.5, 2)])
def test_cluster_long_records_word_first(cuda_device, db_type, s, w):
    """Short-word test first, on candidates both sides of 2,048 residues:
    the filter counts the longer ones with the whole warp."""
    if db_type == 0:
        db = family_db(0, n=160, anc=6, seed=61, len_a=2100.0, len_b=500.0, len_min=1200, len_max=6000,
                       subst_max=0.05)
    else:
        db = family_db(1, n=160, anc=6, seed=62, len_a=2000.0, len_b=0.6, len_min=200, len_max=9000,
                       subst_max=0.15)
    net = db.words[db.rec_off + 1]
    assert (net > 2048).sum() >= 20 and (net <= 2048).sum() >= 20
    _check_cluster(db, ngia.params_clamp(db_type, s, w, 0))


@pytest.mark.parametrize("order", ["1", "2"])
def test_word_orders_agree(cuda_device, order, monkeypatch):
    """Short-word test before or after the alignment: same members."""
    monkeypatch.setenv("NGIA_WORD_ORDER", order)
    db = family_db(0, n=400, anc=8, seed=41)
    for s in (0.85, 0.95):
        _check_cluster(db, ngia.params_clamp(0, s, 5, 0), modes=(ngia.MODE_GRAPH,))


@pytest.mark.parametrize("warp_pairs", ["0", "100000000"])
@pytest.mark.parametrize("db_type,s,w", [(0, 0.85, 5), (0, 0.5, 4), (1, 0.9, 3)])
def test_thread_and_warp_per_pair_agree(cuda_device, monkeypatch, warp_pairs, db_type, s, w):
    """Every class forced to thread-per-pair (0) or warp-per-pair (always):
    both give the oracle's clustering, long records (multi-strip bands)
    included."""
    monkeypatch.setenv("NGIA_WARP_PAIRS", warp_pairs)
    db = noisy_db(db_type, 300, seed=44 + db_type, long_records=3)
    _check_cluster(db, ngia.params_clamp(db_type, s, w, 0))


def test_reload_reuses_the_context(cuda_device):
    """ngia_reload: the same database again (graph kept), a smaller one, and
    one that does not fit."""
    big = family_db(0, n=400, anc=8, seed=52)
    small = family_db(0, n=150, anc=4, seed=53, len_max=600)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    exp_big = oracle.cluster(big.words, big.rec_off, 0, p.similarity, p.word_length, p.precise)
    exp_small = oracle.cluster(small.words, small.rec_off, 0, p.similarity, p.word_length, p.precise)
    with ngia.Context(big) as ctx:
        first = ctx.cluster(p, ngia.MODE_GRAPH)
        ctx.reload(big)
        again = ctx.cluster(p, ngia.MODE_GRAPH)
        ctx.reload(small)
        sm = ctx.cluster(p, ngia.MODE_GRAPH)
        sm_plain = ctx.cluster(p, ngia.MODE_PLAIN)
        with pytest.raises(ngia.NgiaError) as ex:
            ctx.reload(family_db(0, n=500, anc=8, seed=54))
        assert ex.value.code == -8
    for got, exp in ((first, exp_big), (again, exp_big), (sm, exp_small), (sm_plain, exp_small)):
        assert np.array_equal(got[0], exp[0]) and np.array_equal(got[1], exp[1])


@pytest.mark.parametrize("mode", [ngia.MODE_PLAIN, ngia.MODE_GRAPH])
def test_checkpoint_resume(cuda_device, tmp_path, mode):
    """A run saved after some iterations and resumed in another context ends
    exactly as the uninterrupted run; foreign or damaged files are refused."""
    db = family_db(0, n=400, anc=8, seed=55)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    ck = tmp_path / "run.ckpt"
    with ngia.Context(db) as ctx:
        full = ctx.cluster(p, ngia.MODE_GRAPH)
        ctx.begin(p, mode)
        ctx.step(9)
        ctx.save(ck)
    with ngia.Context(db) as ctx:
        ctx.resume(ck, mode)
        while not ctx.step(50):
            pass
        cl, ident, st = ctx.end()
    assert np.array_equal(cl, full[0]) and np.array_equal(ident, full[1])
    assert st["iterations"] == full[2]["iterations"] and st["candidates"] == full[2]["candidates"]
    other = family_db(0, n=400, anc=8, seed=56)
    with ngia.Context(other) as ctx:
        with pytest.raises(ngia.NgiaError) as ex:
            ctx.resume(ck, mode)
        assert ex.value.code == -3
    raw = bytearray(ck.read_bytes())
    raw[len(raw) // 2] ^= 0x40
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(bytes(raw))
    with ngia.Context(db) as ctx:
        with pytest.raises(ngia.NgiaError) as ex:
            ctx.resume(bad, mode)
        assert ex.value.code == -3


@pytest.mark.parametrize("db_type,s,w", [(0, 0.85, 5), (0, 0.95, 5), (1, 0.9, 3)])
def test_tuning_changes_speed_not_results(cuda_device, db_type, s, w):
    """ngia_autotune and explicit settings: the clustering stays the oracle's."""
    db = noisy_db(db_type, 300, seed=66 + db_type, long_records=2)
    p = ngia.params_clamp(db_type, s, w, 0)
    ocl, oid, _ = oracle.cluster(db.words, db.rec_off, db_type, p.similarity, p.word_length, p.precise)
    with ngia.Context(db) as ctx:
        t = ctx.autotune(p, iters=3)
        assert t["candidates"] >= 6 and t["ms_per_iter"] > 0
        got = [ctx.cluster(p, ngia.MODE_GRAPH)]
        for wo, rf, wp in ((1, 24, 0), (2, 1, 10 ** 8), (0, 32, -1)):
            ctx.set_tuning(wo, rf, wp)
            got.append(ctx.cluster(p, ngia.MODE_GRAPH))
            got.append(ctx.cluster(p, ngia.MODE_PLAIN))
        # per length bucket: alternating thread-only / warp-heavy cut-offs and
        # halved CTA counts, and the one-word filter tile
        ctx.set_tuning(2 if db_type == 0 else 1, 32, -1, class_warp_pairs=[0, 10 ** 6] * 4,
                       class_grid_div=[2, 1] * 4, filter_tile=1)
        got.append(ctx.cluster(p, ngia.MODE_GRAPH))
        got.append(ctx.cluster(p, ngia.MODE_PLAIN))
        with pytest.raises(ngia.NgiaError):
            ctx.set_tuning(3, 32, -1)
        with pytest.raises(ngia.NgiaError):
            ctx.set_tuning(0, 32, -1, filter_tile=4)
    with ngia.Context(db) as ctx:  # the same database shape and parameters: from the cache
        t2 = ctx.autotune(p, iters=3)
        assert t2["cached"] == 1 and t2["candidates"] == 0
        assert (t2["word_order"], t2["refill"], t2["warp_pairs"], t2["filter_tile"]) == \
            (t["word_order"], t["refill"], t["warp_pairs"], t["filter_tile"])
        assert t2["class_warp_pairs"] == t["class_warp_pairs"] and t2["class_grid_div"] == t["class_grid_div"]
        got.append(ctx.cluster(p, ngia.MODE_GRAPH))
    for cl, ident, _ in got:
        assert np.array_equal(cl, ocl) and np.array_equal(ident, oid)


def test_stepwise_equals_full(cuda_device):
    db = family_db(0, n=400, anc=8, seed=51)
    p = ngia.params_clamp(0, 0.85, 5, 0)
    with ngia.Context(db) as ctx:
        full = ctx.cluster(p, ngia.MODE_GRAPH)
        for mode in (ngia.MODE_PLAIN, ngia.MODE_GRAPH):
            ctx.begin(p, mode)
            steps = 0
            while not ctx.step(7):
                steps += 1
            cl, ident, st = ctx.end()
            assert np.array_equal(cl, full[0]) and np.array_equal(ident, full[1])
            assert st["iterations"] == full[2]["iterations"]
            assert steps == (st["iterations"] - 1) // 7


def test_cli_outputs_identical(cuda_device, tmp_path):
    """makeDB -> cluster CLI -> cluster.txt / represent.fasta byte-identical
    to the oracle's restatement of the reference writer."""
    seq, off = ngia.synth(type=0, n_seqs=300, n_ancestors=6, len_a=500.0, len_b=50.0, len_min=300,
                          len_max=700, seed=61)
    fa = tmp_path / "in.fasta"
    ngia.write_fasta(str(fa), seq, off, width=70)
    dbdir, o1, o2 = tmp_path / "db", tmp_path / "gpu", tmp_path / "cpu"
    for d in (dbdir, o1, o2):
        d.mkdir()
    b = ROOT / "ngia-metax_gb300" / "_build"
    subprocess.run([str(b / "makeDB"), "-i", str(fa), "-o", str(dbdir), "-t", "0"], check=True,
                   capture_output=True)
    r = subprocess.run([str(b / "cluster"), "-i", str(dbdir), "-o", str(o1), "-w", "5", "-s", "0.85"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    subprocess.run([str(ROOT / "oracle" / "_build" / "ngia_oracle"), "-i", str(dbdir), "-o", str(o2), "-w", "5",
                    "-s", "0.85"], check=True, capture_output=True)
    for f in ("cluster.txt", "represent.fasta"):
        assert (o1 / f).read_bytes() == (o2 / f).read_bytes(), f
    assert "Cluster:\t" in r.stdout


def test_cli_resumes_a_checkpoint(cuda_device, tmp_path):
    """cluster with NGIA_CHECKPOINT: resumes a run saved through the C ABI and
    writes the same files as an uninterrupted run."""
    seq, off = ngia.synth(type=0, n_seqs=300, n_ancestors=6, len_a=500.0, len_b=50.0, len_min=300,
                          len_max=700, seed=62)
    fa = tmp_path / "in.fasta"
    ngia.write_fasta(str(fa), seq, off, width=70)
    dbdir, o1, o2 = tmp_path / "db", tmp_path / "plain", tmp_path / "resumed"
    for d in (dbdir, o1, o2):
        d.mkdir()
    b = ROOT / "ngia-metax_gb300" / "_build"
    subprocess.run([str(b / "makeDB"), "-i", str(fa), "-o", str(dbdir), "-t", "0"], check=True, capture_output=True)
    args = ["-i", str(dbdir), "-w", "5", "-s", "0.85"]
    subprocess.run([str(b / "cluster"), "-o", str(o1)] + args, check=True, capture_output=True)
    db = ngia.DB.load(str(dbdir))
    ck = tmp_path / "run.ckpt"
    with ngia.Context(db) as ctx:
        ctx.begin(ngia.params_clamp(0, 0.85, 5, 0), ngia.MODE_GRAPH)
        ctx.step(11)
        ctx.save(ck)
    env = dict(os.environ, NGIA_CHECKPOINT=str(ck), NGIA_CHECKPOINT_EVERY="7")
    r = subprocess.run([str(b / "cluster"), "-o", str(o2)] + args, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    for f in ("cluster.txt", "represent.fasta"):
        assert (o1 / f).read_bytes() == (o2 / f).read_bytes(), f
