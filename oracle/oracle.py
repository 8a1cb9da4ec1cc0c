"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py as the reference results; the product never
imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
NSTATS = 8
STAT_NAMES = ["iterations", "candidates", "base_pass", "word_eval", "word_pass", "members", "cells",
              "filter_bytes"]

_lib = None
_nofma = None


def lib(nofma: bool = False) -> C.CDLL:
    """The oracle library; nofma=True gives the separately rounded band-shift
    variant used only to search for inputs that tell the two apart."""
    global _lib, _nofma
    if nofma:
        if _nofma is None:
            _nofma = _load(HERE / "_build" / "liboracle_nofma.so")
        return _nofma
    if _lib is None:
        _lib = _load(LIB)
    return _lib


def _load(path: Path) -> C.CDLL:
    if True:
        if not path.exists():
            raise ImportError(f"{path} is missing: build it with oracle/build_oracle.py")
        L = C.CDLL(str(path))
        P = C.POINTER
        L.ora_cluster.restype = C.c_int64
        L.ora_cluster.argtypes = [P(C.c_uint32), P(C.c_int64), C.c_int, C.c_int, C.c_float, C.c_int, C.c_int,
                                  C.c_int, C.c_int64, P(C.c_int32), P(C.c_int32), P(C.c_int64)]
        L.ora_pair.restype = None
        L.ora_pair.argtypes = [P(C.c_uint32), P(C.c_int64), C.c_int, C.c_float, C.c_int, C.c_int, C.c_int,
                               P(C.c_int32)]
        L.ora_clamp.restype = None
        L.ora_clamp.argtypes = [C.c_int, P(C.c_float), P(C.c_int), P(C.c_int)]
        L.ora_dp_sum.restype = C.c_int
        L.ora_dp_sum.argtypes = [P(C.c_uint32), P(C.c_uint32), C.c_int, C.c_float, P(C.c_int), P(C.c_int64)]
        L.ora_pack.restype = C.c_int64
        L.ora_pack.argtypes = [C.c_int, C.c_char_p, P(C.c_int64), C.c_int64, P(C.c_uint32), P(C.c_int64),
                               P(C.c_int64)]
    return L


def pack(db_type: int, seq, off: np.ndarray):
    """makeDB records of raw sequences in FASTA order (the oracle's own
    restatement of makeDB's packing): (words uint32, rec_off int64)."""
    buf = seq.tobytes() if isinstance(seq, np.ndarray) else bytes(seq)
    off = np.ascontiguousarray(off, dtype=np.int64)
    n = len(off) - 1
    nw = C.c_int64()
    k = lib().ora_pack(db_type, buf, off.ctypes.data_as(C.POINTER(C.c_int64)), n, None, None, C.byref(nw))
    words = np.empty(max(1, nw.value), dtype=np.uint32)
    rec_off = np.empty(max(1, k), dtype=np.int64)
    lib().ora_pack(db_type, buf, off.ctypes.data_as(C.POINTER(C.c_int64)), n,
                   words.ctypes.data_as(C.POINTER(C.c_uint32)), rec_off.ctypes.data_as(C.POINTER(C.c_int64)),
                   C.byref(nw))
    return words[:nw.value], rec_off[:k]


class _SynthParams(C.Structure):
    _fields_ = [("type", C.c_int32), ("len_dist", C.c_int32), ("n_seqs", C.c_int64), ("n_ancestors", C.c_int32),
                ("len_min", C.c_int32), ("len_max", C.c_int32), ("len_a", C.c_double), ("len_b", C.c_double),
                ("subst_max", C.c_double), ("indel_frac", C.c_double), ("indel_max", C.c_int32),
                ("novel_frac", C.c_double), ("seed", C.c_uint64)]


_synth = None


def synth(seed: int, **cfg):
    """The seeded workload generator (oracle/_build/libsynth.so, built from
    the generator source alone): (residues as a uint8 array, offsets[n+1])."""
    global _synth
    if _synth is None:
        path = HERE / "_build" / "libsynth.so"
        if not path.exists():
            raise ImportError(f"{path} is missing: build it with oracle/build_oracle.py")
        _synth = C.CDLL(str(path))
    sp = _SynthParams(type=cfg.get("type", 0), len_dist=cfg.get("len_dist", 0), n_seqs=cfg["n_seqs"],
                      n_ancestors=cfg["n_ancestors"], len_min=cfg["len_min"], len_max=cfg["len_max"],
                      len_a=cfg["len_a"], len_b=cfg["len_b"], subst_max=cfg.get("subst_max", 0.2),
                      indel_frac=cfg.get("indel_frac", 0.05), indel_max=cfg.get("indel_max", 3),
                      novel_frac=cfg.get("novel_frac", 0.0), seed=seed)
    sp_ptr, off_ptr, n = C.c_void_p(), C.POINTER(C.c_int64)(), C.c_int64()
    rc = _synth.ngia_synth_generate(C.byref(sp), C.byref(sp_ptr), C.byref(off_ptr), C.byref(n))
    if rc != 0:
        raise RuntimeError(f"synth failed ({rc})")
    off = np.ctypeslib.as_array(off_ptr, shape=(n.value + 1,)).copy()
    seq = np.ctypeslib.as_array(C.cast(sp_ptr, C.POINTER(C.c_uint8)), shape=(int(off[-1]),)).copy()
    _synth.ngia_free(sp_ptr)
    _synth.ngia_free(C.cast(off_ptr, C.c_void_p))
    return seq, off


def clamp(db_type: int, s: float, w: int, precise: int = 0):
    sf, wi, pi = C.c_float(s), C.c_int(w), C.c_int(precise)
    lib().ora_clamp(db_type, C.byref(sf), C.byref(wi), C.byref(pi))
    return sf.value, wi.value, pi.value


def cluster(words: np.ndarray, rec_off: np.ndarray, db_type: int, s: float, w: int, precise: int = 0,
            threads: int = 0, max_iters: int = 0, nofma: bool = False):
    """Clusters with already-clamped parameters; returns (cluster, identity, stats)."""
    words = np.ascontiguousarray(words, dtype=np.uint32)
    rec_off = np.ascontiguousarray(rec_off, dtype=np.int64)
    n = len(rec_off)
    cl = np.empty(n, dtype=np.int32)
    ident = np.empty(n, dtype=np.int32)
    st = np.zeros(NSTATS, dtype=np.int64)
    lib(nofma).ora_cluster(words.ctypes.data_as(C.POINTER(C.c_uint32)), rec_off.ctypes.data_as(C.POINTER(C.c_int64)),
                      n, db_type, C.c_float(s), w, precise, threads, max_iters,
                      cl.ctypes.data_as(C.POINTER(C.c_int32)), ident.ctypes.data_as(C.POINTER(C.c_int32)),
                      st.ctypes.data_as(C.POINTER(C.c_int64)))
    return cl, ident, dict(zip(STAT_NAMES, (int(x) for x in st)))


def pair(words: np.ndarray, rec_off: np.ndarray, db_type: int, s: float, w: int, rep: int, cand: int):
    """(composition sum, word count or -1, dp score, band, base ok, word ok, dp ok, band cells)."""
    words = np.ascontiguousarray(words, dtype=np.uint32)
    rec_off = np.ascontiguousarray(rec_off, dtype=np.int64)
    out = np.zeros(8, dtype=np.int32)
    lib().ora_pair(words.ctypes.data_as(C.POINTER(C.c_uint32)), rec_off.ctypes.data_as(C.POINTER(C.c_int64)),
                   db_type, C.c_float(s), w, rep, cand, out.ctypes.data_as(C.POINTER(C.c_int32)))
    return out


def assign(rep_words: np.ndarray, rep_off: np.ndarray, q_words: np.ndarray, q_off: np.ndarray, db_type: int,
           s: float, w: int, precise: int = 0, threads: int = 0):
    """Serving semantics (ora_assign): (rep_out, ident_out, new representatives)."""
    rw = np.ascontiguousarray(rep_words, dtype=np.uint32)
    ro = np.ascontiguousarray(rep_off, dtype=np.int64)
    qw = np.ascontiguousarray(q_words, dtype=np.uint32)
    qo = np.ascontiguousarray(q_off, dtype=np.int64)
    nq = len(qo)
    rep = np.empty(nq, dtype=np.int32)
    ident = np.empty(nq, dtype=np.int32)
    f = lib().ora_assign
    f.restype = C.c_int64
    k = f(rw.ctypes.data_as(C.POINTER(C.c_uint32)), ro.ctypes.data_as(C.POINTER(C.c_int64)), len(ro),
          qw.ctypes.data_as(C.POINTER(C.c_uint32)), qo.ctypes.data_as(C.POINTER(C.c_int64)), nq, db_type,
          C.c_float(s), w, precise, threads, rep.ctypes.data_as(C.POINTER(C.c_int32)),
          ident.ctypes.data_as(C.POINTER(C.c_int32)))
    return rep, ident, int(k)


def dp_sum(rep_rec: np.ndarray, query_rec: np.ndarray, db_type: int, s: float):
    """Alignment score of two raw records; returns (score, band, cells)."""
    r = np.ascontiguousarray(rep_rec, dtype=np.uint32)
    q = np.ascontiguousarray(query_rec, dtype=np.uint32)
    band, cells = C.c_int(), C.c_int64()
    sc = lib().ora_dp_sum(r.ctypes.data_as(C.POINTER(C.c_uint32)), q.ctypes.data_as(C.POINTER(C.c_uint32)),
                          db_type, C.c_float(s), C.byref(band), C.byref(cells))
    return sc, band.value, cells.value
