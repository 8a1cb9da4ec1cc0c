"""Python binding of libngia (include/ngia.h) over ctypes.

The library is the product; this module only marshals arguments.  It loads
``_build/libngia.so`` next to this file and raises if it is missing (there is
no fallback implementation).  Arrays cross the boundary as numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libngia.so"

MODE_PLAIN = 0
MODE_GRAPH = 1
MODE_SPEC = 2
MODE_POOL = 3  # batches only: the jobs of one record type share every launch
POLICY_THREAD, POLICY_CUTOFF, POLICY_TUNED = 0, 1, 2  # batch policies of MODE_GRAPH runs


class NgiaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ngia error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("similarity", C.c_float), ("word_length", C.c_int32), ("precise", C.c_int32)]


class DBView(C.Structure):
    _fields_ = [("n", C.c_int32), ("type", C.c_int32), ("longest", C.c_int32), ("shortest", C.c_int32),
                ("words", C.POINTER(C.c_uint32)), ("n_words", C.c_int64), ("rec_off", C.POINTER(C.c_int64))]


class DBHost(C.Structure):
    _fields_ = [("view", DBView), ("name_len", C.POINTER(C.c_int32)), ("read_len", C.POINTER(C.c_int32)),
                ("fasta_off", C.POINTER(C.c_int64)), ("pack_off", C.POINTER(C.c_int64))]


class SynthParams(C.Structure):
    _fields_ = [("type", C.c_int32), ("len_dist", C.c_int32), ("n_seqs", C.c_int64), ("n_ancestors", C.c_int32),
                ("len_min", C.c_int32), ("len_max", C.c_int32), ("len_a", C.c_double), ("len_b", C.c_double),
                ("subst_max", C.c_double), ("indel_frac", C.c_double), ("indel_max", C.c_int32),
                ("novel_frac", C.c_double), ("seed", C.c_uint64)]


class ServeConfig(C.Structure):
    _fields_ = [("slots", C.c_int32), ("max_batch", C.c_int32), ("max_record_blocks", C.c_int32),
                ("reserved", C.c_int32), ("max_batch_words", C.c_int64), ("memory_budget", C.c_int64)]


class ServeResult(C.Structure):
    _fields_ = [("done", C.c_int32), ("slot", C.c_int32), ("rounds", C.c_int32), ("resident", C.c_int32),
                ("new_reps", C.c_int32), ("reserved", C.c_int32), ("queued_ms", C.c_double),
                ("run_ms", C.c_double), ("pairs", C.c_int64), ("cells", C.c_int64)]


class Tuning(C.Structure):
    _fields_ = [("word_order", C.c_int32), ("refill", C.c_int32), ("warp_pairs", C.c_int32),
                ("candidates", C.c_int32), ("ms_per_iter", C.c_double), ("default_ms_per_iter", C.c_double),
                ("class_warp_pairs", C.c_int32 * 8), ("class_grid_div", C.c_int32 * 8), ("filter_tile", C.c_int32),
                ("cached", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("iterations", "candidates", "base_pass", "align_pairs", "members",
                                         "band_cells", "filter_bytes", "word_checks", "done_cells")] + \
        [("ms_filter", C.c_double), ("ms_align", C.c_double), ("class_pairs", C.c_int64 * 8),
         ("class_ms", C.c_double * 8), ("class_cells", C.c_int64 * 8),
         ("class_bytes", C.c_int64 * 8)]

    def as_dict(self) -> dict:
        d = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            d[n] = list(v) if n.startswith("class_") else (float(v) if n.startswith("ms_") else int(v))
        return d


_lib = None


def lib() -> C.CDLL:
    """Loads libngia.so (built by build_native.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
    L = C.CDLL(str(LIB_PATH))
    P, I32, I64, VP = C.POINTER, C.c_int32, C.c_int64, C.c_void_p
    sig = {
        "ngia_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "ngia_version": (C.c_char_p, []),
        "ngia_free": (None, [VP]),
        "ngia_params_clamp": (C.c_int, [I32, P(Params)]),
        "ngia_db_load": (C.c_int, [C.c_char_p, P(P(DBHost))]),
        "ngia_db_pack": (C.c_int, [I32, C.c_char_p, P(I64), I64, P(I32), P(P(DBHost))]),
        "ngia_makedb": (C.c_int, [C.c_char_p, C.c_char_p, I32]),
        "ngia_save_result": (C.c_int, [C.c_char_p, C.c_char_p, P(DBHost), P(I32), P(I32)]),
        "ngia_db_free": (None, [P(DBHost)]),
        "ngia_synth_generate": (C.c_int, [P(SynthParams), P(VP), P(P(I64)), P(I64)]),
        "ngia_write_fasta": (C.c_int, [C.c_char_p, C.c_char_p, P(I64), I64, I32]),
        "ngia_open": (C.c_int, [P(DBView), P(VP)]),
        "ngia_cluster": (C.c_int, [VP, P(Params), I32, P(I32), P(I32), P(Stats)]),
        "ngia_cluster_begin": (C.c_int, [VP, P(Params), I32]),
        "ngia_cluster_step": (C.c_int, [VP, I64, P(I32)]),
        "ngia_cluster_end": (C.c_int, [VP, P(I32), P(I32), P(Stats)]),
        "ngia_pair_scores": (C.c_int, [VP, P(Params), I32, P(I32), I32, P(I32)]),
        "ngia_stream": (VP, [VP]),
        "ngia_device_count": (C.c_int, [P(I32)]),
        "ngia_set_device": (C.c_int, [I32]),
        "ngia_pin_host": (C.c_int, [VP, C.c_size_t]),
        "ngia_unpin_host": (C.c_int, [VP]),
        "ngia_measure_int_peak": (C.c_int, [P(C.c_double)]),
        "ngia_measure_filter_floor": (C.c_int, [VP, P(C.c_double), P(C.c_double)]),
        "ngia_cluster_stats": (C.c_int, [VP, P(Stats)]),
        "ngia_step_device_ms": (C.c_int, [VP, P(C.c_float)]),
        "ngia_set_profiling": (C.c_int, [VP, I32]),
        "ngia_rep_scores_noalloc": (C.c_int, [VP, I64, VP, I32, I32, C.c_float, VP, VP]),
        "ngia_batch_open": (C.c_int, [P(DBView), I32, P(VP)]),
        "ngia_batch_run": (C.c_int, [VP, P(Params), I32, I64, P(P(I32)), P(P(I32)), P(Stats)]),
        "ngia_batch_close": (C.c_int, [VP]),
        "ngia_batch_autotune": (C.c_int, [VP, P(Params), I32, P(Tuning)]),
        "ngia_batch_set_policy": (C.c_int, [VP, I32]),
        "ngia_batch_policy": (C.c_int, [VP, P(I32)]),
        "ngia_serve_open": (C.c_int, [P(DBView), P(Params), P(ServeConfig), P(VP)]),
        "ngia_serve_slots": (C.c_int, [VP, P(I32)]),
        "ngia_serve_submit": (C.c_int, [VP, P(DBView), P(I64)]),
        "ngia_serve_poll": (C.c_int, [VP, I64, I32, P(I32), P(I32), P(ServeResult)]),
        "ngia_serve_close": (C.c_int, [VP]),
        "ngia_close": (C.c_int, [VP]),
        "ngia_reload": (C.c_int, [VP, P(DBView)]),
        "ngia_cluster_save": (C.c_int, [VP, C.c_char_p]),
        "ngia_autotune": (C.c_int, [VP, P(Params), I32, P(Tuning)]),
        "ngia_set_tuning": (C.c_int, [VP, P(Tuning)]),
        "ngia_cluster_resume": (C.c_int, [VP, C.c_char_p, I32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib().ngia_last_error(buf, 512)
        raise NgiaError(rc, buf.value.decode(errors="replace"))


def _i32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _i64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def device_count() -> int:
    n = C.c_int32()
    _check(lib().ngia_device_count(C.byref(n)))
    return n.value


def set_device(dev: int) -> None:
    _check(lib().ngia_set_device(dev))


def measure_int_peak() -> float:
    """INT32 lane-operations per second / 1e9 of the current device (probe)."""
    g = C.c_double()
    _check(lib().ngia_measure_int_peak(C.byref(g)))
    return g.value


def pin_host(arr: np.ndarray) -> None:
    _check(lib().ngia_pin_host(arr.ctypes.data, arr.nbytes))


def unpin_host(arr: np.ndarray) -> None:
    _check(lib().ngia_unpin_host(arr.ctypes.data))


def rep_scores_noalloc(d_words: int, rep_off: int, d_query_off: int, n: int, db_type: int, similarity: float,
                       d_scores: int, stream: int = 0) -> None:
    """Scores one representative against n queries; all pointers are device
    addresses owned by the caller (the library allocates nothing)."""
    _check(lib().ngia_rep_scores_noalloc(d_words, rep_off, d_query_off, n, db_type, similarity, d_scores,
                                         stream or None))


def params_clamp(db_type: int, similarity: float, word_length: int, precise: int = 0) -> Params:
    p = Params(similarity, word_length, precise)
    _check(lib().ngia_params_clamp(db_type, C.byref(p)))
    return p


# ---- synthetic workloads (the five benchmark configurations) ----------------
CONFIGS = {
    # 20,000 DNA from 400 ancestors, N(1450, 80) clipped [1200, 1700]
    "dna_small": dict(type=0, len_dist=0, n_seqs=20000, n_ancestors=400, len_a=1450.0, len_b=80.0,
                      len_min=1200, len_max=1700, subst_max=0.20, indel_frac=0.05, indel_max=3),
    # 1,000,000 DNA from 20,000 ancestors, N(1450, 120) clipped [900, 2000]
    "dna_1m": dict(type=0, len_dist=0, n_seqs=1000000, n_ancestors=20000, len_a=1450.0, len_b=120.0,
                   len_min=900, len_max=2000, subst_max=0.20, indel_frac=0.05, indel_max=3),
    # 200,000 proteins from 8,000 ancestors, lognormal(median 380, sigma 0.7) clipped [20, 35000]
    "protein_200k": dict(type=1, len_dist=1, n_seqs=200000, n_ancestors=8000, len_a=380.0, len_b=0.7,
                         len_min=20, len_max=35000, subst_max=0.50, indel_frac=0.05, indel_max=5),
}


def class_kernels(db_type: int) -> list[str]:
    """Thread-per-pair kernel of each alignment work class (by band window,
    in 32-residue blocks); every class also launches the warp-per-pair
    kernel, which does the class's work instead when it has few pairs."""
    if db_type == 0:
        return ["k_align_win<2,8>", "k_align_win<2,16>", "k_align_win<2,24>", "k_align_win<2,32>",
                "k_align_tiled<2,64>", "k_align_tiled<2,128>", "k_align_tiled<2,0>"]
    return ["k_align_win<5,8>", "k_align_win<5,16>", "k_align_tiled<5,64>", "k_align_tiled<5,128>",
            "k_align_tiled<5,0>"]


class Seqs:
    """Generated residues, owned by the library (no Python-side copy).

    ``seq`` is a zero-copy uint8 view, ``off`` the int64 offsets[n+1];
    ``bytes(i)`` returns sequence i."""

    def __init__(self, ptr: C.c_void_p, off: np.ndarray):
        self._ptr = ptr
        self.off = off
        size = int(off[-1])
        self.seq = (np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(size,)) if size
                    else np.zeros(0, np.uint8))

    @property
    def n(self) -> int:
        return len(self.off) - 1

    def bytes(self, i: int) -> bytes:
        return self.seq[self.off[i]:self.off[i + 1]].tobytes()

    def all_bytes(self) -> list[bytes]:
        return [self.bytes(i) for i in range(self.n)]

    def close(self) -> None:
        if self._ptr:
            lib().ngia_free(self._ptr)
            self._ptr = None
            self.seq = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __iter__(self):  # (seq, off) unpacking
        yield self
        yield self.off


def synth(type: int = 0, n_seqs: int = 1000, n_ancestors: int = 20, len_dist: int = 0, len_a: float = 1450.0,
          len_b: float = 80.0, len_min: int = 1200, len_max: int = 1700, subst_max: float = 0.2,
          indel_frac: float = 0.05, indel_max: int = 3, novel_frac: float = 0.0, seed: int = 1) -> Seqs:
    """Generates sequences (library-owned buffer); unpacks as (seqs, offsets)."""
    p = SynthParams(type, len_dist, n_seqs, n_ancestors, len_min, len_max, len_a, len_b, subst_max, indel_frac,
                    indel_max, novel_frac, seed)
    seq = C.c_void_p()
    off = C.POINTER(C.c_int64)()
    n = C.c_int64()
    _check(lib().ngia_synth_generate(C.byref(p), C.byref(seq), C.byref(off), C.byref(n)))
    try:
        offs = np.ctypeslib.as_array(off, shape=(n.value + 1,)).copy()
    finally:
        lib().ngia_free(C.cast(off, C.c_void_p))
    return Seqs(seq, offs)


def _seq_ptr(seq):
    """Pointer to residue bytes given bytes, a uint8 array or a Seqs."""
    if isinstance(seq, Seqs):
        return C.cast(seq._ptr, C.c_char_p), seq
    if isinstance(seq, np.ndarray):
        a = np.ascontiguousarray(seq, dtype=np.uint8)
        return a.ctypes.data_as(C.c_char_p), a
    return seq, seq


def write_fasta(path: str, seq, off: np.ndarray, width: int = 80) -> None:
    off = np.ascontiguousarray(off, dtype=np.int64)
    ptr, keep = _seq_ptr(seq)
    _check(lib().ngia_write_fasta(str(path).encode(), ptr, _i64p(off), len(off) - 1, width))
    del keep


class DB:
    """A makeDB database in host memory (owned by the library)."""

    def __init__(self, ptr):
        self._ptr = ptr
        h = ptr.contents
        v = h.view
        self.n, self.type, self.longest, self.shortest = v.n, v.type, v.longest, v.shortest
        self.words = np.ctypeslib.as_array(v.words, shape=(v.n_words,))
        self.rec_off = np.ctypeslib.as_array(v.rec_off, shape=(v.n,))
        self.read_len = np.ctypeslib.as_array(h.read_len, shape=(v.n,))
        self.name_len = np.ctypeslib.as_array(h.name_len, shape=(v.n,))
        self.fasta_off = np.ctypeslib.as_array(h.fasta_off, shape=(v.n,))
        self.pack_off = np.ctypeslib.as_array(h.pack_off, shape=(v.n,))

    @property
    def view(self) -> DBView:
        return self._ptr.contents.view

    @classmethod
    def load(cls, dirpath: str) -> "DB":
        p = C.POINTER(DBHost)()
        _check(lib().ngia_db_load(str(dirpath).encode(), C.byref(p)))
        return cls(p)

    @classmethod
    def pack(cls, db_type: int, seq, off: np.ndarray) -> "DB":
        off = np.ascontiguousarray(off, dtype=np.int64)
        p = C.POINTER(DBHost)()
        ptr, keep = _seq_ptr(seq)
        _check(lib().ngia_db_pack(db_type, ptr, _i64p(off), len(off) - 1, None, C.byref(p)))
        del keep
        return cls(p)

    def record(self, i: int) -> np.ndarray:
        o = int(self.rec_off[i])
        hw = 6 if self.type == 0 else 30
        P = 2 if self.type == 0 else 5
        L = int(self.words[o])
        return self.words[o:o + hw + (L + 31) // 32 * P]

    def save_result(self, dbdir: str, outdir: str, cluster: np.ndarray) -> int:
        cl = np.ascontiguousarray(cluster, dtype=np.int32)
        nc = C.c_int32()
        _check(lib().ngia_save_result(str(dbdir).encode(), str(outdir).encode(), self._ptr, _i32p(cl),
                                      C.byref(nc)))
        return nc.value

    def close(self) -> None:
        if self._ptr:
            lib().ngia_db_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Records:
    """A makeDB-layout database over caller-owned arrays, records in the given
    order (nothing is re-sorted): e.g. a representative set in creation order,
    or a slice of a database."""

    def __init__(self, db_type: int, words: np.ndarray, rec_off: np.ndarray):
        self.type = db_type
        self.words = np.ascontiguousarray(words, dtype=np.uint32)
        self.rec_off = np.ascontiguousarray(rec_off, dtype=np.int64)
        self.n = len(self.rec_off)
        lens = self.words[self.rec_off] if self.n else np.zeros(1, np.uint32)
        self.longest, self.shortest = int(lens.max()), int(lens.min())
        self._view = DBView(self.n, db_type, self.longest, self.shortest,
                            self.words.ctypes.data_as(C.POINTER(C.c_uint32)), len(self.words), _i64p(self.rec_off))

    @property
    def view(self) -> DBView:
        return self._view

    @classmethod
    def subset(cls, db, idx) -> "Records":
        """Records idx of db (in that order), copied into one compact array."""
        hw, P = (6, 2) if db.type == 0 else (30, 5)
        parts, off, pos = [], [], 0
        for i in np.asarray(idx, dtype=np.int64):
            o = int(db.rec_off[i])
            L = int(db.words[o])
            rec = db.words[o:o + hw + (L + 31) // 32 * P]
            parts.append(rec)
            off.append(pos)
            pos += len(rec)
        words = np.concatenate(parts) if parts else np.zeros(1, np.uint32)
        return cls(db.type, words, np.array(off, dtype=np.int64))

    def close(self) -> None:
        pass


class Server:
    """Continuous-batching assignment against a resident representative set
    (ngia_serve_*): submit() queues a batch and returns a ticket, poll()
    returns (rep, ident, info) once it is done (None before)."""

    def __init__(self, reps, params: Params, slots: int = 4, max_batch: int = 4096, max_record_blocks: int = 128,
                 memory_budget: int = 0):
        self.reps = reps
        cfg = ServeConfig(slots, max_batch, max_record_blocks, 0, 0, memory_budget)
        self._h = C.c_void_p()
        _check(lib().ngia_serve_open(C.byref(reps.view), C.byref(params), C.byref(cfg), C.byref(self._h)))
        self._n = {}

    @property
    def slots(self) -> int:
        n = C.c_int32()
        _check(lib().ngia_serve_slots(self._h, C.byref(n)))
        return n.value

    def submit(self, batch) -> int:
        t = C.c_int64()
        _check(lib().ngia_serve_submit(self._h, C.byref(batch.view), C.byref(t)))
        self._n[t.value] = batch.n
        return t.value

    def poll(self, ticket: int, wait_ms: int = 0):
        n = self._n.get(ticket, 0)  # unknown tickets: the library reports the error
        rep = np.empty(max(n, 1), dtype=np.int32)
        ident = np.empty(max(n, 1), dtype=np.int32)
        res = ServeResult()
        try:
            _check(lib().ngia_serve_poll(self._h, ticket, wait_ms, _i32p(rep), _i32p(ident), C.byref(res)))
        except NgiaError:
            self._n.pop(ticket, None)
            raise
        if not res.done:
            return None
        del self._n[ticket]
        info = {f: getattr(res, f) for f, _ in ServeResult._fields_ if f != "reserved"}
        return rep[:n], ident[:n], info

    def wait(self, ticket: int):
        return self.poll(ticket, -1)

    def close(self) -> None:
        if self._h:
            lib().ngia_serve_close(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def makedb(fasta: str, outdir: str, db_type: int) -> None:
    _check(lib().ngia_makedb(str(fasta).encode(), str(outdir).encode(), db_type))


class Context:
    """Device context: the database resident in HBM plus run buffers."""

    def __init__(self, db: DB):
        self.db = db
        self._h = C.c_void_p()
        _check(lib().ngia_open(C.byref(db.view), C.byref(self._h)))

    def cluster(self, params: Params, mode: int = MODE_GRAPH):
        n = self.db.n
        cl = np.empty(n, dtype=np.int32)
        ident = np.empty(n, dtype=np.int32)
        st = Stats()
        _check(lib().ngia_cluster(self._h, C.byref(params), mode, _i32p(cl), _i32p(ident), C.byref(st)))
        return cl, ident, st.as_dict()

    def reload(self, db) -> None:
        """Loads another database (within this context's capacity) in place."""
        _check(lib().ngia_reload(self._h, C.byref(db.view)))
        self.db = db

    def autotune(self, params: Params, iters: int = 4) -> dict:
        """Times the speed-only settings on the first iterations; keeps the fastest."""
        t = Tuning()
        _check(lib().ngia_autotune(self._h, C.byref(params), iters, C.byref(t)))
        return {f: (list(getattr(t, f)) if f.startswith("class_") else getattr(t, f)) for f, _ in Tuning._fields_}

    def set_tuning(self, word_order: int = 0, refill: int = 32, warp_pairs: int = -1, class_warp_pairs=None,
                   class_grid_div=None, filter_tile: int = 8) -> None:
        t = Tuning(word_order, refill, warp_pairs, 0, 0.0, 0.0)
        for k in range(8):
            t.class_warp_pairs[k] = -1 if class_warp_pairs is None else class_warp_pairs[k]
            t.class_grid_div[k] = 1 if class_grid_div is None else class_grid_div[k]
        t.filter_tile = filter_tile
        _check(lib().ngia_set_tuning(self._h, C.byref(t)))

    def save(self, path: str) -> None:
        """Checkpoint of the run in progress."""
        _check(lib().ngia_cluster_save(self._h, str(path).encode()))

    def resume(self, path: str, mode: int = MODE_GRAPH) -> None:
        """Continues a checkpointed run of this context's database."""
        _check(lib().ngia_cluster_resume(self._h, str(path).encode(), mode))

    def begin(self, params: Params, mode: int = MODE_GRAPH) -> None:
        _check(lib().ngia_cluster_begin(self._h, C.byref(params), mode))

    def step(self, max_iters: int) -> bool:
        done = C.c_int32()
        _check(lib().ngia_cluster_step(self._h, max_iters, C.byref(done)))
        return bool(done.value)

    def end(self):
        n = self.db.n
        cl = np.empty(n, dtype=np.int32)
        ident = np.empty(n, dtype=np.int32)
        st = Stats()
        _check(lib().ngia_cluster_end(self._h, _i32p(cl), _i32p(ident), C.byref(st)))
        return cl, ident, st.as_dict()

    def stats(self) -> dict:
        st = Stats()
        _check(lib().ngia_cluster_stats(self._h, C.byref(st)))
        return st.as_dict()

    def step_ms(self) -> float:
        ms = C.c_float()
        _check(lib().ngia_step_device_ms(self._h, C.byref(ms)))
        return ms.value

    def set_profiling(self, on: bool) -> None:
        _check(lib().ngia_set_profiling(self._h, 1 if on else 0))

    def filter_floor(self) -> tuple[float, float]:
        """(empty launch, read-only pass) in microseconds on the filter's grid
        for the current unclustered set (DNA, begun context)."""
        a, b = C.c_double(), C.c_double()
        _check(lib().ngia_measure_filter_floor(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def pair_scores(self, params: Params, rep: int, cands) -> np.ndarray:
        c = np.ascontiguousarray(cands, dtype=np.int32)
        out = np.empty((len(c), 4), dtype=np.int32)
        _check(lib().ngia_pair_scores(self._h, C.byref(params), rep, _i32p(c), len(c), _i32p(out)))
        return out

    @property
    def stream(self) -> int:
        return lib().ngia_stream(self._h) or 0

    def close(self) -> None:
        if self._h:
            lib().ngia_close(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent clustering jobs run side by side (ngia_batch_*)."""

    def __init__(self, dbs: list):
        self.dbs = list(dbs)
        views = (DBView * len(self.dbs))(*[d.view for d in self.dbs])
        self._h = C.c_void_p()
        _check(lib().ngia_batch_open(views, len(self.dbs), C.byref(self._h)))

    def run(self, params: list, mode: int = MODE_GRAPH, max_iters: int = 0):
        """Returns ([cluster arrays], [identity arrays], summed stats)."""
        n = len(self.dbs)
        ps = (Params * n)(*params)
        cls = [np.empty(d.n, dtype=np.int32) for d in self.dbs]
        ids = [np.empty(d.n, dtype=np.int32) for d in self.dbs]
        cptr = (C.POINTER(C.c_int32) * n)(*[_i32p(a) for a in cls])
        iptr = (C.POINTER(C.c_int32) * n)(*[_i32p(a) for a in ids])
        st = Stats()
        _check(lib().ngia_batch_run(self._h, ps, mode, max_iters, cptr, iptr, C.byref(st)))
        return cls, ids, st.as_dict()

    def autotune(self, params: list, iters: int = 4) -> list:
        """Times the three batch policies (thread per pair, default cut-off,
        each job's own tuning) and keeps the fastest; returns each job's
        settings under it."""
        n = len(self.dbs)
        ps = (Params * n)(*params)
        ts = (Tuning * n)()
        _check(lib().ngia_batch_autotune(self._h, ps, iters, ts))
        return [{f: (list(getattr(t, f)) if f.startswith("class_") else getattr(t, f)) for f, _ in Tuning._fields_}
                for t in ts]

    def set_policy(self, policy: int) -> None:
        """Applies a batch policy (POLICY_*) to later MODE_GRAPH runs."""
        _check(lib().ngia_batch_set_policy(self._h, policy))

    def policy(self) -> int:
        """The policy in force (-1: none chosen)."""
        v = C.c_int32()
        _check(lib().ngia_batch_policy(self._h, C.byref(v)))
        return v.value

    def close(self) -> None:
        if self._h:
            lib().ngia_batch_close(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
