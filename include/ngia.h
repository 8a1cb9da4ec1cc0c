/*
 * ngia.h — C ABI of the GB300 greedy sequence-clustering library (libngia.so).
 *
 * The reference program (nGIA, CUDA/signalNode) exposes its hot path as six
 * in-process C++ calls declared in CUDA/signalNode/src/func.h:72-77
 * (init, readIndex, readData, clustering, saveResult, finish) over the
 * structs Option/Index/Data/Bench (func.h:14-70).  This header replaces
 * that boundary with plain C entry points: every call returns an int status
 * (0 = ok, negative = error; text via ngia_last_error), buffers are plain
 * pointers plus sizes, and no CUDA or C++ type appears in a signature.
 *
 * Data model (identical to the makeDB database, makeDB/src/makeDB.cpp:1-16):
 *   sequences are numbered in "sorted order" (raw length descending, ties
 *   in FASTA order); record i is a run of uint32 words
 *     DNA:     [len, net, cntA, cntC, cntG, cntT, {plane0, plane1} x ceil(len/32)]
 *     protein: [len, net, cnt[28],               {plane0..plane4} x ceil(len/32)]
 *   and records are contiguous in sorted order.
 */
#ifndef NGIA_H
#define NGIA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NGIA_OK             0
#define NGIA_E_ARG         -1   /* bad argument / null pointer               */
#define NGIA_E_IO          -2   /* file missing, truncated or unreadable     */
#define NGIA_E_FORMAT      -3   /* data.bin inconsistent (type word, sizes)  */
#define NGIA_E_NOMEM       -4   /* host or device allocation failed          */
#define NGIA_E_CUDA        -5   /* CUDA runtime error                        */
#define NGIA_E_DEVICE      -6   /* device-side status (bounded wait expired) */
#define NGIA_E_STATE       -7   /* call out of order                         */
#define NGIA_E_LIMIT       -8   /* size beyond a documented maximum          */

/* Copies the calling thread's last error message (NUL-terminated) into buf.
 * Returns the status code of that error (0 if none). */
int ngia_last_error(char *buf, size_t len);

/* Library version string, e.g. "ngia-gb300 1.0". */
const char *ngia_version(void);

/* Frees any buffer this library returned through an out-pointer. */
void ngia_free(void *p);

/* ---- clustering parameters --------------------------------------------- */
typedef struct ngia_params {
    float   similarity;   /* -s : 0.1 .. 1.0                                  */
    int32_t word_length;  /* -w : DNA 4..8, protein 2..3                      */
    int32_t precise;      /* -p : 1 = skip the short-word filter              */
} ngia_params;

/* Applies the reference's parameter clamps in place for a database of the
 * given type (0 DNA, 1 protein).  Replaces the clamp block of readIndex,
 * CUDA/signalNode/src/func.cu:57-75. */
int ngia_params_clamp(int32_t type, ngia_params *p);

/* ---- database (host side) ---------------------------------------------- */
typedef struct ngia_db_view {
    int32_t         n;         /* number of sequences                          */
    int32_t         type;      /* 0 DNA, 1 protein                             */
    int32_t         longest;   /* raw length of sequence 0                     */
    int32_t         shortest;  /* raw length of sequence n-1                   */
    const uint32_t *words;     /* all records, contiguous, sorted order        */
    int64_t         n_words;
    const int64_t  *rec_off;   /* word offset of each record inside words      */
} ngia_db_view;

typedef struct ngia_db_host {
    ngia_db_view view;
    int32_t *name_len;         /* header length incl. '>' (data.bin index)     */
    int32_t *read_len;         /* raw sequence length                          */
    int64_t *fasta_off;        /* byte offset of the record's '>' in data.fasta */
    int64_t *pack_off;         /* byte offset of the record in data.bin        */
} ngia_db_host;

/* Reads <dir>/data.bin: header, index and all records into host memory.
 * Replaces readIndex + readData, CUDA/signalNode/src/func.cu:42-154. */
int ngia_db_load(const char *dir, ngia_db_host **out);

/* Packs raw sequences (given in FASTA order) into an in-memory database laid
 * out exactly as makeDB would write it: records longer than 65,536 are
 * dropped, the rest stable-sorted by raw length descending and bit-plane
 * packed (makeDB/src/makeDB.cpp:62-106, 108-252).  name_len may be NULL
 * (then every header is taken as 1 byte long and fasta_off is 0). */
int ngia_db_pack(int32_t type, const char *seq, const int64_t *seq_off,
                 int64_t n, const int32_t *name_len, ngia_db_host **out);

/* Builds <outdir>/data.bin and the <outdir>/data.fasta symlink from a FASTA
 * file; the drop-in for the makeDB tool (makeDB/src/makeDB.cpp:254-334). */
int ngia_makedb(const char *fasta_path, const char *outdir, int32_t type);

/* Writes <outdir>/cluster.txt and <outdir>/represent.fasta from a cluster
 * assignment (cluster[i] = representative of sequence i, sorted order),
 * reading names and residues from <dbdir>/data.fasta.  Replaces saveResult,
 * CUDA/signalNode/src/func.cu:680-764.  *n_clusters receives the count the
 * reference prints as "Cluster:\t<n>". */
int ngia_save_result(const char *dbdir, const char *outdir,
                     const ngia_db_host *db, const int32_t *cluster,
                     int32_t *n_clusters);

void ngia_db_free(ngia_db_host *db);

/* ---- synthetic inputs (seeded; same bytes on x86-64 and aarch64) -------- */
typedef struct ngia_synth_params {
    int32_t  type;         /* 0 DNA (ACGT), 1 protein (20 residues)            */
    int32_t  len_dist;     /* 0 normal(a,b)  1 lognormal(median a, sigma b)    */
                           /* 2 loguniform[a,b]                                */
    int64_t  n_seqs;
    int32_t  n_ancestors;
    int32_t  len_min, len_max;  /* clip range of ancestor lengths             */
    double   len_a, len_b;
    double   subst_max;    /* per-sequence substitution rate ~ U[0,subst_max] */
    double   indel_frac;   /* indel event rate = indel_frac * substitution    */
    int32_t  indel_max;    /* indel length ~ U{1..indel_max}                  */
    double   novel_frac;   /* share of sequences taken from extra ancestors   */
    uint64_t seed;
} ngia_synth_params;

/* Generates sequences in FASTA order: *seq holds all residues back to back,
 * (*seq_off)[i] .. (*seq_off)[i+1] delimits sequence i (n+1 offsets).
 * Free both with ngia_free. */
int ngia_synth_generate(const ngia_synth_params *p, char **seq,
                        int64_t **seq_off, int64_t *n);

/* Writes sequences as FASTA (headers ">s<i>", lines of `width` residues). */
int ngia_write_fasta(const char *path, const char *seq, const int64_t *seq_off,
                     int64_t n, int32_t width);

/* ---- device clustering -------------------------------------------------- */
typedef struct ngia_ctx ngia_ctx;

/* Driver forms of the greedy loop. */
#define NGIA_MODE_PLAIN  0  /* host loop: one launch sequence per representative */
#define NGIA_MODE_GRAPH  1  /* device-side driver in a captured CUDA graph
                               (conditional while node), no host round trip  */
#define NGIA_MODE_SPEC   2  /* speculative rounds once the unclustered set is
                               small (<= 32,768 sequences, K x unclustered <=
                               2^20 pairs, 2 <= K <= 64): the next K are
                               candidate representatives of one round, every
                               pair against them runs at once and the greedy
                               order is replayed on the device (same result as
                               the one-representative loop); host loop per
                               round.  While the set is larger, iterations of
                               the captured loop (as NGIA_MODE_GRAPH, 8 between
                               looks at the set), and only those when the
                               database has records of net length < 16,
                               precise is 0 and more than 16,384 sequences
                               (the reference's short-word kernel then makes a
                               pair's test depend on its iteration's job
                               list).                                         */

typedef struct ngia_stats {
    int64_t iterations;    /* representatives taken (= clusters)             */
    int64_t candidates;    /* (representative, candidate) visits             */
    int64_t base_pass;     /* visits passing the composition filter          */
    int64_t align_pairs;   /* pairs entering the alignment stage             */
    int64_t members;       /* pairs accepted (incl. each representative)     */
    int64_t band_cells;    /* reference band cells of the alignment pairs    */
    int64_t filter_bytes;  /* algorithmic filter bytes (headers + planes)    */
    int64_t word_checks;   /* pairs the short-word filter was evaluated on   */
    int64_t done_cells;    /* in-band cells the alignment kernels computed   */
                           /* (fewer than band_cells: early rejection)       */
    double  ms_filter;     /* device time of the filter launches and         */
    double  ms_align;      /* of the alignment launches (profiling, plain)   */
    int64_t class_pairs[8];   /* pairs queued per alignment work class       */
    double  class_ms[8];      /* device time per class (profiling, plain)    */
    int64_t class_cells[8];   /* in-band cells computed per class            */
    int64_t class_bytes[8];   /* query plane bytes of the pairs per class    */
} ngia_stats;

/* Copies the database to the device (one host-to-device transfer) and
 * builds the per-sequence header arrays.  Replaces the device half of
 * readData, CUDA/signalNode/src/func.cu:104-154.  The caller keeps
 * ownership of the host buffers. */
int ngia_open(const ngia_db_view *db, ngia_ctx **out);

/* Full greedy clustering.  Replaces clustering(),
 * CUDA/signalNode/src/func.cu:607-677.  cluster_out[n] receives the
 * representative (sorted index) of every sequence; identity_out[n] (may be
 * NULL) the banded-LCS score each member reached against its representative
 * (-1 for a representative that failed its own tests).  stats may be NULL. */
int ngia_cluster(ngia_ctx *ctx, const ngia_params *p, int32_t mode,
                 int32_t *cluster_out, int32_t *identity_out,
                 ngia_stats *stats);

/* Stepwise form of ngia_cluster for benchmarking and checkpointing:
 * begin resets the state; step runs up to max_iters representatives
 * (all remaining if max_iters <= 0) and reports *done; end copies results. */
int ngia_cluster_begin(ngia_ctx *ctx, const ngia_params *p, int32_t mode);
int ngia_cluster_step(ngia_ctx *ctx, int64_t max_iters, int32_t *done);
int ngia_cluster_end(ngia_ctx *ctx, int32_t *cluster_out,
                     int32_t *identity_out, ngia_stats *stats);

/* Current statistics of the run started by ngia_cluster_begin, without
 * copying the assignment arrays. */
int ngia_cluster_stats(ngia_ctx *ctx, ngia_stats *stats);

/* Device time (CUDA events on the context stream) of the last
 * ngia_cluster_step call. */
int ngia_step_device_ms(ngia_ctx *ctx, float *ms);

/* 1 = time every stage launch with CUDA events (plain driver form only; the
 * totals land in ngia_stats.ms_filter / ms_align). */
int ngia_set_profiling(ngia_ctx *ctx, int32_t on);

/* ---- batches of independent jobs ---------------------------------------- */
typedef struct ngia_batch ngia_batch;

/* Opens n_jobs independent clustering jobs (one database view each; each is
 * copied to the device with grids sized to the job). */
int ngia_batch_open(const ngia_db_view *jobs, int32_t n_jobs, ngia_batch **out);

/* Batch-only driver form: the jobs of one record type advance together, one
 * representative each per round, and every stage of a round is one launch
 * over all of them (cross-job work queues per length bucket). */
#define NGIA_MODE_POOL   3

/* Clusters every job with its own parameters (params[j], clamped).
 * NGIA_MODE_GRAPH: the whole batch is one launch of one CUDA graph holding
 * one conditional while node per job, side by side, so jobs run
 * concurrently with no host round trip per representative;
 * NGIA_MODE_POOL: one launch of one CUDA graph holding one while node per
 * record type: each round prepares every job's representative, filters the
 * unclustered sequences of all jobs in one launch into each job's length
 * buckets (alignment classes), and aligns each bucket across all jobs in one
 * persistent launch whose CTAs claim chunks of pairs from any job and stage
 * that job's representative in shared memory.  A job whose database has
 * records of net length < 16 while precise is 0 keeps its own while node
 * (the reference's word kernel then depends on job positions, func.cu:375);
 * at most 8,192 jobs of one record type (NGIA_E_LIMIT beyond);
 * NGIA_MODE_SPEC: every job's speculative-round driver (as ngia_cluster in
 * that mode), the jobs taken in turn by host worker threads
 * (NGIA_BATCH_WORKERS, default 16), each job on its own stream, so one
 * job's host round trips overlap the other jobs' GPU work;
 * NGIA_MODE_PLAIN: the jobs one after the other with the host-loop driver.
 * No reference counterpart (the reference clusters one database per run,
 * cluster.cpp:4-17).
 * max_iters > 0 stops each job after that many representatives (sampling).
 * cluster_out[j] / identity_out[j] (either may be NULL) receive job j's
 * arrays (jobs[j].n entries); stats (may be NULL) the sums over jobs.
 * Results are identical to clustering every job alone. */
int ngia_batch_run(ngia_batch *b, const ngia_params *params, int32_t mode,
                   int64_t max_iters, int32_t **cluster_out,
                   int32_t **identity_out, ngia_stats *stats);

int ngia_batch_close(ngia_batch *b);

/* ---- serving: continuous batching against a resident representative set --
 * No counterpart in the reference (its program clusters one database per
 * run); the per-pair tests and thresholds are those of ngia_cluster.
 * ngia_serve_open keeps a representative set resident on the GPU (records
 * plus one k-mer bitset per representative).  Each submitted batch (a
 * database of queries of the same type, in makeDB layout) is assigned
 * against it: query q joins the first representative r, in the order of
 * `reps` (their creation order), whose pair (r as representative, q as
 * candidate) passes the composition test, the short-word test (when precise
 * is 0 and both net lengths are >= 16) and the banded-LCS test:
 * rep_out[q] = r, ident_out[q] = the banded-LCS score.  The queries no
 * resident representative takes are then clustered among themselves exactly
 * as ngia_cluster clusters a database holding only them: rep_out[q] = -1 - j,
 * j = the batch index of q's new representative (ident_out[j] = -1).  The
 * resident set never changes, so a batch's result does not depend on the
 * batches around it.
 *
 * Batches run on `slots` workers side by side on the GPU, each with its own
 * stream and device memory for batches of up to max_batch records,
 * max_batch_words record words and records of max_record_blocks plane
 * blocks (32 residues each).  A submitted batch waits in a FIFO until a
 * slot is free; the slot count is capped so that all slots fit
 * memory_budget bytes of device memory. */
typedef struct ngia_server ngia_server;

typedef struct ngia_serve_config {
    int32_t slots;              /* workers (0 = 4)                              */
    int32_t max_batch;          /* records per batch (0 = 4,096)                */
    int32_t max_record_blocks;  /* plane blocks per query record (0 = 128)      */
    int32_t reserved;
    int64_t max_batch_words;    /* record words per batch (0 = max_batch x the  */
                                /* words of a record of max_record_blocks)      */
    int64_t memory_budget;      /* device bytes for all slots (0 = half free)   */
} ngia_serve_config;

typedef struct ngia_serve_result {
    int32_t done;        /* 1 when the batch is finished (results written)      */
    int32_t slot;        /* worker that ran it                                  */
    int32_t rounds;      /* assignment rounds (chunks of representatives)       */
    int32_t resident;    /* queries that joined a resident representative       */
    int32_t new_reps;    /* representatives created among the leftovers         */
    int32_t reserved;
    double  queued_ms;   /* submit -> start on a slot                           */
    double  run_ms;      /* start on a slot -> finished                         */
    int64_t pairs;       /* (representative, query) pairs aligned in assignment */
    int64_t cells;       /* in-band cells those alignments computed             */
} ngia_serve_result;

/* Opens the service on the current device; params are clamped
 * (ngia_params_clamp) and apply to every batch. */
int ngia_serve_open(const ngia_db_view *reps, const ngia_params *params,
                    const ngia_serve_config *cfg, ngia_server **out);

/* Number of slots (batches that can run at the same time). */
int ngia_serve_slots(const ngia_server *s, int32_t *slots);

/* Queues a batch (copied; the caller may free it on return) and returns its
 * ticket.  NGIA_E_LIMIT when the batch exceeds a slot's capacity. */
int ngia_serve_submit(ngia_server *s, const ngia_db_view *batch, int64_t *ticket);

/* Looks at a ticket, waiting up to wait_ms milliseconds for it (0 = do not
 * wait, < 0 = until done).  When the batch is done: rep_out / ident_out
 * (batch.n entries each, either may be NULL) receive the results, res->done
 * is 1 and the ticket is released; otherwise res->done is 0.  A batch that
 * failed returns its error code (and releases the ticket). */
int ngia_serve_poll(ngia_server *s, int64_t ticket, int32_t wait_ms, int32_t *rep_out,
                    int32_t *ident_out, ngia_serve_result *res);

/* Finishes the queued and running batches, then frees the service. */
int ngia_serve_close(ngia_server *s);

/* Per-pair stage values for (rep, cands[k]) pairs, for unit-level parity:
 * out[4k+0] = composition sum, out[4k+1] = short-word count (-1 when the
 * reference skips it because a net length is < 16), out[4k+2] = banded-LCS
 * score, out[4k+3] = block band.  Mirrors the per-job bodies of the six
 * reference kernels, CUDA/signalNode/src/func.cu:323-604. */
int ngia_pair_scores(ngia_ctx *ctx, const ngia_params *p, int32_t rep,
                     const int32_t *cands, int32_t n, int32_t *out);

/* Number of CUDA devices visible to the process (0 when there is none). */
int ngia_device_count(int32_t *count);

/* Selects the CUDA device for contexts opened later by the calling thread. */
int ngia_set_device(int32_t device);

/* Page-locks / releases a caller buffer so host<->device copies of it run at
 * full link speed (e.g. the database words before ngia_open). */
int ngia_pin_host(void *ptr, size_t bytes);
int ngia_unpin_host(void *ptr);

/* Measures the INT32 logic/add issue rate of the current device with an
 * instruction-mix probe (three LOP3 and one IADD3 per step, the mix of the
 * alignment inner loop); *gops receives lane-operations per second / 1e9. */
int ngia_measure_int_peak(double *gops);

/* The floor under the composition filter's time on an open, begun DNA
 * context: *launch_us = the mean device time of an empty kernel launched
 * with the filter's grid, *read_us = the mean time of a kernel with the same
 * grid that only reads what the filter reads for the current unclustered set
 * (each warp's bitmap words, then length and counts of every unclustered
 * sequence in them).  The run state is not changed.  No reference
 * counterpart: it bounds kernel_baseFilterGen (func.cu:323-338) from below. */
int ngia_measure_filter_floor(ngia_ctx *ctx, double *launch_us, double *read_us);

/* Banded-LCS scores of the representative record at d_words + rep_off
 * against the n query records at d_words + d_query_off[k], written to
 * d_scores[k]; all three arrays are device memory the caller owns, and the
 * call allocates nothing.  It has no counterpart in the reference: it is for
 * callers that cannot allocate device memory — applications whose device
 * memory is owned by another allocator or pool, or loops that must not pay
 * for cudaMalloc/cudaFree.  Working rows live in a fixed 4 MiB device array
 * of this library (held by every GPU that loads it until the process exits),
 * which limits the representative to 65,536 residues (NGIA_E_LIMIT beyond).
 * The first call on a device looks the array up and must precede any stream
 * capture; the address is kept for the life of the process, so do not call
 * this across a cudaDeviceReset of that device.  Calls that overlap on the
 * GPU share the array and race — serialise them.  Each call first reads the
 * representative's two header words back to the host (to size its grid), so
 * it waits until `stream` (NULL = default stream) has reached that point;
 * the kernel is then queued on `stream` and the scores are ready when it
 * completes. */
int ngia_rep_scores_noalloc(const uint32_t *d_words, int64_t rep_off,
                            const int64_t *d_query_off, int32_t n, int32_t type,
                            float similarity, int32_t *d_scores, void *stream);

/* Checkpoint of a run in progress (after ngia_cluster_begin / _step): the
 * run state, the unclustered set, the assignment and scores, and the
 * parameters, written to `path` (via a temporary file, then renamed).  No
 * counterpart in the reference.  ngia_cluster_resume continues such a run in
 * a context holding the same database (checked by record count, word count
 * and a hash of the records; NGIA_E_FORMAT for another database or a damaged
 * file), with either driver; the run then ends exactly as if uninterrupted. */
int ngia_cluster_save(ngia_ctx *ctx, const char *path);
int ngia_cluster_resume(ngia_ctx *ctx, const char *path, int32_t mode);

/* Run-time tuning (no counterpart in the reference).  These settings change
 * the speed of a run, never its result: the order of the two cheap tests
 * (short-word test before or after the alignment), the number of idle lanes
 * a warp of the tiled alignment waits for before it claims new pairs, the
 * pair count up to which a class is aligned warp-per-pair, and per length
 * bucket (alignment class: pairs grouped by band window) its own
 * warp-per-pair cut-off and CTA count, and the composition filter's tile.
 * ngia_autotune times candidate settings on the first `iters` greedy
 * iterations of a fresh run of this context's database (graph driver, device
 * time), keeps the fastest for later runs of the context and reports it;
 * the result is cached in the process by database shape (type, record
 * count and longest record, each rounded to a power of two) and parameters,
 * and a later ngia_autotune with the same key applies it without timing
 * (cached = 1).  ngia_set_tuning applies settings found before. */
typedef struct ngia_tuning {
    int32_t word_order;   /* 0 by similarity, 1 short words first, 2 alignment first */
    int32_t refill;       /* 1..32 idle lanes                                        */
    int32_t warp_pairs;   /* warp-per-pair up to this many pairs; -1 = default      */
    int32_t candidates;   /* settings timed (ngia_autotune)                          */
    double  ms_per_iter;  /* device time per iteration of the chosen setting         */
    double  default_ms_per_iter;  /* the same for the default setting                */
    int32_t class_warp_pairs[8];  /* per length bucket: its warp-per-pair cut-off,   */
                                  /* -1 = warp_pairs                                 */
    int32_t class_grid_div[8];    /* per length bucket: its CTAs divided by 1 or 2   */
    int32_t filter_tile;          /* composition filter: bitmap words per warp and   */
                                  /* tile, 8 (default) or 1                          */
    int32_t cached;               /* 1: applied from the tuning cache, not timed     */
} ngia_tuning;
int ngia_autotune(ngia_ctx *ctx, const ngia_params *p, int32_t iters, ngia_tuning *out);
int ngia_set_tuning(ngia_ctx *ctx, const ngia_tuning *t);

/* Chooses the settings the batch's NGIA_MODE_GRAPH runs (one greedy loop
 * per job, side by side) give their jobs, by timing three policies on the
 * whole batch over the first `iters` greedy iterations of every job:
 *   NGIA_BATCH_POLICY_THREAD  every length bucket of every job aligned
 *                             thread per pair (the untuned batch default);
 *   NGIA_BATCH_POLICY_CUTOFF  each job's default warp-per-pair cut-off;
 *   NGIA_BATCH_POLICY_TUNED   each job's own ngia_autotune settings, found
 *                             with the job alone on the GPU (cached by
 *                             database shape and parameters).
 * The thread-per-pair policy stays unless another is at least 2% faster.
 * Later NGIA_MODE_GRAPH runs apply the chosen policy; out[j] (may be NULL)
 * receives job j's settings under it (candidates = 3, ms_per_iter and
 * default_ms_per_iter the batch's wall time per iteration under the chosen
 * and the thread-per-pair policy).  Results never change.  No reference
 * counterpart. */
#define NGIA_BATCH_POLICY_THREAD 0
#define NGIA_BATCH_POLICY_CUTOFF 1
#define NGIA_BATCH_POLICY_TUNED  2
int ngia_batch_autotune(ngia_batch *b, const ngia_params *params, int32_t iters, ngia_tuning *out);
/* Applies a policy without timing (NGIA_BATCH_POLICY_TUNED only after
 * ngia_batch_autotune, NGIA_E_STATE before); ngia_batch_policy reports the
 * policy in force (-1 before either call). */
int ngia_batch_set_policy(ngia_batch *b, int32_t policy);
int ngia_batch_policy(const ngia_batch *b, int32_t *policy);

/* Loads another database into an open context, reusing its device memory
 * (one host-to-device copy of the records and offsets, then the header
 * arrays are rebuilt on the device).  The database must fit what the context
 * was opened with: at most as many records and words, records of at most as
 * many plane blocks (NGIA_E_LIMIT otherwise); same sequence type.  A run in
 * progress ends; a captured graph is kept when the new database has the same
 * record count, longest record and short-record flag. */
int ngia_reload(ngia_ctx *ctx, const ngia_db_view *db);

/* CUDA stream the context launches on (as an opaque handle, for timing). */
void *ngia_stream(ngia_ctx *ctx);

int ngia_close(ngia_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* NGIA_H */
