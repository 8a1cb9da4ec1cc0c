/*
 * ngia_oracle.h — CPU restatement of nGIA's single-node clustering
 * (CUDA/signalNode/src/func.cu) used as the parity reference of the tests
 * and the timed CPU baseline.  TEST INFRASTRUCTURE ONLY: the product library
 * never links, loads or calls it.
 */
#ifndef NGIA_ORACLE_H
#define NGIA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_db {
  int32_t n, longest, shortest, type;
  int32_t *name_len, *read_len;
  int64_t *fasta_off, *pack_off;
  int64_t *offsets;   /* word offset of record i in buf (func.cu:117-124) */
  uint32_t *buf;      /* records                                          */
  int64_t buf_words;
} ora_db;

/* stats[] slots filled by ora_cluster */
enum {
  ORA_ITER = 0,      /* representatives                                   */
  ORA_CAND,          /* (rep, candidate) visits = base-filter jobs        */
  ORA_BASE_PASS,     /* base-filter survivors                             */
  ORA_WORD_EVAL,     /* word-filter jobs that were evaluated (not skipped) */
  ORA_WORD_PASS,     /* word-filter survivors = alignment jobs            */
  ORA_MEMBERS,       /* alignment survivors (members incl. reps)          */
  ORA_CELLS,         /* band cells of the alignment jobs                  */
  ORA_FILTER_BYTES,  /* header bytes of every job + planes of word jobs   */
  ORA_NSTATS
};

int  ora_load(const char *dir, ora_db *db);
void ora_free(ora_db *db);
void ora_clamp(int type, float *s, int *w, int *precise);

/* Greedy clustering of func.cu:607-677.  cluster[n], identity[n] out;
 * stats[ORA_NSTATS] out (may be NULL).  max_iters > 0 stops after that many
 * representatives (cluster[] then holds -1 for unassigned sequences).
 * nthreads <= 0 uses all OpenMP threads.  Returns the iteration count. */
int64_t ora_cluster(const uint32_t *buf, const int64_t *offsets, int n, int type,
                    float s, int w, int precise, int nthreads, int64_t max_iters,
                    int32_t *cluster, int32_t *identity, int64_t *stats);

/* Per-pair stage values (rep, cand): out[0] composition sum, out[1]
 * short-word count (-1 if a net length < 16 skips the filter), out[2]
 * banded-LCS score, out[3] block band; out[4..6] = pass flags of the three
 * stages; out[7] = band cells. */
void ora_pair(const uint32_t *buf, const int64_t *offsets, int type, float s, int w,
              int rep, int cand, int32_t *out);

/* The reference's per-pair alignment on raw records (rep, query). */
int ora_dp_sum(const uint32_t *rep, const uint32_t *query, int type, float s,
               int *band, int64_t *cells);

/* Serving (no counterpart in the reference; defined by this project from
 * the reference's per-pair tests): query q of a batch joins the first
 * resident representative r (in the order given, i.e. creation order) whose
 * pair passes the composition test, the short-word test (when precise == 0
 * and both net lengths are >= 16) and the banded-LCS test of func.cu with r
 * as the representative; rep_out[q] = r, ident_out[q] = its banded-LCS
 * score.  Queries no resident representative takes are clustered among
 * themselves by ora_cluster over the leftover records in batch order:
 * rep_out[q] = -1 - j where j is the batch index of q's new representative
 * (j = q for the representative itself, whose ident_out is -1).  Returns
 * the number of new representatives. */
int64_t ora_assign(const uint32_t *rbuf, const int64_t *roff, int nrep, const uint32_t *qbuf,
                   const int64_t *qoff, int nq, int type, float s, int w, int precise, int nthreads,
                   int32_t *rep_out, int32_t *ident_out);

/* makeDB's records (makeDB/src/makeDB.cpp:62-106, 108-252) from raw
 * sequences given in FASTA order (seq[off[i] .. off[i+1])): records longer
 * than 65,536 residues are dropped, the rest stable-sorted by raw length,
 * longest first, and packed.  Called with words == NULL it only returns the
 * record count and word count (*n_words); then again with words[n_words]
 * and rec_off[count] to fill them.  Returns the record count. */
int64_t ora_pack(int type, const char *seq, const int64_t *off, int64_t n, uint32_t *words,
                 int64_t *rec_off, int64_t *n_words);

/* saveResult (func.cu:680-764): writes cluster.txt and represent.fasta. */
int ora_save(const char *dbdir, const char *outdir, const ora_db *db, const int32_t *cluster,
             int32_t *n_clusters);

#ifdef __cplusplus
}
#endif
#endif
