/*
 * oracle_main.c — command-line front end of the CPU oracle (test
 * infrastructure).  Same flags as the reference `cluster` program
 * (-i dbdir -o outdir -w word -s similarity [-p 0|1]) plus
 *   -t threads      OpenMP threads (default: all)
 *   -m max_iters    stop after this many representatives (0 = all)
 *   -r rawdir       also write cluster.i32 / identity.i32 / stats.json there
 * Writes cluster.txt and represent.fasta to outdir (skipped if outdir is "-").
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ngia_oracle.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
  const char *in = NULL, *out = NULL, *raw = NULL;
  int w = 0, precise = 0, threads = 0, have_w = 0, have_s = 0;
  float s = 0.95f;
  long long max_iters = 0;
  for (int i = 1; i + 1 < argc; i += 2) {
    if (!strcmp(argv[i], "-i")) in = argv[i + 1];
    else if (!strcmp(argv[i], "-o")) out = argv[i + 1];
    else if (!strcmp(argv[i], "-w")) { w = atoi(argv[i + 1]); have_w = 1; }
    else if (!strcmp(argv[i], "-s")) { s = strtof(argv[i + 1], NULL); have_s = 1; }
    else if (!strcmp(argv[i], "-p")) precise = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "-t")) threads = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "-m")) max_iters = atoll(argv[i + 1]);
    else if (!strcmp(argv[i], "-r")) raw = argv[i + 1];
    else { fprintf(stderr, "unknown option %s\n", argv[i]); return 1; }
  }
  if (!in || !out || !have_w || !have_s) {
    fprintf(stderr, "usage: %s -i dbdir -o outdir -w word -s similarity [-p 0|1] [-t threads] [-m iters] [-r rawdir]\n", argv[0]);
    return 1;
  }
  ora_db db;
  int rc = ora_load(in, &db);
  if (rc) { fprintf(stderr, "cannot load %s/data.bin (%d)\n", in, rc); return 2; }
  ora_clamp(db.type, &s, &w, &precise);
  int32_t *cluster = (int32_t *)malloc(4 * (size_t)db.n), *ident = (int32_t *)malloc(4 * (size_t)db.n);
  int64_t st[ORA_NSTATS];
  double t0 = now_s();
  ora_cluster(db.buf, db.offsets, db.n, db.type, s, w, precise, threads, max_iters, cluster, ident, st);
  double t1 = now_s();
  int32_t nc = 0;
  if (strcmp(out, "-") != 0 && max_iters <= 0) {
    if (ora_save(in, out, &db, cluster, &nc)) { fprintf(stderr, "cannot write results to %s\n", out); return 3; }
  }
  if (raw) {
    char p[4096];
    snprintf(p, sizeof(p), "%s/cluster.i32", raw);
    FILE *f = fopen(p, "wb");
    if (f) { fwrite(cluster, 4, (size_t)db.n, f); fclose(f); }
    snprintf(p, sizeof(p), "%s/identity.i32", raw);
    f = fopen(p, "wb");
    if (f) { fwrite(ident, 4, (size_t)db.n, f); fclose(f); }
    snprintf(p, sizeof(p), "%s/stats.json", raw);
    f = fopen(p, "w");
    if (f) {
      fprintf(f, "{\"seconds\": %.6f, \"iterations\": %lld, \"candidates\": %lld, \"base_pass\": %lld, "
                 "\"word_eval\": %lld, \"word_pass\": %lld, \"members\": %lld, \"cells\": %lld, "
                 "\"filter_bytes\": %lld, \"s\": %.9g, \"w\": %d, \"precise\": %d}\n",
              t1 - t0, (long long)st[ORA_ITER], (long long)st[ORA_CAND], (long long)st[ORA_BASE_PASS],
              (long long)st[ORA_WORD_EVAL], (long long)st[ORA_WORD_PASS], (long long)st[ORA_MEMBERS],
              (long long)st[ORA_CELLS], (long long)st[ORA_FILTER_BYTES], (double)s, w, precise);
      fclose(f);
    }
  }
  printf("Cluster:\t%d\n", nc);
  printf("%g seconds.\n", t1 - t0);
  free(cluster);
  free(ident);
  ora_free(&db);
  return 0;
}
