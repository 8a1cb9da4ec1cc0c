// cluster_main.cpp — drop-in replacement for the reference `cluster` program
// (CUDA/signalNode/src/cluster.cpp:4-17):
//   cluster -i <dbdir> -o <outdir> -w <word> -s <similarity> [-p 0|1]
// reads <dbdir>/data.bin + data.fasta, clusters on the GPU through the C ABI
// and writes <outdir>/cluster.txt and <outdir>/represent.fasta.
// Environment: NGIA_MODE=spec|graph|plain (default spec: plain iterations
// while the unclustered set is large, speculative rounds once it is small)
// selects the driver form;
// NGIA_IDENTITY=<path> also writes "index<TAB>representative<TAB>score" lines.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include "../../include/ngia.h"
#include "cli_args.h"

namespace {

struct Timer {  // "<s> seconds." like the reference timer (timer.h:49-52)
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  void print() const {
    std::chrono::duration<double> d = std::chrono::steady_clock::now() - t0;
    std::cout << d.count() << " seconds." << std::endl;
  }
};

[[noreturn]] void die(const char *what, int rc) {
  char msg[512];
  ngia_last_error(msg, sizeof(msg));
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, msg);
  std::exit(2);
}

}  // namespace

int main(int argc, char **argv) {
  Timer total;
  ngia::Cli cli({{"input", 'i', "input directory", true, ""},
                 {"output", 'o', "output directory", true, ""},
                 {"word", 'w', "word length gene:4-8, protein:2-3", true, ""},
                 {"precise", 'p', "precise mode 0 or 1", false, ""},
                 {"similarity", 's', "similarity 0.1-1.0", true, ""}});
  cli.parse_check(argc, argv);
  const std::string in = cli.str("input"), out = cli.str("output");
  ngia_params p;
  p.word_length = cli.num<int>("word", 0);
  p.precise = cli.num<int>("precise", 0);
  p.similarity = cli.num<float>("similarity", 0.95f);

  Timer tread;
  ngia_db_host *db = nullptr;
  int rc = ngia_db_load(in.c_str(), &db);
  if (rc) die("reading data.bin", rc);
  ngia_params_clamp(db->view.type, &p);
  const char *types[2] = {"Gene", "Protein"};
  std::cout << "Data type:\t" << types[db->view.type] << "\n";
  std::cout << "Similarity:\t" << p.similarity << "\n";
  std::cout << "Word length:\t" << p.word_length << "\n";
  std::cout << "Precise mode:\t" << p.precise << "\n";
  std::cout << "Threads:\t" << 1 << "\n";
  std::cout << "Reads count:\t" << db->view.n << std::endl;
  std::cout << "Longest:\t" << db->view.longest << std::endl;
  std::cout << "Shortest:\t" << db->view.shortest << std::endl;
  std::cout << "Reads/thread:\t" << db->view.n << std::endl;
  std::cout << std::endl;
  std::cout << "Read data:\t";
  tread.print();
  std::cout << std::endl;

  int mode = NGIA_MODE_SPEC;
  if (const char *m = std::getenv("NGIA_MODE")) {
    if (!std::strcmp(m, "plain")) mode = NGIA_MODE_PLAIN;
    if (!std::strcmp(m, "graph")) mode = NGIA_MODE_GRAPH;
  }
  ngia_ctx *ctx = nullptr;
  rc = ngia_open(&db->view, &ctx);
  if (rc) die("ngia_open", rc);
  std::vector<int32_t> cluster((size_t)db->view.n), ident((size_t)db->view.n);
  // NGIA_CHECKPOINT=<file>: resume from the file when it exists and save the
  // run to it every NGIA_CHECKPOINT_EVERY representatives (default 10,000)
  const char *ck = std::getenv("NGIA_CHECKPOINT");
  if (!ck || !*ck) {
    rc = ngia_cluster(ctx, &p, mode, cluster.data(), ident.data(), nullptr);
    if (rc) die("ngia_cluster", rc);
  } else {
    int64_t every = 10000;
    if (const char *e = std::getenv("NGIA_CHECKPOINT_EVERY")) every = std::max<int64_t>(1, std::atoll(e));
    FILE *probe = std::fopen(ck, "rb");
    if (probe) {
      std::fclose(probe);
      rc = ngia_cluster_resume(ctx, ck, mode);
      if (rc) die("resuming the checkpoint", rc);
    } else {
      rc = ngia_cluster_begin(ctx, &p, mode);
      if (rc) die("ngia_cluster_begin", rc);
    }
    for (int32_t done = 0; !done;) {
      rc = ngia_cluster_step(ctx, every, &done);
      if (rc) die("ngia_cluster_step", rc);
      if (!done && (rc = ngia_cluster_save(ctx, ck))) die("saving the checkpoint", rc);
    }
    rc = ngia_cluster_end(ctx, cluster.data(), ident.data(), nullptr);
    if (rc) die("ngia_cluster_end", rc);
  }
  ngia_close(ctx);
  std::cout << "\r" << db->view.n << "/" << db->view.n << "\n" << std::endl;

  Timer tsave;
  int32_t nc = 0;
  rc = ngia_save_result(in.c_str(), out.c_str(), db, cluster.data(), &nc);
  if (rc) die("writing results", rc);
  std::cout << "Cluster:\t" << nc << std::endl;
  if (const char *ip = std::getenv("NGIA_IDENTITY")) {
    FILE *f = std::fopen(ip, "w");
    if (!f) die("writing identity file", NGIA_E_IO);
    for (int32_t i = 0; i < db->view.n; i++) std::fprintf(f, "%d\t%d\t%d\n", i, cluster[(size_t)i], ident[(size_t)i]);
    std::fclose(f);
  }
  std::cout << "Save result:\t";
  tsave.print();
  ngia_db_free(db);
  total.print();
  return 0;
}
