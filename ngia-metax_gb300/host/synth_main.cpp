// synth_main.cpp — writes a seeded synthetic FASTA file.
//   ngia_synth -o out.fasta -t 0|1 -n seqs -a ancestors -d dist -A a -B b
//              -m min -M max -r subst_max -x indel_max -f novel_frac -S seed
// dist: 0 normal(A,B), 1 lognormal(median A, sigma B), 2 loguniform[A,B].
#include <cstdio>

#include "../../include/ngia.h"
#include "cli_args.h"

int main(int argc, char **argv) {
  ngia::Cli cli({{"output", 'o', "output FASTA path", true, ""},
                 {"type", 't', "0 DNA, 1 protein", false, ""},
                 {"seqs", 'n', "number of sequences", true, ""},
                 {"ancestors", 'a', "number of ancestors", true, ""},
                 {"dist", 'd', "length distribution 0/1/2", false, ""},
                 {"lena", 'A', "length parameter a", false, ""},
                 {"lenb", 'B', "length parameter b", false, ""},
                 {"min", 'm', "minimum ancestor length", false, ""},
                 {"max", 'M', "maximum ancestor length", false, ""},
                 {"subst", 'r', "maximum substitution rate", false, ""},
                 {"indel", 'x', "maximum indel length", false, ""},
                 {"novel", 'f', "novel-ancestor fraction", false, ""},
                 {"width", 'W', "FASTA line width", false, ""},
                 {"seed", 'S', "random seed", false, ""}});
  cli.parse_check(argc, argv);
  ngia_synth_params p{};
  p.type = cli.num<int>("type", 0);
  p.n_seqs = cli.num<long long>("seqs", 0);
  p.n_ancestors = cli.num<int>("ancestors", 1);
  p.len_dist = cli.num<int>("dist", 0);
  p.len_a = cli.num<double>("lena", 1450.0);
  p.len_b = cli.num<double>("lenb", 80.0);
  p.len_min = cli.num<int>("min", 1200);
  p.len_max = cli.num<int>("max", 1700);
  p.subst_max = cli.num<double>("subst", 0.20);
  p.indel_frac = 0.05;
  p.indel_max = cli.num<int>("indel", 3);
  p.novel_frac = cli.num<double>("novel", 0.0);
  p.seed = cli.num<unsigned long long>("seed", 1);
  char *seq = nullptr;
  int64_t *off = nullptr, n = 0;
  int rc = ngia_synth_generate(&p, &seq, &off, &n);
  if (!rc) rc = ngia_write_fasta(cli.str("output").c_str(), seq, off, n, cli.num<int>("width", 80));
  ngia_free(seq);
  ngia_free(off);
  if (rc) {
    char msg[512];
    ngia_last_error(msg, sizeof(msg));
    std::fprintf(stderr, "ngia_synth failed (%d): %s\n", rc, msg);
    return 2;
  }
  return 0;
}
