// makedb_main.cpp — drop-in replacement for the reference makeDB tool
// (makeDB/src/makeDB.cpp:336-346):  makeDB -i <fasta> -o <outdir> -t 0|1
// writes <outdir>/data.bin and the <outdir>/data.fasta symlink.
#include <chrono>
#include <cstdio>
#include <iostream>

#include "../../include/ngia.h"
#include "cli_args.h"

int main(int argc, char **argv) {
  auto t0 = std::chrono::steady_clock::now();
  ngia::Cli cli({{"input", 'i', "input file", true, ""},
                 {"output", 'o', "output directory", true, ""},
                 {"type", 't', "input type 0:gene 1:protein", true, ""}});
  cli.parse_check(argc, argv);
  const int type = cli.num<int>("type", 0);
  if (type < 0 || type > 1) {
    std::cout << "t: 0-1\n";
    return 0;
  }
  int rc = ngia_makedb(cli.str("input").c_str(), cli.str("output").c_str(), type);
  if (rc) {
    char msg[512];
    ngia_last_error(msg, sizeof(msg));
    std::fprintf(stderr, "makeDB failed (%d): %s\n", rc, msg);
    return 2;
  }
  std::chrono::duration<double> d = std::chrono::steady_clock::now() - t0;
  std::cout << "Make data base total:\t" << d.count() << " seconds." << std::endl;
  return 0;
}
