// cli_args.h — small option parser with the semantics of the cmdline.h
// parser the reference tools use (CUDA/signalNode/src/cmdline.h:440-600):
// "-x value", "--name=value", "--name value"; values converted with
// istringstream and rejected unless fully consumed; missing required options
// or bad values print the usage to stderr and exit(1); no arguments or
// --help / -? print the usage and exit(0).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace ngia {

struct CliOpt {
  std::string name;
  char short_name;
  std::string desc;
  bool required;
  std::string value;
  bool set = false;
};

class Cli {
 public:
  explicit Cli(std::vector<CliOpt> opts) : opts_(std::move(opts)) {
    opts_.push_back({"help", '?', "print this message", false, "", false});
  }

  void parse_check(int argc, char **argv) {
    prog_ = argv[0];
    std::vector<std::string> errs;
    bool help = false;
    for (int i = 1; i < argc; i++) {
      std::string a = argv[i];
      CliOpt *o = nullptr;
      std::string val;
      bool has_val = false;
      if (a.rfind("--", 0) == 0) {
        std::string n = a.substr(2);
        size_t eq = n.find('=');
        if (eq != std::string::npos) {
          val = n.substr(eq + 1);
          n = n.substr(0, eq);
          has_val = true;
        }
        o = find(n);
        if (!o) {
          errs.push_back("undefined option: --" + n);
          continue;
        }
      } else if (a.size() >= 2 && a[0] == '-') {
        o = find(a.back());
        if (!o) {
          errs.push_back(std::string("undefined short option: -") + a.back());
          continue;
        }
      } else {
        continue;  // positional arguments are ignored
      }
      if (o->name == "help") {
        help = true;
        continue;
      }
      if (!has_val) {
        if (i + 1 >= argc) {
          errs.push_back("option needs value: --" + o->name);
          continue;
        }
        val = argv[++i];
      }
      o->value = val;
      o->set = true;
    }
    for (auto &o : opts_)
      if (o.required && !o.set) errs.push_back("need option: --" + o.name);
    if ((argc == 1 && !errs.empty()) || help) {
      std::fputs(usage().c_str(), stderr);
      std::exit(0);
    }
    if (!errs.empty()) {
      std::fprintf(stderr, "%s\n%s", errs[0].c_str(), usage().c_str());
      std::exit(1);
    }
  }

  std::string str(const std::string &n) const { return get(n)->value; }
  template <class T>
  T num(const std::string &n, T def) const {
    const CliOpt *o = get(n);
    if (!o->set) return def;
    std::istringstream ss(o->value);
    T v;
    if (!(ss >> v && ss.eof())) {
      std::fprintf(stderr, "option value is invalid: --%s=%s\n%s", n.c_str(), o->value.c_str(), usage().c_str());
      std::exit(1);
    }
    return v;
  }

 private:
  CliOpt *find(const std::string &n) {
    for (auto &o : opts_)
      if (o.name == n) return &o;
    return nullptr;
  }
  CliOpt *find(char c) {
    for (auto &o : opts_)
      if (o.short_name == c) return &o;
    return nullptr;
  }
  const CliOpt *get(const std::string &n) const {
    for (auto &o : opts_)
      if (o.name == n) return &o;
    return nullptr;
  }
  std::string usage() const {
    std::string u = "usage: " + prog_;
    for (auto &o : opts_)
      if (o.required) u += " --" + o.name + "=value";
    u += " [options] ... \noptions:\n";
    for (auto &o : opts_) {
      u += "  -";
      u += o.short_name;
      u += ", --" + o.name;
      u += std::string(o.name.size() < 14 ? 14 - o.name.size() : 1, ' ');
      u += o.desc + "\n";
    }
    return u;
  }
  std::vector<CliOpt> opts_;
  std::string prog_;
};

}  // namespace ngia
