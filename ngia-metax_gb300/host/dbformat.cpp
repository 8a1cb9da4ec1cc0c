// dbformat.cpp — the makeDB database format: FASTA indexing and bit-plane
// packing (the makeDB tool), the data.bin loader (readIndex/readData) and the
// cluster.txt / represent.fasta writer (saveResult).
//
// Format (makeDB/src/makeDB.cpp:1-16, 254-292):
//   int32 n, longest, shortest, type
//   int32 name_len[n], int32 read_len[n], int64 fasta_off[n], int64 pack_off[n]
//   records in sorted order, pack_off[0] = 16 + 24 n
// Record: [len, net, counts[4|28], planes] where residue k of a 32-residue
// block is bit k of each plane word; plane p holds bit p of the residue code;
// characters outside the alphabet are skipped (they count toward len only).
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "host_common.h"

using ngia::fail;

namespace {

// Residue codes of makeDataGen / makeDataPro (makeDB.cpp:117-129, 162-218);
// -1 = skipped character.
struct CodeTable {
  int8_t dna[256], pro[256];
  CodeTable() {
    std::memset(dna, -1, sizeof(dna));
    std::memset(pro, -1, sizeof(pro));
    const char *d = "ACGT";
    for (int i = 0; i < 4; i++) {
      dna[(unsigned char)d[i]] = (int8_t)i;
      dna[(unsigned char)(d[i] + 32)] = (int8_t)i;
    }
    dna[(unsigned char)'U'] = dna[(unsigned char)'u'] = 3;
    for (int i = 0; i < 26; i++) {
      pro['A' + i] = (int8_t)i;
      pro['a' + i] = (int8_t)i;
    }
    pro[(unsigned char)'*'] = 26;
    pro[(unsigned char)'-'] = 27;
  }
};
const CodeTable kCodes;

// Packs one record of raw length `len` into out[0 .. record_words).
void pack_record(int type, const char *s, int64_t len, uint32_t *out) {
  const int hw = ngia::header_words(type), P = ngia::plane_count(type);
  const int64_t nw = ngia::record_words(type, len);
  std::memset(out, 0, sizeof(uint32_t) * (size_t)nw);
  const int8_t *tab = type == 0 ? kCodes.dna : kCodes.pro;
  uint32_t cnt[28] = {0};
  uint32_t acc[5] = {0, 0, 0, 0, 0};
  uint32_t *packed = out + hw;
  int64_t count = 0;
  for (int64_t i = 0; i < len; i++) {
    int c = tab[(unsigned char)s[i]];
    if (c < 0) continue;
    cnt[c]++;
    const int k = (int)(count & 31);
    for (int p = 0; p < P; p++) acc[p] |= (uint32_t)((c >> p) & 1) << k;
    count++;
    if ((count & 31) == 0) {
      for (int p = 0; p < P; p++) {
        packed[p] = acc[p];
        acc[p] = 0;
      }
      packed += P;
    }
  }
  if (count & 31)
    for (int p = 0; p < P; p++) packed[p] = acc[p];
  out[0] = (uint32_t)len;
  out[1] = (uint32_t)count;
  for (int c = 0; c < ngia::count_words(type); c++) out[2 + c] = cnt[c];
}

ngia_db_host *alloc_db(int64_t n, int64_t n_words) {
  auto *db = (ngia_db_host *)std::calloc(1, sizeof(ngia_db_host));
  if (!db) return nullptr;
  size_t nn = (size_t)std::max<int64_t>(n, 1);
  db->name_len = (int32_t *)std::malloc(sizeof(int32_t) * nn);
  db->read_len = (int32_t *)std::malloc(sizeof(int32_t) * nn);
  db->fasta_off = (int64_t *)std::malloc(sizeof(int64_t) * nn);
  db->pack_off = (int64_t *)std::malloc(sizeof(int64_t) * nn);
  int64_t *rec_off = (int64_t *)std::malloc(sizeof(int64_t) * nn);
  uint32_t *words = (uint32_t *)std::malloc(sizeof(uint32_t) * (size_t)std::max<int64_t>(n_words, 1));
  db->view.rec_off = rec_off;
  db->view.words = words;
  if (!db->name_len || !db->read_len || !db->fasta_off || !db->pack_off || !rec_off || !words) {
    ngia_db_free(db);
    return nullptr;
  }
  db->view.n = (int32_t)n;
  db->view.n_words = n_words;
  return db;
}

// Reads a whole file into memory.
bool slurp(const std::string &path, std::vector<char> &out) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    return false;
  }
  out.resize((size_t)sz);
  size_t got = sz ? std::fread(out.data(), 1, (size_t)sz, f) : 0;
  std::fclose(f);
  return got == (size_t)sz;
}

// One getline() step of the reference's FASTA scan: [b, e) is the line,
// returns the position after the newline.  A trailing '\r' is dropped the
// way makeDB does (makeDB.cpp:82, 88); for an empty line the reference reads
// line[-1] (undefined) — here an empty line is left empty.
inline size_t next_line(const std::vector<char> &t, size_t pos, size_t &b, size_t &e) {
  const size_t n = t.size();
  const char *nl = (const char *)std::memchr(t.data() + pos, '\n', n - pos);
  size_t end = nl ? (size_t)(nl - t.data()) : n;
  b = pos;
  e = end;
  if (e > b && t[e - 1] == '\r') e--;
  return nl ? end + 1 : n;
}

struct FastaRec {
  int64_t offset;      // byte offset of the header line
  int64_t name_len;    // header length without '\r' (includes '>')
  int64_t read_len;    // residue characters over all sequence lines
  int64_t seq_begin;   // first sequence line
  int64_t seq_end;     // end of the record in the file
};

// makeIndex, makeDB.cpp:62-106: scan records, drop those longer than 65,536,
// stable-sort by raw length descending.
void index_fasta(const std::vector<char> &t, std::vector<FastaRec> &recs) {
  size_t pos = 0, b, e;
  const size_t n = t.size();
  while (pos < n) {
    FastaRec r;
    r.offset = (int64_t)pos;
    pos = next_line(t, pos, b, e);
    r.name_len = (int64_t)(e - b);
    r.read_len = 0;
    r.seq_begin = (int64_t)pos;
    while (pos < n && t[pos] != '>') {
      pos = next_line(t, pos, b, e);
      r.read_len += (int64_t)(e - b);
    }
    r.seq_end = (int64_t)pos;
    if (r.read_len <= ngia::kMaxLen) recs.push_back(r);
  }
  std::stable_sort(recs.begin(), recs.end(),
                   [](const FastaRec &a, const FastaRec &b) { return a.read_len > b.read_len; });
}

// Concatenates the sequence lines of one record ('\r' stripped).
void record_sequence(const std::vector<char> &t, const FastaRec &r, std::string &out) {
  out.clear();
  size_t pos = (size_t)r.seq_begin, b, e;
  while (pos < (size_t)r.seq_end) {
    pos = next_line(t, pos, b, e);
    out.append(t.data() + b, e - b);
  }
}

// Offsets of the sorted records (makeDB.cpp:278-288) and word offsets of the
// in-memory copy (func.cu:117-124).
void layout(ngia_db_host *db, int type) {
  const int64_t n = db->view.n;
  int64_t *rec_off = const_cast<int64_t *>(db->view.rec_off);
  int64_t w = 0;
  for (int64_t i = 0; i < n; i++) {
    rec_off[i] = w;
    db->pack_off[i] = 16 + 24 * n + 4 * w;
    w += ngia::record_words(type, db->read_len[i]);
  }
}

}  // namespace

extern "C" void ngia_db_free(ngia_db_host *db) {
  if (!db) return;
  std::free(db->name_len);
  std::free(db->read_len);
  std::free(db->fasta_off);
  std::free(db->pack_off);
  std::free(const_cast<int64_t *>(db->view.rec_off));
  std::free(const_cast<uint32_t *>(db->view.words));
  std::free(db);
}

extern "C" int ngia_db_pack(int32_t type, const char *seq, const int64_t *seq_off, int64_t n,
                            const int32_t *name_len, ngia_db_host **out) {
  if (!out || (n && (!seq || !seq_off))) return fail(NGIA_E_ARG, "db_pack: null argument");
  if (type != 0 && type != 1) return fail(NGIA_E_ARG, "db_pack: type %d", type);
  std::vector<int64_t> keep;
  keep.reserve((size_t)n);
  for (int64_t i = 0; i < n; i++)
    if (seq_off[i + 1] - seq_off[i] <= ngia::kMaxLen) keep.push_back(i);
  if (keep.empty()) return fail(NGIA_E_FORMAT, "db_pack: no sequence of length <= 65536");
  if (keep.size() > (size_t)INT_MAX) return fail(NGIA_E_LIMIT, "db_pack: too many sequences");
  std::stable_sort(keep.begin(), keep.end(), [&](int64_t a, int64_t b) {
    return seq_off[a + 1] - seq_off[a] > seq_off[b + 1] - seq_off[b];
  });
  const int64_t N = (int64_t)keep.size();
  int64_t words = 0;
  for (int64_t i : keep) words += ngia::record_words(type, seq_off[i + 1] - seq_off[i]);
  ngia_db_host *db = alloc_db(N, words);
  if (!db) return fail(NGIA_E_NOMEM, "db_pack: out of host memory");
  db->view.type = type;
  for (int64_t k = 0; k < N; k++) {
    int64_t i = keep[(size_t)k];
    db->read_len[k] = (int32_t)(seq_off[i + 1] - seq_off[i]);
    db->name_len[k] = name_len ? name_len[i] : 1;
    db->fasta_off[k] = 0;
  }
  layout(db, type);
  db->view.longest = db->read_len[0];
  db->view.shortest = db->read_len[N - 1];
  uint32_t *w = const_cast<uint32_t *>(db->view.words);
  ngia::parallel_for(N, 256, [&](int64_t k) {
    int64_t i = keep[(size_t)k];
    pack_record(type, seq + seq_off[i], seq_off[i + 1] - seq_off[i], w + db->view.rec_off[k]);
  });
  *out = db;
  return NGIA_OK;
}

extern "C" int ngia_makedb(const char *fasta_path, const char *outdir, int32_t type) {
  if (!fasta_path || !outdir) return fail(NGIA_E_ARG, "makedb: null argument");
  if (type != 0 && type != 1) return fail(NGIA_E_ARG, "makedb: type must be 0 or 1");
  // data.fasta: symlink to the absolute path of the input (makeDB.cpp:63-70).
  std::string in(fasta_path), dir(outdir);
  std::string in_dir = in.find('/') == std::string::npos ? "." : in.substr(0, in.rfind('/'));
  if (in_dir.empty()) in_dir = "/";
  std::string base = in.substr(in.rfind('/') == std::string::npos ? 0 : in.rfind('/') + 1);
  char *rdir = realpath(in_dir.c_str(), nullptr);
  if (!rdir) return fail(NGIA_E_IO, "makedb: cannot resolve %s", in_dir.c_str());
  std::string abs_in = std::string(rdir) + (std::string(rdir) == "/" ? "" : "/") + base;
  std::free(rdir);
  std::string link = dir + "/data.fasta";
  char *r_in = realpath(abs_in.c_str(), nullptr);
  char *r_link = realpath(link.c_str(), nullptr);
  bool same = r_in && r_link && std::strcmp(r_in, r_link) == 0;
  std::free(r_in);
  std::free(r_link);
  if (!same) {
    ::unlink(link.c_str());
    if (::symlink(abs_in.c_str(), link.c_str()) != 0)
      return fail(NGIA_E_IO, "makedb: cannot create %s", link.c_str());
  }
  std::vector<char> text;
  if (!slurp(link, text)) return fail(NGIA_E_IO, "makedb: cannot read %s", link.c_str());
  std::vector<FastaRec> recs;
  index_fasta(text, recs);
  if (recs.empty()) return fail(NGIA_E_FORMAT, "makedb: no sequence of length <= 65536");
  if (recs.size() > (size_t)INT_MAX) return fail(NGIA_E_LIMIT, "makedb: too many sequences");
  const int64_t N = (int64_t)recs.size();
  int64_t words = 0;
  for (auto &r : recs) words += ngia::record_words(type, r.read_len);
  ngia_db_host *db = alloc_db(N, words);
  if (!db) return fail(NGIA_E_NOMEM, "makedb: out of host memory");
  db->view.type = type;
  for (int64_t i = 0; i < N; i++) {
    db->name_len[i] = (int32_t)recs[(size_t)i].name_len;
    db->read_len[i] = (int32_t)recs[(size_t)i].read_len;
    db->fasta_off[i] = recs[(size_t)i].offset;
  }
  layout(db, type);
  uint32_t *w = const_cast<uint32_t *>(db->view.words);
  std::vector<std::string> scratch((size_t)ngia::hardware_threads());
  ngia::parallel_for(N, 256, [&](int64_t i, int t) {
    std::string &s = scratch[(size_t)t];
    record_sequence(text, recs[(size_t)i], s);
    pack_record(type, s.data(), (int64_t)s.size(), w + db->view.rec_off[i]);
  });
  std::string bin = dir + "/data.bin";
  FILE *f = std::fopen(bin.c_str(), "wb");
  if (!f) {
    ngia_db_free(db);
    return fail(NGIA_E_IO, "makedb: cannot create %s", bin.c_str());
  }
  int32_t hdr[4] = {(int32_t)N, db->read_len[0], db->read_len[N - 1], type};
  bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1;
  ok = ok && std::fwrite(db->name_len, sizeof(int32_t), (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(db->read_len, sizeof(int32_t), (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(db->fasta_off, sizeof(int64_t), (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(db->pack_off, sizeof(int64_t), (size_t)N, f) == (size_t)N;
  ok = ok && std::fwrite(db->view.words, sizeof(uint32_t), (size_t)words, f) == (size_t)words;
  ok = (std::fclose(f) == 0) && ok;
  ngia_db_free(db);
  if (!ok) return fail(NGIA_E_IO, "makedb: short write to %s", bin.c_str());
  return NGIA_OK;
}

extern "C" int ngia_db_load(const char *dirp, ngia_db_host **out) {
  if (!dirp || !out) return fail(NGIA_E_ARG, "db_load: null argument");
  std::string path = std::string(dirp) + "/data.bin";
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(NGIA_E_IO, "db_load: cannot open %s", path.c_str());
  std::fseek(f, 0, SEEK_END);
  const int64_t fsize = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  int32_t hdr[4];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1) {
    std::fclose(f);
    return fail(NGIA_E_IO, "db_load: %s shorter than its header", path.c_str());
  }
  const int64_t N = hdr[0];
  const int type = hdr[3];
  if (type != 0 && type != 1) {
    std::fclose(f);
    return fail(NGIA_E_FORMAT, "db_load: type word %d is not 0 (gene) or 1 (protein)", type);
  }
  if (N <= 0 || 16 + 24 * N > fsize) {
    std::fclose(f);
    return fail(NGIA_E_FORMAT, "db_load: sequence count %lld does not fit the file", (long long)N);
  }
  std::vector<int32_t> name_len((size_t)N), read_len((size_t)N);
  std::vector<int64_t> fasta_off((size_t)N), pack_off((size_t)N);
  bool ok = std::fread(name_len.data(), 4, (size_t)N, f) == (size_t)N &&
            std::fread(read_len.data(), 4, (size_t)N, f) == (size_t)N &&
            std::fread(fasta_off.data(), 8, (size_t)N, f) == (size_t)N &&
            std::fread(pack_off.data(), 8, (size_t)N, f) == (size_t)N;
  if (!ok) {
    std::fclose(f);
    return fail(NGIA_E_IO, "db_load: truncated index in %s", path.c_str());
  }
  int64_t words = 0;
  for (int64_t i = 0; i < N; i++) {
    if (read_len[(size_t)i] < 0 || read_len[(size_t)i] > ngia::kMaxLen) {
      std::fclose(f);
      return fail(NGIA_E_FORMAT, "db_load: record %lld has length %d", (long long)i, read_len[(size_t)i]);
    }
    words += ngia::record_words(type, read_len[(size_t)i]);
  }
  ngia_db_host *db = alloc_db(N, words);
  if (!db) {
    std::fclose(f);
    return fail(NGIA_E_NOMEM, "db_load: out of host memory");
  }
  db->view.type = type;
  std::memcpy(db->name_len, name_len.data(), 4 * (size_t)N);
  std::memcpy(db->read_len, read_len.data(), 4 * (size_t)N);
  std::memcpy(db->fasta_off, fasta_off.data(), 8 * (size_t)N);
  layout(db, type);
  db->view.longest = hdr[1];
  db->view.shortest = hdr[2];
  // Records: one read when they are contiguous (as makeDB writes them),
  // otherwise one seek + read per record like readData (func.cu:138-147).
  bool contiguous = true;
  for (int64_t i = 0; i < N && contiguous; i++) contiguous = pack_off[(size_t)i] == db->pack_off[i];
  uint32_t *w = const_cast<uint32_t *>(db->view.words);
  if (contiguous) {
    ok = 4 * words + pack_off[0] <= fsize && std::fseek(f, (long)pack_off[0], SEEK_SET) == 0 &&
         std::fread(w, 4, (size_t)words, f) == (size_t)words;
  } else {
    for (int64_t i = 0; i < N && ok; i++) {
      int64_t nw = ngia::record_words(type, read_len[(size_t)i]);
      ok = pack_off[(size_t)i] >= 0 && pack_off[(size_t)i] + 4 * nw <= fsize &&
           std::fseek(f, (long)pack_off[(size_t)i], SEEK_SET) == 0 &&
           std::fread(w + db->view.rec_off[i], 4, (size_t)nw, f) == (size_t)nw;
    }
  }
  std::memcpy(db->pack_off, pack_off.data(), 8 * (size_t)N);
  std::fclose(f);
  if (!ok) {
    ngia_db_free(db);
    return fail(NGIA_E_IO, "db_load: truncated records in %s", path.c_str());
  }
  for (int64_t i = 0; i < N; i++) {
    const uint32_t *r = w + db->view.rec_off[i];
    if ((int64_t)r[0] != read_len[(size_t)i] || r[1] > r[0]) {
      ngia_db_free(db);
      return fail(NGIA_E_FORMAT, "db_load: record %lld header disagrees with the index", (long long)i);
    }
  }
  *out = db;
  return NGIA_OK;
}

extern "C" int ngia_save_result(const char *dbdir, const char *outdir, const ngia_db_host *db,
                                const int32_t *cluster, int32_t *n_clusters) {
  if (!dbdir || !outdir || !db || !cluster) return fail(NGIA_E_ARG, "save_result: null argument");
  const int64_t N = db->view.n;
  // Members grouped by representative, ascending (func.cu:700-705).
  std::vector<int64_t> head((size_t)N, -1), tail((size_t)N, -1), next((size_t)N, -1);
  int32_t count = 0;
  for (int64_t i = 0; i < N; i++) {
    int32_t r = cluster[i];
    if (r < 0 || r >= N) return fail(NGIA_E_ARG, "save_result: cluster[%lld] = %d out of range", (long long)i, r);
    if (head[(size_t)r] < 0) {
      head[(size_t)r] = i;
      count++;
    } else {
      next[(size_t)tail[(size_t)r]] = i;
    }
    tail[(size_t)r] = i;
  }
  std::vector<char> text;
  std::string fa = std::string(dbdir) + "/data.fasta";
  if (!slurp(fa, text)) return fail(NGIA_E_IO, "save_result: cannot read %s", fa.c_str());
  std::string cpath = std::string(outdir) + "/cluster.txt", rpath = std::string(outdir) + "/represent.fasta";
  FILE *cf = std::fopen(cpath.c_str(), "wb");
  FILE *rf = std::fopen(rpath.c_str(), "wb");
  if (!cf || !rf) {
    if (cf) std::fclose(cf);
    if (rf) std::fclose(rf);
    return fail(NGIA_E_IO, "save_result: cannot create output files in %s", outdir);
  }
  // Record i: header line and concatenated sequence lines read at its FASTA
  // offset (func.cu:733-742).  Clusters in representative order, each
  // representative unindented, members indented by two spaces; reps also go
  // to represent.fasta as name + one-line sequence (func.cu:743-752).
  std::string name, seqbuf, cbuf, rbuf;
  bool ok = true;
  auto read_record = [&](int64_t i) {
    size_t pos = (size_t)db->fasta_off[i], b, e;
    if (pos > text.size()) pos = text.size();
    pos = next_line(text, pos, b, e);
    name.assign(text.data() + b, e - b);
    seqbuf.clear();
    while (pos < text.size() && text[pos] != '>') {
      pos = next_line(text, pos, b, e);
      seqbuf.append(text.data() + b, e - b);
    }
  };
  for (int64_t r = 0; r < N && ok; r++) {
    for (int64_t i = head[(size_t)r]; i >= 0; i = next[(size_t)i]) {
      read_record(i);
      if (i == head[(size_t)r]) {
        cbuf += name;
        cbuf += '\n';
        rbuf += name;
        rbuf += '\n';
        rbuf += seqbuf;
        rbuf += '\n';
      } else {
        cbuf += "  ";
        cbuf += name;
        cbuf += '\n';
      }
      if (cbuf.size() > (1u << 20)) {
        ok = std::fwrite(cbuf.data(), 1, cbuf.size(), cf) == cbuf.size();
        cbuf.clear();
      }
      if (rbuf.size() > (1u << 20)) {
        ok = ok && std::fwrite(rbuf.data(), 1, rbuf.size(), rf) == rbuf.size();
        rbuf.clear();
      }
    }
  }
  if (ok && !cbuf.empty()) ok = std::fwrite(cbuf.data(), 1, cbuf.size(), cf) == cbuf.size();
  if (ok && !rbuf.empty()) ok = std::fwrite(rbuf.data(), 1, rbuf.size(), rf) == rbuf.size();
  ok = (std::fclose(cf) == 0) && ok;
  ok = (std::fclose(rf) == 0) && ok;
  if (!ok) return fail(NGIA_E_IO, "save_result: short write in %s", outdir);
  if (n_clusters) *n_clusters = count;
  return NGIA_OK;
}
