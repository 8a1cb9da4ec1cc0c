// synth.cpp — seeded synthetic sequence families (ancestors + mutated
// descendants) for the clustering workloads: DNA over ACGT, proteins over the
// 20 amino acids with background residue frequencies.
//
// Every random quantity comes from integer generators (xoshiro256**), and
// the only floating-point operations are +, -, *, / and conversions, so the
// same seed gives the same bytes on x86-64 and aarch64 (the file is compiled
// with -ffp-contract=off; exp/log are evaluated by the series below rather
// than by libm, whose last-bit results differ between platforms).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "host_common.h"

namespace {

inline uint64_t splitmix64(uint64_t &z) {
  uint64_t x = (z += 0x9E3779B97F4A7C15ull);
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct Rng {
  uint64_t s[4];
  Rng(uint64_t seed, uint64_t tag, uint64_t idx) {
    uint64_t z = seed ^ (tag * 0xD1B54A32D192ED03ull) ^ (idx * 0x8CB92BA72F3D8DD7ull);
    for (auto &x : s) x = splitmix64(z);
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  inline uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  inline double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  inline uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
  // Approximately standard normal: Irwin-Hall sum of 12 uniforms.
  inline double normal() {
    double acc = 0.0;
    for (int i = 0; i < 12; i++) acc += uni();
    return acc - 6.0;
  }
};

const double kLn2 = 0.69314718055994530942;

// exp(x) by range reduction x = k ln2 + r, |r| <= ln2/2, and a degree-22
// Taylor polynomial; ldexp is exact.
double det_exp(double x) {
  double kf = std::floor(x / kLn2 + 0.5);
  double r = x - kf * kLn2;
  double term = 1.0, sum = 1.0;
  for (int n = 1; n <= 22; n++) {
    term = term * r / (double)n;
    sum = sum + term;
  }
  return std::ldexp(sum, (int)kf);
}

// log(x), x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh((m-1)/(m+1)) summed to t^41.
double det_log(double x) {
  int e = 0;
  double m = std::frexp(x, &e);  // exact
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  double t = (m - 1.0) / (m + 1.0);
  double t2 = t * t, pw = t, sum = 0.0;
  for (int k = 1; k <= 41; k += 2) {
    sum = sum + pw / (double)k;
    pw = pw * t2;
  }
  return (double)e * kLn2 + 2.0 * sum;
}

// Background amino-acid frequencies (Robinson & Robinson 1991), in
// one-letter order ARNDCQEGHILKMFPSTWYV.
const char kAmino[21] = "ARNDCQEGHILKMFPSTWYV";
const double kAminoFreq[20] = {0.07805, 0.05129, 0.04487, 0.05364, 0.01925,
                               0.04264, 0.06295, 0.07377, 0.02199, 0.05142,
                               0.09019, 0.05744, 0.02243, 0.03856, 0.05203,
                               0.07120, 0.05841, 0.01330, 0.03216, 0.06441};

struct Alphabet {
  int type;
  uint32_t cum[20];  // cumulative thresholds on 32-bit draws (protein)
  explicit Alphabet(int t) : type(t) {
    double total = 0.0;
    for (double f : kAminoFreq) total = total + f;
    double acc = 0.0;
    for (int i = 0; i < 20; i++) {
      acc = acc + kAminoFreq[i];
      double v = acc / total * 4294967296.0;
      cum[i] = i == 19 ? 0xFFFFFFFFu : (uint32_t)v;
    }
  }
  // Residue code: DNA 0..3 (ACGT), protein 0..19 (index into kAmino).
  inline int draw(Rng &g) const {
    if (type == 0) return (int)(g.next() >> 62);
    uint32_t u = (uint32_t)(g.next() >> 32);
    int i = 0;
    while (i < 19 && u >= cum[i]) i++;
    return i;
  }
  inline char letter(int c) const { return type == 0 ? "ACGT"[c] : kAmino[c]; }
};

int64_t draw_length(const ngia_synth_params &p, Rng &g) {
  double v;
  if (p.len_dist == 0) {
    v = p.len_a + p.len_b * g.normal();
  } else if (p.len_dist == 1) {
    v = det_exp(det_log(p.len_a) + p.len_b * g.normal());
  } else {
    double la = det_log(p.len_a), lb = det_log(p.len_b);
    v = det_exp(la + g.uni() * (lb - la));
  }
  int64_t L = (int64_t)std::floor(v + 0.5);
  if (L < p.len_min) L = p.len_min;
  if (L > p.len_max) L = p.len_max;
  return L;
}

// Stream tags.
enum : uint64_t { kTagAncestor = 1, kTagNovel = 2, kTagDescendant = 3 };

std::string make_ancestor(const ngia_synth_params &p, const Alphabet &ab,
                          uint64_t tag, int64_t idx) {
  Rng g(p.seed, tag, (uint64_t)idx);
  int64_t L = draw_length(p, g);
  std::string s((size_t)L, 'A');
  for (int64_t i = 0; i < L; i++) s[(size_t)i] = (char)ab.draw(g);
  return s;  // residue codes, not letters
}

// One descendant: substitutions at rate r ~ U[0, subst_max] and indel events
// (insert or delete U{1..indel_max} residues) at rate indel_frac * r.
void make_descendant(const ngia_synth_params &p, const Alphabet &ab,
                     const std::vector<std::string> &anc,
                     const std::vector<std::string> &novel, int64_t i,
                     std::string &out) {
  Rng g(p.seed, kTagDescendant, (uint64_t)i);
  const std::string *a;
  if (p.novel_frac > 0.0 && !novel.empty() && g.uni() < p.novel_frac)
    a = &novel[g.below((uint32_t)novel.size())];
  else
    a = &anc[g.below((uint32_t)anc.size())];
  double r = g.uni() * p.subst_max;
  uint32_t sub_thr = (uint32_t)(r * 4294967295.0);
  uint32_t indel_thr = (uint32_t)(r * p.indel_frac * 4294967295.0);
  uint32_t imax = (uint32_t)(p.indel_max < 1 ? 1 : p.indel_max);
  const int64_t La = (int64_t)a->size();
  out.clear();
  out.reserve((size_t)(La + La / 16 + 8));
  for (int64_t q = 0; q < La; q++) {
    uint64_t u = g.next();
    uint32_t u_indel = (uint32_t)(u >> 32), u_sub = (uint32_t)u;
    if (u_indel < indel_thr) {
      uint64_t v = g.next();
      uint32_t len = 1 + (uint32_t)(((v >> 32) * (uint64_t)imax) >> 32);
      if (v & 1) {  // insertion before ancestor residue q
        for (uint32_t k = 0; k < len; k++) out.push_back(ab.letter(ab.draw(g)));
      } else {      // deletion of ancestor residues q .. q+len-1
        q += len - 1;
        continue;
      }
    }
    int c = (unsigned char)(*a)[(size_t)q];
    if (u_sub < sub_thr) {
      if (ab.type == 0) {
        c = (c + 1 + (int)g.below(3)) & 3;
      } else {
        int d = c;
        for (int t = 0; t < 16 && d == c; t++) d = ab.draw(g);
        c = d;
      }
    }
    out.push_back(ab.letter(c));
  }
}

}  // namespace

extern "C" int ngia_synth_generate(const ngia_synth_params *pp, char **seq,
                                   int64_t **seq_off, int64_t *n) {
  if (!pp || !seq || !seq_off || !n) return ngia::fail(NGIA_E_ARG, "synth: null argument");
  const ngia_synth_params p = *pp;
  if (p.type != 0 && p.type != 1) return ngia::fail(NGIA_E_ARG, "synth: type %d", p.type);
  if (p.n_seqs < 0 || p.n_ancestors < 1 || p.len_min < 0 || p.len_max < p.len_min)
    return ngia::fail(NGIA_E_ARG, "synth: bad sizes");
  if (p.len_dist != 0 && (p.len_a <= 0.0 || (p.len_dist == 2 && p.len_b <= 0.0)))
    return ngia::fail(NGIA_E_ARG, "synth: bad length distribution");
  Alphabet ab(p.type);

  std::vector<std::string> anc((size_t)p.n_ancestors), novel;
  size_t n_novel = p.novel_frac > 0.0 ? (size_t)p.n_ancestors : 0;
  novel.resize(n_novel);
  ngia::parallel_for((int64_t)anc.size() + (int64_t)n_novel, 64, [&](int64_t a) {
    if (a < (int64_t)anc.size())
      anc[(size_t)a] = make_ancestor(p, ab, kTagAncestor, a);
    else
      novel[(size_t)(a - (int64_t)anc.size())] =
          make_ancestor(p, ab, kTagNovel, a - (int64_t)anc.size());
  });

  const int64_t N = p.n_seqs;
  const int64_t chunk = 2048;
  const int64_t nchunks = (N + chunk - 1) / chunk;
  std::vector<std::string> parts((size_t)nchunks);
  std::vector<std::vector<int64_t>> lens((size_t)nchunks);
  // One allocation per chunk (sized for the longest possible descendants) and
  // one scratch string per thread.
  const size_t max_desc = (size_t)p.len_max + (size_t)p.len_max / 4 + 64;
  std::vector<std::string> scratch((size_t)ngia::hardware_threads());
  ngia::parallel_for(nchunks, 1, [&](int64_t c, int t) {
    std::string &tmp = scratch[(size_t)t];
    std::string &dst = parts[(size_t)c];
    const int64_t cnt = std::min(N, (c + 1) * chunk) - c * chunk;
    dst.reserve((size_t)cnt * max_desc);
    lens[(size_t)c].reserve((size_t)cnt);
    for (int64_t i = c * chunk; i < c * chunk + cnt; i++) {
      make_descendant(p, ab, anc, novel, i, tmp);
      dst += tmp;
      lens[(size_t)c].push_back((int64_t)tmp.size());
    }
  });
  int64_t total = 0;
  for (auto &s : parts) total += (int64_t)s.size();
  char *buf = (char *)std::malloc((size_t)total + 1);
  int64_t *off = (int64_t *)std::malloc(sizeof(int64_t) * (size_t)(N + 1));
  if (!buf || !off) {
    std::free(buf);
    std::free(off);
    return ngia::fail(NGIA_E_NOMEM, "synth: out of host memory (%lld bytes)", (long long)total);
  }
  int64_t pos = 0, k = 0;
  off[0] = 0;
  for (int64_t c = 0; c < nchunks; c++) {
    std::memcpy(buf + pos, parts[(size_t)c].data(), parts[(size_t)c].size());
    for (int64_t L : lens[(size_t)c]) {
      pos += L;
      off[++k] = pos;
    }
    std::string().swap(parts[(size_t)c]);
  }
  buf[total] = 0;
  *seq = buf;
  *seq_off = off;
  *n = N;
  return NGIA_OK;
}

extern "C" int ngia_write_fasta(const char *path, const char *seq, const int64_t *seq_off,
                                int64_t n, int32_t width) {
  if (!path || (!seq && n) || (!seq_off && n)) return ngia::fail(NGIA_E_ARG, "write_fasta: null argument");
  if (width <= 0) width = 80;
  FILE *f = std::fopen(path, "wb");
  if (!f) return ngia::fail(NGIA_E_IO, "write_fasta: cannot create %s", path);
  std::vector<char> buf;
  buf.reserve(1 << 20);
  for (int64_t i = 0; i < n; i++) {
    char hdr[32];
    int h = std::snprintf(hdr, sizeof(hdr), ">s%lld\n", (long long)i);
    buf.insert(buf.end(), hdr, hdr + h);
    for (int64_t p = seq_off[i]; p < seq_off[i + 1]; p += width) {
      int64_t e = std::min(seq_off[i + 1], p + (int64_t)width);
      buf.insert(buf.end(), seq + p, seq + e);
      buf.push_back('\n');
    }
    if (buf.size() > (1u << 20)) {
      if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) {
        std::fclose(f);
        return ngia::fail(NGIA_E_IO, "write_fasta: short write to %s", path);
      }
      buf.clear();
    }
  }
  size_t w = buf.empty() ? 0 : std::fwrite(buf.data(), 1, buf.size(), f);
  int rc = std::fclose(f);
  if (w != buf.size() || rc != 0) return ngia::fail(NGIA_E_IO, "write_fasta: short write to %s", path);
  return NGIA_OK;
}
