// GFmatrix restart files (save_gfprime / read_gfprime,
// VCA_AUX_FUNX.f90:486-697): encoder and decoder of the two layouts.
#include "vca_gfmatrix.h"

#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

// bounds on what a file may ask the reader to allocate
constexpr int64_t kMaxCount = int64_t(1) << 20;     // states or channels of one element
constexpr int64_t kMaxExcTotal = int64_t(1) << 24;  // excitations in one file

void put_u32(std::vector<unsigned char>& b, uint32_t v) {
  for (int i = 0; i < 4; i++) b.push_back((unsigned char)((v >> (8 * i)) & 0xffu));
}
void put_f64(std::vector<unsigned char>& b, double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  for (int i = 0; i < 8; i++) b.push_back((unsigned char)((u >> (8 * i)) & 0xffu));
}
uint32_t get_u32(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
double get_f64(const unsigned char* p) {
  uint64_t u = 0;
  for (int i = 7; i >= 0; i--) u = (u << 8) | p[i];
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

bool slurp(const std::string& path, std::string& data, std::string& err) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open " + path + ": " + std::strerror(errno);
    return false;
  }
  data.clear();
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) data.append(buf, n);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) err = "read error on " + path;
  return !bad;
}

bool emit(std::FILE* f, const void* p, size_t n, std::string& err) {
  if (n && std::fwrite(p, 1, n, f) != n) {
    err = std::string("write error: ") + std::strerror(errno);
    return false;
  }
  return true;
}

// ---- unformatted: one sequential record per element (write_unformatted,
// VCA_AUX_FUNX.f90:547-566; the parent write at :636) ----------------------
int write_unformatted(std::FILE* f, const GfmTable& t, std::string& err) {
  size_t is = 0, ic = 0, ix = 0;
  std::vector<unsigned char> rec;
  for (size_t e = 0; e < t.nstates.size(); e++) {
    int64_t bytes = 4;
    for (size_t s = is, c = ic; s < is + (size_t)t.nstates[e]; s++) {
      bytes += 4;
      for (int k = 0; k < t.nchan[s]; k++, c++) bytes += 4 + 32 * (int64_t)t.nexc[c];
    }
    if (bytes > INT32_MAX) {
      err = "element " + std::to_string(e) + ": record over 2 GiB (continued records are not written)";
      return -1;
    }
    rec.clear();
    put_u32(rec, (uint32_t)bytes);
    put_u32(rec, (uint32_t)t.nstates[e]);
    for (int s = 0; s < t.nstates[e]; s++, is++) {
      put_u32(rec, (uint32_t)t.nchan[is]);
      for (int k = 0; k < t.nchan[is]; k++, ic++) {
        const int32_t n = t.nexc[ic];
        put_u32(rec, (uint32_t)n);
        for (int j = 0; j < n; j++) {
          put_f64(rec, t.poles[2 * (ix + j)]);
          put_f64(rec, t.poles[2 * (ix + j) + 1]);
        }
        for (int j = 0; j < n; j++) {
          put_f64(rec, t.weights[2 * (ix + j)]);
          put_f64(rec, t.weights[2 * (ix + j) + 1]);
        }
        ix += (size_t)n;
      }
    }
    put_u32(rec, (uint32_t)bytes);
    if (!emit(f, rec.data(), rec.size(), err)) return -1;
  }
  return 0;
}

// read_unformatted (:572-593): the child reads of one element continue in
// the element's record; bytes left in a record are skipped
int read_unformatted(const std::string& data, int64_t nelem, GfmTable& t, std::string& err) {
  const unsigned char* p = (const unsigned char*)data.data();
  const size_t n = data.size();
  size_t off = 0;
  int64_t total = 0;
  for (int64_t e = 0; e < nelem; e++) {
    const std::string where = "element " + std::to_string(e) + ": ";
    if (n - off < 4) {
      err = where + "end of file";
      return -1;
    }
    const int32_t m = (int32_t)get_u32(p + off);
    if (m < 0) {
      err = where + "continued record (over 2 GiB): not supported";
      return -1;
    }
    if ((size_t)m > n - off - 4 || n - off - 4 - (size_t)m < 4) {
      err = where + "truncated record";
      return -1;
    }
    const unsigned char* r = p + off + 4;
    if ((int32_t)get_u32(r + m) != m) {
      err = where + "leading and trailing record markers differ";
      return -1;
    }
    size_t q = 0;
    auto count = [&](int64_t cap, int32_t& v) {
      if ((size_t)m - q < 4) {
        err = where + "record too short";
        return false;
      }
      v = (int32_t)get_u32(r + q);
      q += 4;
      if (v < 0 || v > cap) {
        err = where + "count out of range: " + std::to_string(v);
        return false;
      }
      return true;
    };
    int32_t ns;
    if (!count(kMaxCount, ns)) return -1;
    t.nstates.push_back(ns);
    for (int s = 0; s < ns; s++) {
      int32_t nc;
      if (!count(kMaxCount, nc)) return -1;
      t.nchan.push_back(nc);
      for (int k = 0; k < nc; k++) {
        int32_t nx;
        if (!count(kMaxExcTotal, nx)) return -1;
        if ((uint64_t)nx * 32 > (uint64_t)m - q || total + nx > kMaxExcTotal) {
          err = where + "record too short for " + std::to_string(nx) + " excitations";
          return -1;
        }
        total += nx;
        t.nexc.push_back(nx);
        for (int j = 0; j < 2 * nx; j++, q += 8) t.poles.push_back(get_f64(r + q));
        for (int j = 0; j < 2 * nx; j++, q += 8) t.weights.push_back(get_f64(r + q));
      }
    }
    off += (size_t)m + 8;
  }
  return 0;
}

// ---- formatted: list-directed text (write_formatted / read_formatted,
// :486-539; the parent statements at :634, :685) --------------------------
void put_cplx(std::string& s, double re, double im) {
  char b[80];
  std::snprintf(b, sizeof b, " (%.17g,%.17g)", re, im);
  s += b;
}

int write_formatted(std::FILE* f, const GfmTable& t, std::string& err) {
  size_t is = 0, ic = 0, ix = 0;
  std::string line;
  for (size_t e = 0; e < t.nstates.size(); e++) {
    line.clear();
    line += " " + std::to_string(t.nstates[e]);
    for (int s = 0; s < t.nstates[e]; s++, is++) {
      line += " " + std::to_string(t.nchan[is]);
      for (int k = 0; k < t.nchan[is]; k++, ic++) {
        const int32_t n = t.nexc[ic];
        line += " " + std::to_string(n);
        for (int j = 0; j < n; j++) put_cplx(line, t.poles[2 * (ix + j)], t.poles[2 * (ix + j) + 1]);
        for (int j = 0; j < n; j++) put_cplx(line, t.weights[2 * (ix + j)], t.weights[2 * (ix + j) + 1]);
        ix += (size_t)n;
      }
    }
    // the reference writes the two characters \n after every state (:503);
    // between states they would stop its own reader (a count is read
    // there), so they are written once, after the last state, where the
    // reader's next parent statement skips the rest of the line
    if (t.nstates[e] > 0) line += " \\n";
    line += "\n";
    if (!emit(f, line.data(), line.size(), err)) return -1;
  }
  return 0;
}

// List-directed input: values separated by blanks, line ends or one comma;
// complex values as (re,im), blanks and line ends allowed inside; reals in
// any form strtod reads, with D or E exponents; repeat counts r*c.  Null
// values and the slash terminator are rejected.  The two-character token \n
// (what the reference writes after each state) is skipped between values.
struct ListReader {
  const std::string& s;
  size_t i = 0;
  int64_t rep = 0;
  bool rep_cplx = false;
  int64_t rep_int = 0;
  double rep_re = 0.0, rep_im = 0.0;
  std::string err;

  explicit ListReader(const std::string& src) : s(src) {}

  static bool blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; }
  bool ends_token(size_t j) const { return j >= s.size() || blank(s[j]) || s[j] == ','; }

  void skip_blanks() {
    for (;;) {
      while (i < s.size() && blank(s[i])) i++;
      if (i + 1 < s.size() && s[i] == '\\' && s[i + 1] == 'n' && ends_token(i + 2)) {
        i += 2;
        continue;
      }
      return;
    }
  }
  // after a value: blanks on the same line, then at most one comma
  void end_value() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) i++;
    if (i < s.size() && s[i] == ',') i++;
  }
  // the next statement starts on the next line
  void next_record() {
    rep = 0;
    while (i < s.size() && s[i] != '\n') i++;
    if (i < s.size()) i++;
  }
  bool start_value() {
    skip_blanks();
    if (i >= s.size()) {
      err = "end of file";
      return false;
    }
    if (s[i] == ',' || s[i] == '/') {
      err = s[i] == ',' ? "null value: not supported" : "slash terminator: not supported";
      return false;
    }
    return true;
  }
  // optional r* prefix; sets rep to r - 1 (the copies still to hand out)
  bool repeat_prefix(int64_t& r) {
    r = 1;
    size_t j = i;
    while (j < s.size() && s[j] >= '0' && s[j] <= '9') j++;
    if (j == i || j >= s.size() || s[j] != '*') return true;
    r = 0;
    for (size_t k = i; k < j; k++) {
      r = r * 10 + (s[k] - '0');
      if (r > kMaxExcTotal) {
        err = "repeat count too large";
        return false;
      }
    }
    i = j + 1;
    if (r < 1 || ends_token(i)) {
      err = "null value: not supported";
      return false;
    }
    return true;
  }
  bool real(double& x) {
    size_t j = i;
    while (j < s.size() && !blank(s[j]) && s[j] != ',' && s[j] != ')' && s[j] != '(' && s[j] != '/') j++;
    std::string tok = s.substr(i, j - i);
    if (tok.empty()) {
      err = "missing real value";
      return false;
    }
    for (char& c : tok)
      if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    x = std::strtod(tok.c_str(), &end);
    if (end != tok.c_str() + tok.size()) {
      err = "bad real value '" + tok + "'";
      return false;
    }
    i = j;
    return true;
  }
  void skip_ws() {
    while (i < s.size() && blank(s[i])) i++;
  }
  bool expect(char c) {  // c and the blanks around it
    skip_ws();
    if (i >= s.size() || s[i] != c) {
      err = std::string("expected '") + c + "' in a complex value";
      return false;
    }
    i++;
    skip_ws();
    return true;
  }

  bool integer(int64_t& v) {
    if (rep > 0) {
      if (rep_cplx) {
        err = "complex value where a count is expected";
        return false;
      }
      rep--;
      v = rep_int;
      return true;
    }
    int64_t r;
    if (!start_value() || !repeat_prefix(r)) return false;
    size_t j = i;
    if (j < s.size() && (s[j] == '+' || s[j] == '-')) j++;
    const size_t d0 = j;
    while (j < s.size() && s[j] >= '0' && s[j] <= '9') j++;
    if (j == d0 || !ends_token(j) || j - d0 > 10) {
      size_t k = i;
      while (!ends_token(k)) k++;
      err = "bad integer '" + s.substr(i, k - i) + "'";
      return false;
    }
    v = std::strtoll(s.substr(i, j - i).c_str(), nullptr, 10);
    if (v < INT32_MIN || v > INT32_MAX) {
      err = "integer out of range";
      return false;
    }
    i = j;
    end_value();
    rep = r - 1;
    rep_cplx = false;
    rep_int = v;
    return true;
  }

  bool complex(double& re, double& im) {
    if (rep > 0) {
      if (!rep_cplx) {
        err = "integer where a complex value is expected";
        return false;
      }
      rep--;
      re = rep_re;
      im = rep_im;
      return true;
    }
    int64_t r;
    if (!start_value() || !repeat_prefix(r)) return false;
    if (s[i] != '(') {
      err = "expected '(' of a complex value";
      return false;
    }
    i++;
    skip_ws();
    if (!real(re) || !expect(',') || !real(im)) return false;
    skip_ws();
    if (i >= s.size() || s[i] != ')') {
      err = "expected ')' of a complex value";
      return false;
    }
    i++;
    end_value();
    rep = r - 1;
    rep_cplx = true;
    rep_re = re;
    rep_im = im;
    return true;
  }
};

int read_formatted(const std::string& data, int64_t nelem, GfmTable& t, std::string& err) {
  ListReader L(data);
  int64_t total = 0;
  for (int64_t e = 0; e < nelem; e++) {
    const std::string where = "element " + std::to_string(e) + ": ";
    auto count = [&](int64_t cap, int32_t& v) {
      int64_t x;
      if (!L.integer(x)) {
        err = where + L.err;
        return false;
      }
      if (x < 0 || x > cap) {
        err = where + "count out of range: " + std::to_string(x);
        return false;
      }
      v = (int32_t)x;
      return true;
    };
    int32_t ns;
    if (!count(kMaxCount, ns)) return -1;
    t.nstates.push_back(ns);
    for (int s = 0; s < ns; s++) {
      int32_t nc;
      if (!count(kMaxCount, nc)) return -1;
      t.nchan.push_back(nc);
      for (int k = 0; k < nc; k++) {
        int32_t nx;
        if (!count(kMaxExcTotal - total, nx)) return -1;
        total += nx;
        t.nexc.push_back(nx);
        for (auto* dst : {&t.poles, &t.weights})
          for (int j = 0; j < nx; j++) {
            double re, im;
            if (!L.complex(re, im)) {
              err = where + L.err;
              return -1;
            }
            dst->push_back(re);
            dst->push_back(im);
          }
      }
    }
    L.next_record();
  }
  return 0;
}

}  // namespace

bool gfm_consistent(const GfmTable& t, std::string& err) {
  int64_t ns = 0, nc = 0, ne = 0;
  for (int32_t v : t.nstates) {
    if (v < 0) { err = "negative state count"; return false; }
    ns += v;
  }
  if ((int64_t)t.nchan.size() != ns) {
    err = "channel counts: " + std::to_string(t.nchan.size()) + " given, " + std::to_string(ns) + " states";
    return false;
  }
  for (int32_t v : t.nchan) {
    if (v < 0) { err = "negative channel count"; return false; }
    nc += v;
  }
  if ((int64_t)t.nexc.size() != nc) {
    err = "excitation counts: " + std::to_string(t.nexc.size()) + " given, " + std::to_string(nc) + " channels";
    return false;
  }
  for (int32_t v : t.nexc) {
    if (v < 0) { err = "negative excitation count"; return false; }
    ne += v;
  }
  if ((int64_t)t.poles.size() != 2 * ne || (int64_t)t.weights.size() != 2 * ne) {
    err = "pole or weight array length differs from 2 * sum of the excitation counts";
    return false;
  }
  return true;
}

int gfm_write(const std::string& path, bool formatted, const GfmTable& t, std::string& err) {
  if (!gfm_consistent(t, err)) return -1;
  std::FILE* f = std::fopen(path.c_str(), formatted ? "w" : "wb");
  if (!f) {
    err = "cannot open " + path + ": " + std::strerror(errno);
    return -1;
  }
  int rc = formatted ? write_formatted(f, t, err) : write_unformatted(f, t, err);
  if (std::fclose(f) != 0 && rc == 0) {
    err = "close of " + path + " failed: " + std::strerror(errno);
    rc = -1;
  }
  return rc;
}

int gfm_read(const std::string& path, bool formatted, int64_t nelem, GfmTable& t, std::string& err) {
  t = GfmTable{};
  if (nelem < 0) {
    err = "negative element count";
    return -1;
  }
  std::string data;
  if (!slurp(path, data, err)) return -1;
  const int rc = formatted ? read_formatted(data, nelem, t, err) : read_unformatted(data, nelem, t, err);
  if (rc) {
    err = path + ": " + err;
    t = GfmTable{};
  }
  return rc;
}
