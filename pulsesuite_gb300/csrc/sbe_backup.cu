// Backup text format of the SBE state (SBEs.py:5524-5569 write_sbes_data /
// read_sbes_data, module wrappers WriteSBEsData / ReadSBEsData :6046-6053): one
// line "re im\n" per complex element, each number printed as f"{np.float64}" does,
// i.e. Python's repr of a float64: the shortest digit string that reads back to the
// same double, in positional notation when the decimal point sits between -4 and 16
// digits from the first digit, else d.ddde+XX.  Host code only (no device call): the
// caller copies the state to host memory in the file's element order.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "sbe_gb300.h"
#include "sbe_internal.cuh"

namespace {

constexpr int kMaxNum = 24;    // "-d.dddddddddddddddde-308": 17 digits, 24 characters
constexpr int kMaxLine = 2 * kMaxNum + 2;   // 50 bytes per line at most

// Python repr of x into p (no terminator); returns the number of characters
int repr_double(double x, char* p) {
  char* const p0 = p;
  if (std::isnan(x)) {
    std::memcpy(p, "nan", 3);
    return 3;
  }
  if (std::signbit(x)) {
    *p++ = '-';
    x = -x;
  }
  if (std::isinf(x)) {
    std::memcpy(p, "inf", 3);
    return (int)(p - p0) + 3;
  }
  if (x == 0.0) {
    std::memcpy(p, "0.0", 3);
    return (int)(p - p0) + 3;
  }
  // shortest round-trip digits in scientific form: d[.ddd]e(+|-)XX
  char sci[40];
  auto r = std::to_chars(sci, sci + sizeof(sci), x, std::chars_format::scientific);
  const char* e = std::find(sci, r.ptr, 'e');
  char dig[20];
  int nd = 0;
  for (const char* q = sci; q < e; ++q)
    if (*q != '.') dig[nd++] = *q;
  int exp10 = 0;
  std::from_chars(e + 1 + (e[1] == '+'), r.ptr, exp10);
  const int decpt = exp10 + 1;   // value = 0.DIGITS x 10^decpt
  if (decpt > -4 && decpt <= 16) {
    if (decpt <= 0) {
      *p++ = '0';
      *p++ = '.';
      for (int i = 0; i < -decpt; ++i) *p++ = '0';
      std::memcpy(p, dig, nd);
      p += nd;
    } else if (decpt < nd) {
      std::memcpy(p, dig, decpt);
      p += decpt;
      *p++ = '.';
      std::memcpy(p, dig + decpt, nd - decpt);
      p += nd - decpt;
    } else {
      std::memcpy(p, dig, nd);
      p += nd;
      for (int i = nd; i < decpt; ++i) *p++ = '0';
      *p++ = '.';
      *p++ = '0';
    }
  } else {
    *p++ = dig[0];
    if (nd > 1) {
      *p++ = '.';
      std::memcpy(p, dig + 1, nd - 1);
      p += nd - 1;
    }
    *p++ = 'e';
    const int ex = decpt - 1;
    *p++ = ex < 0 ? '-' : '+';
    const int a = ex < 0 ? -ex : ex;
    if (a >= 100) *p++ = (char)('0' + a / 100);
    *p++ = (char)('0' + (a / 10) % 10);
    *p++ = (char)('0' + a % 10);
  }
  return (int)(p - p0);
}

int pick_threads(int threads, long long work) {
  int t = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  return (int)std::max<long long>(1, std::min<long long>(t, work / 65536 + 1));
}

// the ASCII whitespace of Python's str.split() (the reader splits each line with it)
bool is_space(char ch) {
  return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f' ||
         (ch >= '\x1c' && ch <= '\x1f');
}

bool is_digit(char ch) { return ch >= '0' && ch <= '9'; }

bool ieq(const char* b, const char* e, const char* word) {
  for (; b < e && *word; ++b, ++word)
    if ((*b | 0x20) != *word) return false;
  return b == e && !*word;
}

// Python float() of the token [b, e): an optional sign, then "inf", "infinity" or
// "nan" in any case, or a decimal literal whose digit groups may hold single
// underscores between digits (digits [. digits] [e [sign] digits], either side of the
// point may be empty but not both).  Anything else (a second sign, "nan(...)", hex,
// a misplaced underscore) is rejected as float() rejects it.
bool py_float(const char* b, const char* e, double* out) {
  if (b >= e) return false;
  const bool neg = *b == '-';
  if (*b == '-' || *b == '+') ++b;
  if (b >= e) return false;
  if (ieq(b, e, "inf") || ieq(b, e, "infinity")) {
    *out = neg ? -HUGE_VAL : HUGE_VAL;
    return true;
  }
  if (ieq(b, e, "nan")) {
    *out = neg ? -NAN : NAN;
    return true;
  }
  // grammar check; a digit group is digit (["_"] digit)*
  bool under = false;
  auto group = [&](const char*& p) {
    if (p >= e || !is_digit(*p)) return false;
    ++p;
    while (p < e) {
      if (is_digit(*p)) {
        ++p;
      } else if (*p == '_' && p + 1 < e && is_digit(p[1])) {
        under = true;
        p += 2;
      } else {
        break;
      }
    }
    return true;
  };
  const char* p = b;
  const bool int_any = group(p);
  bool frac_any = false;
  if (p < e && *p == '.') {
    ++p;
    frac_any = group(p);
  }
  if (!int_any && !frac_any) return false;
  if (p < e && (*p == 'e' || *p == 'E')) {
    ++p;
    if (p < e && (*p == '+' || *p == '-')) ++p;
    if (!group(p)) return false;
  }
  if (p != e) return false;
  std::string clean;
  if (under) {
    for (const char* c = b; c < e; ++c)
      if (*c != '_') clean.push_back(*c);
    b = clean.data();
    e = b + clean.size();
  }
  double v = 0.0;
  const auto r = std::from_chars(b, e, v);
  if (r.ptr != e) return false;
  if (r.ec == std::errc::result_out_of_range) {
    // Python reads out-of-range literals as 0 or inf
    v = std::strtod(std::string(b, e).c_str(), nullptr);
  } else if (r.ec != std::errc()) {
    return false;
  }
  *out = neg ? -v : v;
  return true;
}

// the next whitespace-separated token of the line at p (nullptr: none before the
// line's end) parsed as Python's float() does; returns the end of the token
const char* parse_num(const char* p, const char* end, double* out, bool* ok) {
  while (p < end && is_space(*p)) ++p;
  if (p >= end || *p == '\n') return nullptr;
  const char* q = p;
  while (q < end && !is_space(*q) && *q != '\n') ++q;
  *ok = py_float(p, q, out);
  return q;
}

}  // namespace

extern "C" int sbe_backup_format(const double* values, long long count, char* out, long long cap,
                                 long long* written, int threads) {
  if (count < 0 || (count > 0 && (!values || !out)) || !written)
    return sbe::fail(SBE_ERR_ARG, "sbe_backup_format: bad arguments");
  if (cap < (long long)kMaxLine * count)
    return sbe::fail(SBE_ERR_ARG, "sbe_backup_format: out needs " +
                                      std::to_string((long long)kMaxLine * count) + " bytes");
  const int nt = pick_threads(threads, count);
  // each thread formats its slice into its own part of out, then the parts close up
  std::vector<long long> len(nt, 0);
  auto work = [&](int t) {
    const long long a = count * t / nt, b = count * (t + 1) / nt;
    char* p = out + (long long)kMaxLine * a;
    char* const p0 = p;
    for (long long i = a; i < b; ++i) {
      p += repr_double(values[2 * i], p);
      *p++ = ' ';
      p += repr_double(values[2 * i + 1], p);
      *p++ = '\n';
    }
    len[t] = p - p0;
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  long long pos = len[0];
  for (int t = 1; t < nt; ++t) {
    const long long a = count * t / nt;
    std::memmove(out + pos, out + (long long)kMaxLine * a, len[t]);
    pos += len[t];
  }
  *written = pos;
  return SBE_OK;
}

extern "C" int sbe_backup_parse(const char* text, long long len, double* values, long long count,
                                int threads) {
  if (len < 0 || count < 0 || (len > 0 && !text) || (count > 0 && !values))
    return sbe::fail(SBE_ERR_ARG, "sbe_backup_parse: bad arguments");
  const char* const end = text + len;
  const int nt = pick_threads(threads, len / 48);
  // chunk boundaries at line starts, lines per chunk, then each chunk parses its lines
  std::vector<const char*> cut(nt + 1, end);
  cut[0] = text;
  for (int t = 1; t < nt; ++t) {
    const char* p = text + len * t / nt;
    if (p < cut[t - 1]) p = cut[t - 1];
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', end - p));
    cut[t] = nl ? nl + 1 : end;
  }
  std::vector<long long> lines(nt, 0);
  auto count_lines = [&](int t) {
    long long n = 0;
    for (const char* p = cut[t]; p < cut[t + 1]; ++p) n += *p == '\n';
    if (cut[t + 1] == end && cut[t] < end && end[-1] != '\n') ++n;   // last line, no newline
    lines[t] = n;
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(count_lines, t);
  count_lines(0);
  for (auto& th : pool) th.join();
  pool.clear();
  std::vector<long long> first(nt + 1, 0);
  for (int t = 0; t < nt; ++t) first[t + 1] = first[t] + lines[t];
  if (first[nt] < count)
    return sbe::fail(SBE_ERR_ARG, "sbe_backup_parse: " + std::to_string(first[nt]) +
                                      " lines for " + std::to_string(count) + " values");
  std::vector<long long> bad(nt, -1);
  auto parse = [&](int t) {
    const char* p = cut[t];
    for (long long i = first[t]; i < std::min(first[t + 1], count); ++i) {
      bool ok0 = false, ok1 = false;
      const char* q = parse_num(p, cut[t + 1], &values[2 * i], &ok0);
      if (q) q = parse_num(q, cut[t + 1], &values[2 * i + 1], &ok1);
      if (!q || !ok0 || !ok1) {
        bad[t] = i;
        return;
      }
      // the reference stores float(re) + 1j * float(im); CPython promotes both operands
      // to complex, so the element is (re + (0 b - 0), 0 + (0 + b)) in IEEE arithmetic,
      // which decides the signs of zero parts
      {
        const double a = values[2 * i], b = values[2 * i + 1];
        const double zero = 0.0;
        values[2 * i] = a + (zero * b - zero * 1.0);
        values[2 * i + 1] = zero + (zero * zero + 1.0 * b);
      }
      // further tokens of the line are ignored, as split()[0:2] does
      const char* nl = static_cast<const char*>(std::memchr(q, '\n', cut[t + 1] - q));
      p = nl ? nl + 1 : cut[t + 1];
    }
  };
  for (int t = 1; t < nt; ++t) pool.emplace_back(parse, t);
  parse(0);
  for (auto& th : pool) th.join();
  for (int t = 0; t < nt; ++t)
    if (bad[t] >= 0)
      return sbe::fail(SBE_ERR_ARG,
                       "sbe_backup_parse: line " + std::to_string(bad[t] + 1) + " is not 're im'");
  return SBE_OK;
}
