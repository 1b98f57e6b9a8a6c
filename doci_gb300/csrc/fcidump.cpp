// fcidump.cpp -- FCIDUMP input and the reference's integral transform (host).
//
// The file format, the parsing rules and the transform are an interface that
// has to behave exactly as the reference's (src/read_fcidump.c:18-82,
// src/doci.c:630-665): same header scan, same namelist skip, same index
// placement, same propagation domain of the 8-fold symmetry, so that the same
// file gives bit-identical integrals.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "internal.h"

namespace doci {

// read_fcidump.c:88-110: the non-blank characters of `line` spell `word`
static bool is_namelist_end(const char *line, const char *word) {
  const unsigned char *p = reinterpret_cast<const unsigned char *>(line);
  const unsigned char *q = reinterpret_cast<const unsigned char *>(word);
  for (;;) {
    while (*p && std::isspace(*p)) ++p;
    if (!*p) return *q == 0;
    if (*p != *q) return false;
    ++p;
    ++q;
  }
}

int read_fcidump_file(const char *path, Integrals *out, int *bad_line) {
  char buf[255];  // read_fcidump.c:20
  if (bad_line) *bad_line = 0;
  FILE *fp = std::fopen(path, "r");
  if (!fp) return DOCI_ERR_OPEN;
  unsigned norb = 0;
  int nelec = 0, ms2 = 0;
  if (!std::fgets(buf, sizeof buf, fp) ||
      std::sscanf(buf, " &FCI NORB= %u , NELEC= %d , MS2= %d , ", &norb, &nelec, &ms2) != 3) {
    std::fclose(fp);
    if (bad_line) *bad_line = 1;
    return DOCI_ERR_FORMAT;
  }
  if (norb == 0 || norb > 64) {
    std::fclose(fp);
    if (bad_line) *bad_line = 1;
    return norb > 64 ? DOCI_ERR_TOO_MANY_ORBITALS : DOCI_ERR_FORMAT;
  }
  out->L = static_cast<int>(norb);
  out->Na = (nelec + ms2) / 2;  // read_fcidump.c:44-45
  out->Nb = (nelec - ms2) / 2;
  out->core = 0;
  const size_t n = norb, n2 = n * n;
  out->one.assign(n2, 0.0);
  out->two.assign(n2 * n2, 0.0);
  int line = 1;
  while (std::fgets(buf, sizeof buf, fp)) {  // namelist (:53-58)
    ++line;
    if (is_namelist_end(buf, "&END") || is_namelist_end(buf, "/END") || is_namelist_end(buf, "/"))
      break;
  }
  while (std::fgets(buf, sizeof buf, fp)) {  // integrals (:60-80)
    ++line;
    double v;
    int i, j, k, l;
    if (std::sscanf(buf, " %lf %d %d %d %d ", &v, &i, &j, &k, &l) != 5) {
      std::fclose(fp);
      if (bad_line) *bad_line = line;
      return DOCI_ERR_FORMAT;
    }
    double *slot;
    auto in_range = [&](int a) { return a >= 1 && a <= static_cast<int>(n); };
    if (k != 0) {
      if (!(in_range(i) && in_range(j) && in_range(k) && in_range(l))) {
        std::fclose(fp);
        if (bad_line) *bad_line = line;
        return DOCI_ERR_FORMAT;
      }
      slot = &out->two[(size_t)(l - 1) * n2 * n + (size_t)(k - 1) * n2 + (size_t)(j - 1) * n + (i - 1)];
    } else if (i != 0) {
      if (!(in_range(i) && in_range(j))) {
        std::fclose(fp);
        if (bad_line) *bad_line = line;
        return DOCI_ERR_FORMAT;
      }
      slot = &out->one[(size_t)(j - 1) * n + (i - 1)];
    } else {
      slot = &out->core;
    }
    if (std::fabs(*slot) >= 1e-14)
      std::fprintf(stderr, "Doubly inputted value at line %d, hope you don't mind\n", line);
    *slot = v;
  }
  std::fclose(fp);
  return DOCI_OK;
}

// ---------------------------------------------------------------------------
// Relaxed reader (no counterpart in the reference).  The reference's reader
// wants the header on one line in a fixed order and propagates the 8-fold
// symmetry only from the canonical loop domain of transform_integrals, so a
// file written in another index order silently loses integrals.  This reader
// accepts what FCIDUMP writers produce: the namelist over any number of
// lines (&FCI ... &END or /), keys in any order and case, other keys
// (ORBSYM, ISYM, UHF, ...) ignored, Fortran D exponents, blank lines, and
// every two-electron entry stored at its canonical slot (i >= j, k >= l,
// i >= k, and j >= l when i == k), from which the transform propagates it.
// Two entries that name the same integral with different values are an
// error; equal repeats are accepted.
// ---------------------------------------------------------------------------
namespace {

// "KEY = value" pairs of the namelist text (commas and blanks separate)
bool namelist_int(const std::string &text, const char *key, long *value) {
  const size_t n = text.size(), kl = std::strlen(key);
  for (size_t p = 0; p + kl <= n; ++p) {
    bool match = true;
    for (size_t q = 0; q < kl && match; ++q)
      match = std::toupper(static_cast<unsigned char>(text[p + q])) == key[q];
    if (!match) continue;
    // a whole word: not preceded or followed by an identifier character
    if (p > 0 && (std::isalnum(static_cast<unsigned char>(text[p - 1])) || text[p - 1] == '_')) continue;
    size_t r = p + kl;
    while (r < n && std::isspace(static_cast<unsigned char>(text[r]))) ++r;
    if (r >= n || text[r] != '=') continue;
    ++r;
    char *end = nullptr;
    const long v = std::strtol(text.c_str() + r, &end, 10);
    if (end == text.c_str() + r) return false;
    *value = v;
    return true;
  }
  return false;
}

}  // namespace

int read_fcidump_relaxed(const char *path, Integrals *out, int *bad_line) {
  if (bad_line) *bad_line = 0;
  FILE *fp = std::fopen(path, "r");
  if (!fp) return DOCI_ERR_OPEN;
  std::string header;
  std::vector<char> buf(1 << 16);
  int line = 0;
  bool started = false, ended = false;
  while (!ended && std::fgets(buf.data(), static_cast<int>(buf.size()), fp)) {
    ++line;
    std::string s(buf.data());
    std::string up;
    for (char ch : s) up.push_back(static_cast<char>(std::toupper(static_cast<unsigned char>(ch))));
    size_t from = 0;
    if (!started) {
      const size_t at = up.find("&FCI");
      if (at == std::string::npos) {
        bool blank = true;
        for (char ch : s) blank = blank && std::isspace(static_cast<unsigned char>(ch));
        if (blank) continue;
        std::fclose(fp);
        if (bad_line) *bad_line = line;
        return DOCI_ERR_FORMAT;
      }
      started = true;
      from = at + 4;
    }
    size_t stop = up.find("&END", from);
    if (stop == std::string::npos) stop = up.find('/', from);
    if (stop != std::string::npos) {
      ended = true;
      header += up.substr(from, stop - from);
    } else {
      header += up.substr(from);
    }
    header += ' ';
  }
  long norb = 0, nelec = 0, ms2 = 0;
  if (!ended || !namelist_int(header, "NORB", &norb) || !namelist_int(header, "NELEC", &nelec)) {
    std::fclose(fp);
    if (bad_line) *bad_line = line;
    return DOCI_ERR_FORMAT;
  }
  if (!namelist_int(header, "MS2", &ms2)) ms2 = 0;
  if (norb <= 0 || norb > 64 || nelec < 0) {
    std::fclose(fp);
    if (bad_line) *bad_line = 1;
    return norb > 64 ? DOCI_ERR_TOO_MANY_ORBITALS : DOCI_ERR_FORMAT;
  }
  out->L = static_cast<int>(norb);
  out->Na = static_cast<int>((nelec + ms2) / 2);
  out->Nb = static_cast<int>((nelec - ms2) / 2);
  out->core = 0;
  const size_t n = static_cast<size_t>(norb), n2 = n * n;
  out->one.assign(n2, 0.0);
  out->two.assign(n2 * n2, 0.0);
  std::vector<unsigned char> set_two(n2 * n2, 0), set_one(n2, 0);
  bool core_set = false;
  while (std::fgets(buf.data(), static_cast<int>(buf.size()), fp)) {
    ++line;
    for (char *c = buf.data(); *c; ++c)
      if (*c == 'D' || *c == 'd') *c = 'E';  // Fortran double-precision exponent
    bool blank = true;
    for (const char *c = buf.data(); *c; ++c) blank = blank && std::isspace(static_cast<unsigned char>(*c));
    if (blank) continue;
    double v;
    int i, j, k, l;
    if (std::sscanf(buf.data(), " %lf %d %d %d %d", &v, &i, &j, &k, &l) != 5) {
      std::fclose(fp);
      if (bad_line) *bad_line = line;
      return DOCI_ERR_FORMAT;
    }
    auto in_range = [&](int a) { return a >= 1 && a <= static_cast<int>(n); };
    double *slot;
    unsigned char *flag;
    if (k != 0 || l != 0) {
      if (!(in_range(i) && in_range(j) && in_range(k) && in_range(l))) {
        std::fclose(fp);
        if (bad_line) *bad_line = line;
        return DOCI_ERR_FORMAT;
      }
      // canonical representative of the 8 index permutations of (ij|kl)
      if (i < j) std::swap(i, j);
      if (k < l) std::swap(k, l);
      if (i < k || (i == k && j < l)) {
        std::swap(i, k);
        std::swap(j, l);
      }
      const size_t at = (size_t)(l - 1) * n2 * n + (size_t)(k - 1) * n2 + (size_t)(j - 1) * n + (i - 1);
      slot = &out->two[at];
      flag = &set_two[at];
    } else if (i != 0 || j != 0) {
      if (!(in_range(i) && in_range(j))) {
        std::fclose(fp);
        if (bad_line) *bad_line = line;
        return DOCI_ERR_FORMAT;
      }
      if (i < j) std::swap(i, j);  // h is symmetric; the transform mirrors from i >= j
      const size_t at = (size_t)(j - 1) * n + (i - 1);
      slot = &out->one[at];
      flag = &set_one[at];
    } else {
      slot = &out->core;
      flag = nullptr;
    }
    const bool seen = flag ? *flag != 0 : core_set;
    if (seen && *slot != v) {
      std::fclose(fp);
      if (bad_line) *bad_line = line;
      return DOCI_ERR_FORMAT;
    }
    *slot = v;
    if (flag)
      *flag = 1;
    else
      core_set = true;
  }
  std::fclose(fp);
  return DOCI_OK;
}

void transform_integrals(double *one, double *two, int L) {
  const size_t n = L, n2 = n * n, n3 = n2 * n;
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) one[i * n + j] = one[j * n + i];
  // 8-fold symmetry, propagated from the loop domain i>=j, i>=k, k>=l only
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j)
      for (size_t k = 0; k <= i; ++k)
        for (size_t l = 0; l <= k; ++l) {
          const double v = two[i + n * j + n2 * k + n3 * l];
          if (v == 0) continue;
          two[k + n * l + n2 * i + n3 * j] = v;
          two[j + n * i + n2 * l + n3 * k] = v;
          two[l + n * k + n2 * j + n3 * i] = v;
          two[j + n * i + n2 * k + n3 * l] = v;
          two[l + n * k + n2 * i + n3 * j] = v;
          two[i + n * j + n2 * l + n3 * k] = v;
          two[k + n * l + n2 * j + n3 * i] = v;
        }
  // h'_kl = h_kl - 1/2 sum_j (kj|jl)
  for (size_t k = 0; k < n; ++k)
    for (size_t l = 0; l < n; ++l) {
      double s = 0;
      for (size_t j = 0; j < n; ++j) s += two[k + j * n + j * n2 + l * n3];
      one[k + l * n] -= 0.5 * s;
    }
}

uint32_t combination(unsigned n, unsigned m) {  // C(m, n), doci.c:687-701
  if (n > m) return 0;
  unsigned long long r = 1;
  for (unsigned d = 1; d <= n; ++d) {
    r *= m--;
    r /= d;
  }
  return static_cast<uint32_t>(r);
}

uint64_t binom64(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}

void fill_binom_table(uint32_t *t) {
  for (int n = 0; n < kBinomRows; ++n)
    for (int k = 0; k < kBinomCols; ++k) {
      const uint64_t v = binom64(n, k);
      t[n * kBinomCols + k] = v > 0xffffffffull ? 0xffffffffu : static_cast<uint32_t>(v);
    }
}

}  // namespace doci
