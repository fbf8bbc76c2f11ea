// Matrix Market (.mtx) and FROSTT (.tns) readers for 2-D tensors, producing the COO records
// that tacogb_pack_csr turns into CSR on the GPU.  They follow taco's readers:
//
//   readMTX (src/storage/file_io_mtx.cpp:38-77, 79-149, 159-215): header "%%MatrixMarket
//     matrix|tensor coordinate|array real general|symmetric"; comment lines start with '%';
//     the size line holds the dimensions (and, for coordinate files, the entry count);
//     coordinates are 1-based; a symmetric file's off-diagonal entries are inserted mirrored as
//     well; an array file lists every entry in column-major order.
//   readTNS (src/storage/file_io_tns.cpp:37-85): one "i j value" line per entry, 1-based, each
//     dimension the largest coordinate seen.
//
// Values go through strtod as in taco, so they are bit-identical to what taco inserts.  The
// file is read whole and its lines are parsed by all host threads, each over a contiguous range
// of lines, so the records keep the file's order (which sets the order duplicates are summed
// in by the pack).  Unlike taco, blank lines are skipped (taco would insert an entry at -1).

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "taco_gb300.h"
#include "threads.h"

namespace tacogb {
void set_error(int code, const char* fmt, ...);
}

namespace {

struct Lines {
  std::vector<const char*> start;  // first character of every non-blank line
};

// End of the line starting at p (its '\n' or the buffer's terminator).
const char* line_end(const char* p) {
  while (*p && *p != '\n') p++;
  return p;
}

// Next token start on the line [p, e), or nullptr when the line has no more tokens (strtol and
// strtod would otherwise skip the newline and read the next line).
const char* next_token(const char* p, const char* e) {
  while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
  return p < e ? p : nullptr;
}

bool blank(const char* p, const char* e) {
  for (; p < e; p++)
    if (*p != ' ' && *p != '\t' && *p != '\r') return false;
  return true;
}

// Start of every non-blank line of [b, e).
void split_lines(const char* b, const char* e, Lines& out) {
  const char* p = b;
  while (p < e) {
    const char* q = (const char*)memchr(p, '\n', (size_t)(e - p));
    if (!q) q = e;
    if (!blank(p, q)) out.start.push_back(p);
    p = q + 1;
  }
}

int read_file(const char* path, std::string& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    tacogb::set_error(TACOGB_ERR_ARG, "read: cannot open %s: %s", path, strerror(errno));
    return TACOGB_ERR_ARG;
  }
  fseek(f, 0, SEEK_END);
  const long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf.resize(sz > 0 ? (size_t)sz : 0);
  const size_t got = sz > 0 ? fread(&buf[0], 1, (size_t)sz, f) : 0;
  fclose(f);
  if ((long)got != sz) {
    tacogb::set_error(TACOGB_ERR_ARG, "read: short read of %s", path);
    return TACOGB_ERR_ARG;
  }
  buf.push_back('\0');  // strtol/strtod stop at the terminator
  return 0;
}

// Parses lines [l0, l1) as "i j value" (1-based) into r/c/v[0 .. l1-l0) and the largest
// coordinates into maxc; false on a malformed line or a coordinate outside [1, INT32_MAX].
bool parse_entries(const std::vector<const char*>& lines, size_t l0, size_t l1, int order,
                   int32_t* r, int32_t* c, double* v, bool with_value, int64_t* maxc) {
  int64_t m0 = 0, m1 = 0;
  for (size_t l = l0; l < l1; l++) {
    const char* e = line_end(lines[l]);
    const char* p = lines[l];
    long idx[2] = {0, 0};
    for (int k = 0; k < order; k++) {
      p = next_token(p, e);
      if (!p) return false;
      char* q = nullptr;
      idx[k] = strtol(p, &q, 10);
      if (q == p || idx[k] < 1 || idx[k] > INT32_MAX) return false;
      p = q;
    }
    r[l - l0] = (int32_t)(idx[0] - 1);
    c[l - l0] = (int32_t)(idx[1] - 1);
    // a line without a value reads as 0, as taco's strtod on the line alone gives
    const char* vp = next_token(p, e);
    v[l - l0] = !with_value ? 1.0 : vp ? strtod(vp, nullptr) : 0.0;
    m0 = std::max<int64_t>(m0, idx[0]);
    m1 = std::max<int64_t>(m1, idx[1]);
  }
  maxc[0] = m0;
  maxc[1] = m1;
  return true;
}

int nthreads_for(size_t lines) {
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t t = std::min<size_t>(hw ? hw : 4, std::max<size_t>(1, lines / 65536));
  return (int)std::max<size_t>(1, t);
}

// Parses every entry line in parallel; r/c/v sized lines.size().
bool parse_parallel(const std::vector<const char*>& lines, int order, int32_t* r, int32_t* c,
                    double* v, int64_t* maxc) {
  const size_t n = lines.size();
  const int T = nthreads_for(n);
  std::vector<int64_t> mx(2 * T, 0);
  std::vector<char> ok(T, 1);
  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) {
    const size_t a = n * t / T, b = n * (t + 1) / T;
    th.emplace_back([&, t, a, b] {
      tacogb::spread_thread();
      ok[t] = parse_entries(lines, a, b, order, r + a, c + a, v + a, true, &mx[2 * t]);
    });
  }
  for (auto& x : th) x.join();
  maxc[0] = maxc[1] = 0;
  for (int t = 0; t < T; t++) {
    if (!ok[t]) return false;
    maxc[0] = std::max(maxc[0], mx[2 * t]);
    maxc[1] = std::max(maxc[1], mx[2 * t + 1]);
  }
  return true;
}

struct Coo {
  int32_t rows = 0, cols = 0;
  std::vector<int32_t> r, c;
  std::vector<double> v;
};

int fail(const char* fmt, const char* what) {
  tacogb::set_error(TACOGB_ERR_ARG, fmt, what);
  return TACOGB_ERR_ARG;
}

// Inserts the mirror (c, r) right after every off-diagonal entry, as taco's symmetric read does.
void mirror(Coo& m) {
  const size_t n = m.r.size();
  size_t extra = 0;
  for (size_t i = 0; i < n; i++) extra += m.r[i] != m.c[i];
  std::vector<int32_t> r2, c2;
  std::vector<double> v2;
  r2.reserve(n + extra);
  c2.reserve(n + extra);
  v2.reserve(n + extra);
  for (size_t i = 0; i < n; i++) {
    r2.push_back(m.r[i]);
    c2.push_back(m.c[i]);
    v2.push_back(m.v[i]);
    if (m.r[i] != m.c[i]) {
      r2.push_back(m.c[i]);
      c2.push_back(m.r[i]);
      v2.push_back(m.v[i]);
    }
  }
  m.r.swap(r2);
  m.c.swap(c2);
  m.v.swap(v2);
}

int read_mtx(const std::vector<const char*>& lines, Coo& m) {
  char head[64] = {0}, type[64] = {0}, format[64] = {0}, field[64] = {0}, symmetry[64] = {0};
  if (sscanf(lines[0], "%63s %63s %63s %63s %63s", head, type, format, field, symmetry) != 5)
    return fail("read: %s", "malformed MatrixMarket header");
  if (strcmp(type, "matrix") != 0 && strcmp(type, "tensor") != 0)
    return fail("read: MatrixMarket type %s not available", type);
  if (strcmp(field, "real") != 0)
    return fail("read: MatrixMarket field %s not available (taco reads real only)", field);
  if (strcmp(symmetry, "general") != 0 && strcmp(symmetry, "symmetric") != 0)
    return fail("read: MatrixMarket symmetry %s not available", symmetry);
  const bool symm = strcmp(symmetry, "symmetric") == 0;
  size_t l = 1;
  while (l < lines.size() && lines[l][0] == '%') l++;
  if (l == lines.size()) return fail("read: %s", "no size line");
  std::vector<long> dims;
  {
    const char* e = line_end(lines[l]);
    const char* p = lines[l];
    while ((p = next_token(p, e)) != nullptr) {  // taco: strtoul until it reads 0
      char* q = nullptr;
      const long d = strtol(p, &q, 10);
      if (q == p || d <= 0) break;
      dims.push_back(d);
      p = q;
    }
  }
  l++;
  if (strcmp(format, "coordinate") == 0) {
    if (dims.size() != 3) return fail("read: %s", "a 2-D coordinate file needs rows cols nnz");
    const size_t nnz = (size_t)dims[2];
    if (lines.size() - l < nnz) return fail("read: %s", "fewer entry lines than declared");
    std::vector<const char*> ent(lines.begin() + l, lines.begin() + l + nnz);
    m.r.resize(nnz);
    m.c.resize(nnz);
    m.v.resize(nnz);
    int64_t mx[2];
    if (!parse_parallel(ent, 2, m.r.data(), m.c.data(), m.v.data(), mx))
      return fail("read: %s", "malformed entry line");
    if (mx[0] > dims[0] || mx[1] > dims[1]) return fail("read: %s", "entry outside the matrix");
  } else if (strcmp(format, "array") == 0) {
    if (dims.size() != 2) return fail("read: %s", "a 2-D array file needs rows cols");
    const size_t total = (size_t)dims[0] * (size_t)dims[1];
    if (lines.size() - l < total) return fail("read: %s", "fewer values than rows x cols");
    m.r.resize(total);
    m.c.resize(total);
    m.v.resize(total);
    for (size_t k = 0; k < total; k++) {  // column-major, as taco's readDense
      m.r[k] = (int32_t)(k % (size_t)dims[0]);
      m.c[k] = (int32_t)(k / (size_t)dims[0]);
      const char* vp = next_token(lines[l + k], line_end(lines[l + k]));
      m.v[k] = vp ? strtod(vp, nullptr) : 0.0;
    }
  } else {
    return fail("read: MatrixMarket format %s not available", format);
  }
  if (dims[0] > INT32_MAX || dims[1] > INT32_MAX) return fail("read: %s", "dimension too large");
  m.rows = (int32_t)dims[0];
  m.cols = (int32_t)dims[1];
  if (symm) {
    if (m.rows != m.cols) return fail("read: %s", "a symmetric matrix must be square");
    mirror(m);
  }
  return 0;
}

int read_tns(const std::vector<const char*>& lines, Coo& m) {
  // order: whitespace-separated tokens of the first line, minus the value
  int tokens = 0;
  for (const char* p = lines[0]; *p && *p != '\n';) {
    while (*p == ' ' || *p == '\t' || *p == '\r') p++;
    if (!*p || *p == '\n') break;
    tokens++;
    while (*p && *p != ' ' && *p != '\t' && *p != '\r' && *p != '\n') p++;
  }
  if (tokens - 1 != 2) return fail("read: %s", "only 2-D .tns files (i j value) are read");
  const size_t n = lines.size();
  m.r.resize(n);
  m.c.resize(n);
  m.v.resize(n);
  int64_t mx[2];
  if (!parse_parallel(lines, 2, m.r.data(), m.c.data(), m.v.data(), mx))
    return fail("read: %s", "malformed entry line");
  m.rows = (int32_t)mx[0];
  m.cols = (int32_t)mx[1];
  return 0;
}

template <typename T>
T* to_malloc(const std::vector<T>& v) {
  T* p = (T*)malloc(std::max<size_t>(1, v.size()) * sizeof(T));
  if (p && !v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

// Rutherford-Boeing, as taco's readRB loads it (src/storage/file_io_rb.cpp:22-88, 142-228,
// 246-283, 319-350): real unsymmetric assembled matrices only (type RUA, any case), loaded as CSC.
// Line 2 gives the line counts of the sections (pointers, row indices, values); a fifth header
// line follows when right-hand sides are present; within each section every whitespace-separated
// token of the section's lines is read in order (1-based pointers and indices become 0-based).
int read_rb(const std::vector<const char*>& lines, int32_t* rows, int32_t* cols,
            std::vector<int32_t>& colptr, std::vector<int32_t>& rowidx, std::vector<double>& vals) {
  if (lines.size() < 4) return fail("read: %s", "a Rutherford-Boeing file needs four header lines");
  long cnt[5] = {0, 0, 0, 0, 0};
  const char* p = lines[1];
  const char* e = line_end(p);
  for (int k = 0; k < 5; k++) {
    const char* t = next_token(p, e);
    if (!t) return fail("read: %s", "the second header line needs five line counts");
    char* end;
    cnt[k] = strtol(t, &end, 10);
    p = end;
  }
  p = lines[2];
  e = line_end(p);
  const char* t = next_token(p, e);
  if (!t || e - t < 3 || (t[0] != 'R' && t[0] != 'r') || (t[1] != 'U' && t[1] != 'u') ||
      (t[2] != 'A' && t[2] != 'a'))
    return fail("read: %s", "only real unsymmetric assembled (RUA) Rutherford-Boeing matrices");
  p = t + 3;
  long dims[3];
  for (int k = 0; k < 3; k++) {
    t = next_token(p, e);
    if (!t) return fail("read: %s", "the third header line needs rows, columns and entries");
    char* end;
    dims[k] = strtol(t, &end, 10);
    p = end;
  }
  if (dims[0] < 0 || dims[1] < 0 || dims[2] < 0 || dims[0] > INT32_MAX || dims[1] > INT32_MAX ||
      dims[2] > INT32_MAX)
    return fail("read: %s", "sizes out of range");
  size_t l = cnt[4] > 0 ? 5 : 4;  // the right-hand side header line, when present, is skipped
  auto section = [&](long nlines, auto&& take) -> bool {
    for (long k = 0; k < nlines; k++, l++) {
      if (l >= lines.size()) return false;
      const char* q = lines[l];
      const char* qe = line_end(q);
      while (const char* tok = next_token(q, qe)) {
        char* end;
        take(tok, &end);
        if (end == tok) return false;
        q = end;
      }
    }
    return true;
  };
  colptr.clear();
  rowidx.clear();
  vals.clear();
  if (!section(cnt[1], [&](const char* tok, char** end) {
        colptr.push_back((int32_t)strtol(tok, end, 10) - 1);
      }) ||
      !section(cnt[2], [&](const char* tok, char** end) {
        rowidx.push_back((int32_t)strtol(tok, end, 10) - 1);
      }) ||
      !section(cnt[3], [&](const char* tok, char** end) { vals.push_back(strtod(tok, end)); }))
    return fail("read: %s", "a Rutherford-Boeing section is shorter than its header says");
  if ((long)colptr.size() != dims[1] + 1 || (long)rowidx.size() != dims[2] ||
      (long)vals.size() != dims[2] || colptr.front() != 0 || colptr.back() != dims[2])
    return fail("read: %s", "Rutherford-Boeing sections do not match the header's sizes");
  *rows = (int32_t)dims[0];
  *cols = (int32_t)dims[1];
  return 0;
}

}  // namespace

extern "C" int tacogb_read_rb(const char* path, int32_t* rows, int32_t* cols, int64_t* nnz,
                              int32_t** colptr, int32_t** rowidx, double** vals) {
  if (!path || !rows || !cols || !nnz || !colptr || !rowidx || !vals)
    return fail("read: %s", "null argument");
  std::string buf;
  if (int rc = read_file(path, buf)) return rc;
  Lines L;
  split_lines(buf.data(), buf.data() + buf.size() - 1, L);
  std::vector<int32_t> cp, ri;
  std::vector<double> v;
  if (int rc = read_rb(L.start, rows, cols, cp, ri, v)) return rc;
  *colptr = to_malloc(cp);
  *rowidx = to_malloc(ri);
  *vals = to_malloc(v);
  if (!*colptr || !*rowidx || !*vals) {
    free(*colptr);
    free(*rowidx);
    free(*vals);
    return fail("read: %s", "out of host memory");
  }
  *nnz = (int64_t)ri.size();
  return 0;
}

extern "C" int tacogb_read_coo(const char* path, int32_t* rows, int32_t* cols, int64_t* n,
                               int32_t** coord_rows, int32_t** coord_cols, double** vals) {
  if (!path || !rows || !cols || !n || !coord_rows || !coord_cols || !vals)
    return fail("read: %s", "null argument");
  std::string buf;
  if (int rc = read_file(path, buf)) return rc;
  Lines L;
  split_lines(buf.data(), buf.data() + buf.size() - 1, L);
  Coo m;
  if (L.start.empty()) {
    m.rows = m.cols = 0;
  } else if (strncmp(L.start[0], "%%MatrixMarket", 14) == 0) {
    if (int rc = read_mtx(L.start, m)) return rc;
  } else {
    if (int rc = read_tns(L.start, m)) return rc;
  }
  *coord_rows = to_malloc(m.r);
  *coord_cols = to_malloc(m.c);
  *vals = to_malloc(m.v);
  if (!*coord_rows || !*coord_cols || !*vals) {
    free(*coord_rows);
    free(*coord_cols);
    free(*vals);
    return fail("read: %s", "out of host memory");
  }
  *rows = m.rows;
  *cols = m.cols;
  *n = (int64_t)m.r.size();
  return 0;
}

extern "C" void tacogb_free_host(void* p) { free(p); }
