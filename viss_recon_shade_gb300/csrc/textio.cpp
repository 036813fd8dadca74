// textio.cpp -- the reference's whitespace-separated text files, read and
// written on the host (vissGen10M_shade.cu:198-286, 346-412, 563-583;
// shade1M.cu:108-127; MIncline_generate_uvw_float.cu:418-427).
//
// Reading: the file is read into memory, split at line boundaries into one
// chunk per hardware thread, and each chunk is parsed with std::from_chars; the
// chunks' values are then stored in parallel at their place in file order.
// Writing: values are formatted as std::ostream formats a float by default
// (printf "%g", 6 significant digits: std::to_chars with the general format and
// precision 6, which C++17 specifies to match it), chunk-parallel into one
// pre-populated buffer, then written in order.
#include <charconv>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <algorithm>
#include <functional>
#include <memory>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "viss_gb300.h"

namespace viss {
int fail(int status, const std::string& msg);
}

namespace {

// The file's bytes: mapped read-only with its pages populated up front (first
// touches from many threads would serialise on page faults), or read into a
// buffer where mapping is not possible (an empty or special file).
struct FileBuf {
  const char* data = nullptr;
  size_t size = 0;
  void* map = nullptr;
  std::unique_ptr<char[]> own;
  ~FileBuf() {
    if (map) munmap(map, size);
  }
};

int read_all(const char* path, FileBuf& buf) {
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return viss::fail(VISS_ERR_IO, std::string("cannot open ") + path);
  struct stat st;
  if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
    void* m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
    if (m != MAP_FAILED) {
      close(fd);
      buf.map = m;
      buf.size = (size_t)st.st_size;
      buf.data = static_cast<const char*>(m);
      return VISS_OK;
    }
  }
  std::string acc;
  char tmp[1 << 16];
  for (;;) {
    const ssize_t got = read(fd, tmp, sizeof(tmp));
    if (got < 0) {
      close(fd);
      return viss::fail(VISS_ERR_IO, std::string("read error ") + path);
    }
    if (got == 0) break;
    acc.append(tmp, (size_t)got);
  }
  close(fd);
  buf.size = acc.size();
  buf.own.reset(new char[buf.size + 1]);
  if (buf.size) std::memcpy(buf.own.get(), acc.data(), buf.size);
  buf.data = buf.own.get();
  return VISS_OK;
}

unsigned host_threads() { return std::max(1u, std::min(32u, std::thread::hardware_concurrency())); }

// fn(c) for c in [0, n) on n threads (n = 1: inline)
template <class F>
void parallel_chunks(unsigned n, F fn) {
  if (n <= 1) {
    fn(0u);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(n);
  for (unsigned c = 0; c < n; ++c) th.emplace_back([&fn, c] { fn(c); });
  for (auto& t : th) t.join();
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

// Parses whitespace-separated numbers of [b, e) into out (T = float or int).
// Returns false at the first token that does not parse (the reference's
// `while (file >> a >> b ...)` stops there too).
template <class T>
bool parse_range(const char* b, const char* e, std::vector<T>& out) {
  const char* p = b;
  while (true) {
    while (p < e && is_space(*p)) ++p;
    if (p >= e) return true;
    T v{};
    const char* q = p;
    if (*q == '+') ++q;  // from_chars does not accept a leading '+'
    auto r = std::from_chars(q, e, v);
    if (r.ec != std::errc()) {
      if constexpr (std::is_same<T, int>::value) {
        // integer columns written as floats ("12" or "12.0" or "1e+06")
        float fv;
        auto r2 = std::from_chars(q, e, fv);
        if (r2.ec != std::errc()) return false;
        v = (int)fv;
        r = r2;
      } else {
        return false;
      }
    }
    out.push_back(v);
    p = r.ptr;
  }
}

// The numbers of [b, e) after `skip_tokens` header tokens, parsed per chunk of
// whole lines; chunks after the first one holding an unparsable token are
// dropped (that chunk keeps its values before the token).  off[c] = values in
// chunks before c; off.back() = the total.
template <class T>
void parse_numbers(const char* b, const char* e, size_t skip_tokens, std::vector<std::vector<T>>& part,
                   std::vector<int64_t>& off) {
  for (size_t t = 0; t < skip_tokens; ++t) {
    while (b < e && is_space(*b)) ++b;
    while (b < e && !is_space(*b)) ++b;
  }
  const size_t n = (size_t)(e - b);
  const unsigned chunks = n < (1u << 20) ? 1u : host_threads();
  std::vector<const char*> cut(chunks + 1);
  cut[0] = b;
  cut[chunks] = e;
  for (unsigned c = 1; c < chunks; ++c) {
    const char* p = b + n * c / chunks;
    while (p < e && *p != '\n') ++p;
    cut[c] = p;
  }
  part.assign(chunks, {});
  std::vector<char> ok(chunks, 1);
  parallel_chunks(chunks, [&](unsigned c) {
    part[c].reserve((size_t)(cut[c + 1] - cut[c]) / 4 + 16);
    ok[c] = parse_range(cut[c], cut[c + 1], part[c]);
  });
  for (unsigned c = 0; c < chunks; ++c)
    if (!ok[c]) { part.resize(c + 1); break; }
  off.assign(part.size() + 1, 0);
  for (size_t c = 0; c < part.size(); ++c) off[c + 1] = off[c] + (int64_t)part[c].size();
}

// Files of one row per line (the reference's files as written): chunks of whole
// lines count their non-blank lines, then parse straight into out at their first
// row, out[col * cap + row] (columnar) or out[row * ncols + col].  Returns false,
// having stored nothing meaningful, unless every non-blank line holds exactly
// ncols numbers: the general parse then decides (it stops where the reference's
// stream extraction stops).  *rows_out = the rows; a row count above cap returns
// true with nothing stored (the caller reports it).
template <class T>
bool parse_rows_direct(const char* b, const char* e, int ncols, T* out, int64_t cap, bool columnar,
                       int64_t* rows_out) {
  const size_t n = (size_t)(e - b);
  const unsigned chunks = n < (1u << 20) ? 1u : host_threads();
  std::vector<const char*> cut(chunks + 1);
  cut[0] = b;
  cut[chunks] = e;
  for (unsigned c = 1; c < chunks; ++c) {
    const char* p = b + n * c / chunks;
    while (p < e && *p != '\n') ++p;
    cut[c] = p < e ? p + 1 : e;
  }
  std::vector<int64_t> lines(chunks + 1, 0);
  parallel_chunks(chunks, [&](unsigned c) {
    int64_t cnt = 0;
    bool content = false;
    for (const char* p = cut[c]; p < cut[c + 1]; ++p) {
      if (*p == '\n') {
        cnt += content;
        content = false;
      } else if (!is_space(*p)) {
        content = true;
      }
    }
    lines[c + 1] = cnt + content;
  });
  for (unsigned c = 0; c < chunks; ++c) lines[c + 1] += lines[c];
  *rows_out = lines[chunks];
  if (!out || lines[chunks] > cap) return true;
  std::vector<char> ok(chunks, 1);
  parallel_chunks(chunks, [&](unsigned c) {
    int64_t row = lines[c];
    const char* p = cut[c];
    const char* end = cut[c + 1];
    while (p < end) {
      while (p < end && is_space(*p)) ++p;  // blank lines and leading blanks
      if (p >= end) break;
      for (int k = 0; k < ncols; ++k) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
        T v{};
        const char* q = p < end && *p == '+' ? p + 1 : p;
        auto r = std::from_chars(q, end, v);
        if (r.ec != std::errc()) {
          ok[c] = 0;
          return;
        }
        if (columnar) out[(int64_t)k * cap + row] = v;
        else out[row * ncols + k] = v;
        p = r.ptr;
      }
      while (p < end && *p != '\n') {
        if (!is_space(*p)) {  // more numbers on the line than columns
          ok[c] = 0;
          return;
        }
        ++p;
      }
      ++row;
    }
  });
  for (unsigned c = 0; c < chunks; ++c)
    if (!ok[c]) return false;
  return true;
}

// "%g" as std::ostream prints a float by default
inline int fmt_g(char* out, float v) {
  return (int)(std::to_chars(out, out + 32, v, std::chars_format::general, 6).ptr - out);
}

// Rows formatted chunk-parallel into one anonymous mapping populated up front
// (16 bytes per value bound a %g float and its separator), each chunk in its own
// slice, then written in order with writev.
int write_rows(const char* path, int64_t nrows, int ncols, const std::function<float(int64_t, int)>& get) {
  const unsigned chunks = nrows < 65536 ? 1u : host_threads();
  const size_t per_row = (size_t)ncols * 16;
  const size_t cap = (size_t)(nrows > 0 ? nrows : 1) * per_row;
  void* m = mmap(nullptr, cap, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_POPULATE, -1, 0);
  if (m == MAP_FAILED) return viss::fail(VISS_ERR_IO, "no memory to format " + std::string(path));
  char* const base = static_cast<char*>(m);
  std::vector<size_t> start(chunks), len(chunks, 0);
  parallel_chunks(chunks, [&](unsigned c) {
    const int64_t r0 = nrows * c / chunks, r1 = nrows * (c + 1) / chunks;
    start[c] = (size_t)r0 * per_row;
    char* p = base + start[c];
    for (int64_t r = r0; r < r1; ++r) {
      for (int k = 0; k < ncols; ++k) {
        p += fmt_g(p, get(r, k));
        *p++ = k + 1 < ncols ? ' ' : '\n';
      }
    }
    len[c] = (size_t)(p - (base + start[c]));
  });
  int rc = VISS_OK;
  const int fd = open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) {
    rc = viss::fail(VISS_ERR_IO, std::string("cannot write ") + path);
  } else {
    for (unsigned c = 0; c < chunks && rc == VISS_OK; ++c) {
      size_t done = 0;
      while (done < len[c]) {
        const ssize_t w = write(fd, base + start[c] + done, len[c] - done);
        if (w <= 0) {
          rc = viss::fail(VISS_ERR_IO, std::string("short write ") + path);
          break;
        }
        done += (size_t)w;
      }
    }
    if (close(fd) != 0 && rc == VISS_OK) rc = viss::fail(VISS_ERR_IO, std::string("close failed ") + path);
  }
  munmap(m, cap);
  return rc;
}

}  // namespace

extern "C" {

int viss_text_read_floats(const char* path, int header, int ncols, float* out, int64_t cap, int64_t* nrows,
                          int64_t* header_value) {
  if (!path || !nrows || ncols < 1) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  FileBuf buf;
  int rc = read_all(path, buf);
  if (rc) return rc;
  const char* b = buf.data;
  const char* e = b + buf.size;
  if (header && header_value) {
    const char* p = b;
    while (p < e && is_space(*p)) ++p;
    long long hv = 0;
    auto r = std::from_chars(p, e, hv);
    if (r.ec != std::errc()) return viss::fail(VISS_ERR_FORMAT, std::string("bad header in ") + path);
    *header_value = hv;
  }
  if (header) {  // the header token is not a row
    while (b < e && is_space(*b)) ++b;
    while (b < e && !is_space(*b)) ++b;
  }
  int64_t direct_rows = 0;
  if (parse_rows_direct(b, e, ncols, out, cap, true, &direct_rows)) {
    *nrows = direct_rows;
    if (out && direct_rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    return VISS_OK;
  }
  std::vector<std::vector<float>> part;
  std::vector<int64_t> off;
  parse_numbers(b, e, 0, part, off);
  const int64_t rows = off.back() / ncols;
  *nrows = rows;
  if (out) {
    if (rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    // value k of the file -> row k / ncols, column k % ncols (whole rows only)
    parallel_chunks((unsigned)part.size(), [&](unsigned c) {
      const int64_t k0 = off[c];
      int64_t r = k0 / ncols;
      int col = (int)(k0 % ncols);
      for (const float v : part[c]) {
        if (r >= rows) break;
        out[col * cap + r] = v;
        if (++col == ncols) { col = 0; ++r; }
      }
    });
  }
  return VISS_OK;
}

int viss_text_read_ints(const char* path, int ncols, int32_t* out, int64_t cap, int64_t* nrows) {
  if (!path || !nrows || ncols < 1) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  FileBuf buf;
  int rc = read_all(path, buf);
  if (rc) return rc;
  int64_t direct_rows = 0;
  if (parse_rows_direct(buf.data, buf.data + buf.size, ncols, out, cap, false, &direct_rows)) {
    *nrows = direct_rows;
    if (out && direct_rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    return VISS_OK;
  }
  std::vector<std::vector<int>> part;
  std::vector<int64_t> off;
  parse_numbers(buf.data, buf.data + buf.size, 0, part, off);
  const int64_t rows = off.back() / ncols;
  *nrows = rows;
  if (out) {
    if (rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    const int64_t total = rows * ncols;
    parallel_chunks((unsigned)part.size(), [&](unsigned c) {
      const int64_t k0 = off[c];
      const int64_t cnt = std::min<int64_t>((int64_t)part[c].size(), std::max<int64_t>(0, total - k0));
      if (cnt > 0) std::memcpy(out + k0, part[c].data(), sizeof(int32_t) * (size_t)cnt);
    });
  }
  return VISS_OK;
}

int viss_text_write_floats(const char* path, int ncols, const float* cols, int64_t stride, int64_t nrows) {
  if (!path || ncols < 1 || nrows < 0 || (!cols && nrows)) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  return write_rows(path, nrows, ncols, [&](int64_t r, int c) { return cols[c * stride + r]; });
}

int viss_text_write_ints(const char* path, int ncols, const int32_t* rows, int64_t nrows) {
  if (!path || ncols < 1 || nrows < 0 || (!rows && nrows)) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  // written through float as the reference's shadeM writer does (shade1M.cu:118-121)
  return write_rows(path, nrows, ncols, [&](int64_t r, int c) { return (float)rows[r * ncols + c]; });
}

}  // extern "C"
