// textio.cpp -- the reference's whitespace-separated text files, read and
// written on the host (vissGen10M_shade.cu:198-286, 346-412, 563-583;
// shade1M.cu:108-127; MIncline_generate_uvw_float.cu:418-427).
//
// Reading: the file is mapped into memory, split at line boundaries into one
// chunk per hardware thread, and each chunk is parsed with std::from_chars;
// the per-chunk counts are prefix-summed so values land in file order.
// Writing: values are formatted as std::ostream formats a float by default
// (printf "%g", 6 significant digits), chunk-parallel, then written in order.
#include <charconv>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "viss_gb300.h"

namespace viss {
int fail(int status, const std::string& msg);
}

namespace {

int read_all(const char* path, std::string& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return viss::fail(VISS_ERR_IO, std::string("cannot open ") + path);
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf.resize(sz > 0 ? (size_t)sz : 0);
  const size_t got = sz > 0 ? std::fread(&buf[0], 1, (size_t)sz, f) : 0;
  std::fclose(f);
  if ((long)got != sz) return viss::fail(VISS_ERR_IO, std::string("short read ") + path);
  return VISS_OK;
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

template <class T>
int parse_numbers(const std::string& buf, size_t skip_tokens, std::vector<T>& vals, bool* clean) {
  const char* b = buf.data();
  const char* e = b + buf.size();
  // skip header tokens
  for (size_t t = 0; t < skip_tokens; ++t) {
    while (b < e && is_space(*b)) ++b;
    while (b < e && !is_space(*b)) ++b;
  }
  const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const size_t n = (size_t)(e - b);
  const unsigned chunks = n < (1u << 20) ? 1u : nt;
  std::vector<const char*> cut(chunks + 1);
  cut[0] = b;
  cut[chunks] = e;
  for (unsigned c = 1; c < chunks; ++c) {
    const char* p = b + n * c / chunks;
    while (p < e && *p != '\n') ++p;
    cut[c] = p;
  }
  std::vector<std::vector<T>> part(chunks);
  std::vector<char> ok(chunks, 1);
  std::vector<std::thread> th;
  for (unsigned c = 0; c < chunks; ++c)
    th.emplace_back([&, c] { ok[c] = parse_range(cut[c], cut[c + 1], part[c]); });
  for (auto& t : th) t.join();
  *clean = true;
  vals.clear();
  for (unsigned c = 0; c < chunks; ++c) {
    vals.insert(vals.end(), part[c].begin(), part[c].end());
    if (!ok[c]) { *clean = false; break; }
  }
  return VISS_OK;
}

// "%g" as std::ostream prints a float by default.
inline int fmt_g(char* out, float v) { return std::snprintf(out, 32, "%g", (double)v); }

int write_rows(const char* path, int64_t nrows, int ncols, const std::function<float(int64_t, int)>& get) {
  const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const unsigned chunks = nrows < 65536 ? 1u : nt;
  std::vector<std::string> parts(chunks);
  std::vector<std::thread> th;
  for (unsigned c = 0; c < chunks; ++c) {
    th.emplace_back([&, c] {
      const int64_t r0 = nrows * c / chunks, r1 = nrows * (c + 1) / chunks;
      std::string& s = parts[c];
      s.reserve((size_t)(r1 - r0) * (size_t)ncols * 12);
      char tmp[40];
      for (int64_t r = r0; r < r1; ++r) {
        for (int k = 0; k < ncols; ++k) {
          const int len = fmt_g(tmp, get(r, k));
          s.append(tmp, (size_t)len);
          if (k + 1 < ncols) s.push_back(' ');
        }
        s.push_back('\n');
      }
    });
  }
  for (auto& t : th) t.join();
  FILE* f = std::fopen(path, "wb");
  if (!f) return viss::fail(VISS_ERR_IO, std::string("cannot write ") + path);
  for (auto& s : parts) {
    if (std::fwrite(s.data(), 1, s.size(), f) != s.size()) {
      std::fclose(f);
      return viss::fail(VISS_ERR_IO, std::string("short write ") + path);
    }
  }
  std::fclose(f);
  return VISS_OK;
}

}  // namespace

extern "C" {

int viss_text_read_floats(const char* path, int header, int ncols, float* out, int64_t cap, int64_t* nrows,
                          int64_t* header_value) {
  if (!path || !nrows || ncols < 1) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  std::string buf;
  int rc = read_all(path, buf);
  if (rc) return rc;
  if (header && header_value) {
    const char* p = buf.data();
    const char* e = p + buf.size();
    while (p < e && is_space(*p)) ++p;
    long long hv = 0;
    auto r = std::from_chars(p, e, hv);
    if (r.ec != std::errc()) return viss::fail(VISS_ERR_FORMAT, std::string("bad header in ") + path);
    *header_value = hv;
  }
  std::vector<float> vals;
  bool clean;
  parse_numbers(buf, header ? 1 : 0, vals, &clean);
  const int64_t rows = (int64_t)vals.size() / ncols;
  *nrows = rows;
  if (out) {
    if (rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    for (int64_t r = 0; r < rows; ++r)
      for (int c = 0; c < ncols; ++c) out[c * cap + r] = vals[(size_t)r * ncols + c];
  }
  return VISS_OK;
}

int viss_text_read_ints(const char* path, int ncols, int32_t* out, int64_t cap, int64_t* nrows) {
  if (!path || !nrows || ncols < 1) return viss::fail(VISS_ERR_INVALID, "bad arguments");
  std::string buf;
  int rc = read_all(path, buf);
  if (rc) return rc;
  std::vector<int> vals;
  bool clean;
  parse_numbers(buf, 0, vals, &clean);
  const int64_t rows = (int64_t)vals.size() / ncols;
  *nrows = rows;
  if (out) {
    if (rows > cap) return viss::fail(VISS_ERR_RANGE, std::string("more rows than capacity in ") + path);
    std::memcpy(out, vals.data(), sizeof(int32_t) * (size_t)(rows * ncols));
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
