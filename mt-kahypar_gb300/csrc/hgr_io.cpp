// hMetis hypergraph and partition files: lpgpu_read_hgr, lpgpu_read_partition,
// lpgpu_write_partition, lpgpu_free.
//
// Format (the reference reader's rules, io/hypergraph_io.cpp:95-333): lines
// starting with '%' are comments; the header is "num_nets num_vertices
// [type]" with type 1 = net weights, 10 = vertex weights, 11 = both; then one
// line per net (its weight first when the type has net weights, then its pins,
// 1-based); a net line with fewer than two pins is dropped (the reference
// removes single-pin nets); then, when the type has vertex weights, one weight
// per vertex. A partition file holds one block id per line
// (io::writePartitionFile, hypergraph_io.cpp:350-365).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lpgpu.h"

namespace lpgpu {
void set_error(const std::string& msg);
}

namespace {

lpgpu_status fail(const std::string& msg) {
  lpgpu::set_error(msg);
  return LPGPU_ERR_INVALID_ARG;
}

bool read_file(const char* path, std::vector<char>& buf, std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open ") + path + ": " + std::strerror(errno);
    return false;
  }
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf.resize(len > 0 ? (size_t)len : 0);
  const size_t got = len > 0 ? std::fread(buf.data(), 1, (size_t)len, f) : 0;
  std::fclose(f);
  if (got != buf.size()) {
    err = std::string("short read of ") + path;
    return false;
  }
  return true;
}

// Cursor over the file's text, one line at a time.
struct Text {
  const char* p;
  const char* end;
  int64_t line = 0;  // 1-based number of the line `p` is in

  bool done() const { return p >= end; }
  // Moves to the start of the next line that is not a comment; false at EOF.
  bool next_content_line() {
    while (p < end && *p == '%') skip_line();
    return p < end;
  }
  void skip_line() {
    while (p < end && *p != '\n') ++p;
    if (p < end) ++p;
    ++line;
  }
  // Reads the unsigned integers of the current line into `out` and moves past it.
  bool line_numbers(std::vector<int64_t>& out) {
    out.clear();
    while (p < end && *p != '\n') {
      const char ch = *p;
      if (ch == ' ' || ch == '\t' || ch == '\r') {
        ++p;
        continue;
      }
      if (ch < '0' || ch > '9') return false;
      int64_t x = 0;
      while (p < end && *p >= '0' && *p <= '9') {
        x = x * 10 + (*p - '0');
        if (x > INT64_MAX / 16) return false;
        ++p;
      }
      out.push_back(x);
    }
    if (p < end) ++p;
    ++line;
    return true;
  }
};

}  // namespace

extern "C" {

void lpgpu_free(void* p) { std::free(p); }

lpgpu_status lpgpu_read_hgr(const char* path, int64_t* num_vertices, int64_t* num_nets, int64_t** net_offsets,
                            int32_t** pins, int32_t** vertex_weights, int32_t** net_weights,
                            int64_t* num_removed_single_pin_nets) {
  if (!path || !num_vertices || !num_nets || !net_offsets || !pins || !vertex_weights || !net_weights)
    return fail("null argument");
  *net_offsets = nullptr;
  *pins = nullptr;
  *vertex_weights = nullptr;
  *net_weights = nullptr;
  std::vector<char> buf;
  std::string err;
  if (!read_file(path, buf, err)) return fail(err);
  Text t{buf.data(), buf.data() + buf.size(), 1};
  std::vector<int64_t> nums;
  auto where = [&](int64_t line) { return std::string(path) + ":" + std::to_string(line) + ": "; };
  if (!t.next_content_line()) return fail(where(t.line) + "missing header");
  const int64_t hline = t.line;
  if (!t.line_numbers(nums) || nums.size() < 2 || nums.size() > 3)
    return fail(where(hline) + "header must be 'num_nets num_vertices [type]'");
  const int64_t m_file = nums[0], n = nums[1];
  const int64_t type = nums.size() == 3 ? nums[2] : 0;
  if (type != 0 && type != 1 && type != 10 && type != 11) return fail(where(hline) + "type must be 0, 1, 10 or 11");
  if (n > INT32_MAX || m_file > INT32_MAX) return fail(where(hline) + "vertex and net ids must fit int32");
  const bool has_ew = type == 1 || type == 11, has_vw = type == 10 || type == 11;
  std::vector<int64_t> off{0};
  std::vector<int32_t> pin, we;
  off.reserve((size_t)m_file + 1);
  we.reserve((size_t)m_file);
  int64_t removed = 0;
  for (int64_t e = 0; e < m_file; ++e) {
    if (!t.next_content_line()) return fail(where(t.line) + "expected " + std::to_string(m_file) + " net lines");
    const int64_t line = t.line;
    if (!t.line_numbers(nums)) return fail(where(line) + "net lines hold unsigned integers only");
    size_t first = 0;
    int64_t w = 1;
    if (has_ew) {
      if (nums.empty()) {  // an empty line is a net without pins: dropped
        ++removed;
        continue;
      }
      w = nums[0];
      first = 1;
      if (w > INT32_MAX) return fail(where(line) + "net weight exceeds int32");
    }
    if (nums.size() - first < 2) {  // single-pin (or empty) net
      ++removed;
      continue;
    }
    for (size_t i = first; i < nums.size(); ++i) {
      if (nums[i] < 1 || nums[i] > n) return fail(where(line) + "pin id outside 1.." + std::to_string(n));
      pin.push_back((int32_t)(nums[i] - 1));
    }
    off.push_back((int64_t)pin.size());
    we.push_back((int32_t)w);
  }
  std::vector<int32_t> wv((size_t)n, 1);
  if (has_vw) {
    int64_t v = 0;
    while (v < n) {
      if (!t.next_content_line()) return fail(where(t.line) + "expected " + std::to_string(n) + " vertex weights");
      const int64_t line = t.line;
      if (!t.line_numbers(nums)) return fail(where(line) + "vertex weights are unsigned integers");
      for (int64_t x : nums) {
        if (v >= n) return fail(where(line) + "more vertex weights than vertices");
        if (x > INT32_MAX) return fail(where(line) + "vertex weight exceeds int32");
        wv[(size_t)v++] = (int32_t)x;
      }
    }
  }
  const int64_t m = (int64_t)we.size();
  const int64_t P = (int64_t)pin.size();
  int64_t* o = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (size_t)(m + 1)));
  int32_t* pp = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (size_t)(P > 0 ? P : 1)));
  int32_t* vw = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
  int32_t* ew = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1)));
  if (!o || !pp || !vw || !ew) {
    std::free(o);
    std::free(pp);
    std::free(vw);
    std::free(ew);
    lpgpu::set_error("out of host memory");
    return LPGPU_ERR_OOM;
  }
  std::memcpy(o, off.data(), sizeof(int64_t) * (size_t)(m + 1));
  if (P > 0) std::memcpy(pp, pin.data(), sizeof(int32_t) * (size_t)P);
  if (n > 0) std::memcpy(vw, wv.data(), sizeof(int32_t) * (size_t)n);
  if (m > 0) std::memcpy(ew, we.data(), sizeof(int32_t) * (size_t)m);
  *num_vertices = n;
  *num_nets = m;
  *net_offsets = o;
  *pins = pp;
  *vertex_weights = vw;
  *net_weights = ew;
  if (num_removed_single_pin_nets) *num_removed_single_pin_nets = removed;
  return LPGPU_OK;
}

lpgpu_status lpgpu_read_partition(const char* path, int64_t num_vertices, int32_t* partition) {
  if (!path || (num_vertices > 0 && !partition)) return fail("null argument");
  std::vector<char> buf;
  std::string err;
  if (!read_file(path, buf, err)) return fail(err);
  Text t{buf.data(), buf.data() + buf.size(), 1};
  std::vector<int64_t> nums;
  for (int64_t v = 0; v < num_vertices; ++v) {
    if (t.done()) return fail(std::string(path) + ": expected " + std::to_string(num_vertices) + " block ids");
    const int64_t line = t.line;
    if (!t.line_numbers(nums) || nums.size() != 1 || nums[0] > INT32_MAX)
      return fail(std::string(path) + ":" + std::to_string(line) + ": one block id per line");
    partition[v] = (int32_t)nums[0];
  }
  return LPGPU_OK;
}

lpgpu_status lpgpu_write_partition(const char* path, int64_t num_vertices, const int32_t* partition) {
  if (!path || (num_vertices > 0 && !partition)) return fail("null argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(std::string("cannot open ") + path + ": " + std::strerror(errno));
  std::string out;
  out.reserve((size_t)num_vertices * 4);
  char tmp[16];
  for (int64_t v = 0; v < num_vertices; ++v) {
    const int len = std::snprintf(tmp, sizeof(tmp), "%d\n", partition[v]);
    out.append(tmp, (size_t)len);
  }
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok ? LPGPU_OK : fail(std::string("short write to ") + path);
}

}  // extern "C"
