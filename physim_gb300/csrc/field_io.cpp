// field_io.cpp -- SVL scalar-grid files (field output next to the solve).
//
// The reference reads and writes ScalarField_Grid<T> for T in {char, short, int, float,
// double} (source/PhySim/Utils/Serializer_Field.cpp): readGridSVL (:50-112) reads the
// header (shape as 3 int, origin and delta as 3 double each, the value type as an int) and
// then the values, converting value by value (IOUtils::readBinaryArrayWithCast,
// include/PhySim/Utils/IOUtils.h:51-57) when the file's type is not the grid's; writeGridSVL
// (:114-140) writes the same header and the raw values.  The values are the grid's Eigen
// tensor storage, column-major, so x varies fastest.
//
// Differences, each deliberate: type 0 ("char") is signed 8-bit on every host (a plain
// char is unsigned on Arm); a conversion whose value the target type cannot hold is refused
// (PHX_EINVAL) rather than left undefined; an unknown type, a shape below 1 or a short file
// is refused where the reference asserts or returns false; the value count is 64-bit.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <limits>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "errors.h"
#include "phx.h"

namespace {

constexpr size_t kHeaderBytes = 3 * sizeof(int32_t) + 6 * sizeof(double) + sizeof(int32_t);

size_t type_size(int32_t f) {
  switch (f) {
    case PHX_SVL_INT8: return 1;
    case PHX_SVL_INT16: return 2;
    case PHX_SVL_INT32: return 4;
    case PHX_SVL_FLOAT: return 4;
    case PHX_SVL_DOUBLE: return 8;
    default: return 0;
  }
}

int fail(int code, const std::string& msg) { return phx::set_last_error(code, msg); }

int check_grid(const phx_grid& g, int64_t* count) {
  int64_t c = 1;
  for (int d = 0; d < 3; ++d) {
    if (g.shape[d] < 1) return fail(PHX_EINVAL, "svl: every shape entry must be >= 1");
    c *= g.shape[d];
  }
  *count = c;
  return PHX_OK;
}

// Reads the 64-byte header; the stream is left at the first value.
int read_header(std::ifstream& f, const char* path, phx_grid* g, int32_t* format) {
  char h[kHeaderBytes];
  if (!f.read(h, kHeaderBytes)) return fail(PHX_EINVAL, std::string("svl: short header in ") + path);
  std::memcpy(g->shape, h, 12);
  std::memcpy(g->origin, h + 12, 24);
  std::memcpy(g->delta, h + 36, 24);
  std::memcpy(format, h + 60, 4);
  if (type_size(*format) == 0) return fail(PHX_EINVAL, "svl: unknown value type " + std::to_string(*format));
  int64_t count;
  return check_grid(*g, &count);
}

template <typename T>
T load(const char* p) {
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}

// One value of the file's type as a double (every int8/16/32 and float is exact in double).
double file_value(const char* p, int32_t f) {
  switch (f) {
    case PHX_SVL_INT8: return (double)load<int8_t>(p);
    case PHX_SVL_INT16: return (double)load<int16_t>(p);
    case PHX_SVL_INT32: return (double)load<int32_t>(p);
    case PHX_SVL_FLOAT: return (double)load<float>(p);
    default: return load<double>(p);
  }
}

// value -> T as static_cast does (integers truncate toward zero); false if T cannot hold it.
template <typename T>
bool convert(double v, T* out) {
  if (std::is_integral<T>::value) {
    if (!std::isfinite(v)) return false;
    double t = std::trunc(v);
    if (t < (double)std::numeric_limits<T>::min() || t > (double)std::numeric_limits<T>::max()) return false;
    *out = (T)t;
    return true;
  }
  if (std::isfinite(v) && std::fabs(v) > (double)std::numeric_limits<T>::max()) return false;
  *out = (T)v;
  return true;
}

template <typename T>
int convert_all(const char* src, int32_t from, int64_t count, void* dst) {
  const size_t sz = type_size(from);
  T* out = (T*)dst;
  for (int64_t i = 0; i < count; ++i) {
    double v = file_value(src + sz * (size_t)i, from);
    if (!convert<T>(v, &out[i]))
      return fail(PHX_EINVAL, "svl: value " + std::to_string(i) + " (" + std::to_string(v) +
                                  ") does not fit the requested type");
  }
  return PHX_OK;
}

}  // namespace

extern "C" {

int phx_svl_write(const char* path, const phx_grid* grid, int32_t format, const void* values) {
  if (!path || !grid || !values) return fail(PHX_EINVAL, "svl: NULL argument");
  const size_t sz = type_size(format);
  if (!sz) return fail(PHX_EINVAL, "svl: unknown value type " + std::to_string(format));
  int64_t count;
  if (int rc = check_grid(*grid, &count)) return rc;
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) return fail(PHX_EINVAL, std::string("svl: cannot open ") + path + " for writing");
  f.write((const char*)grid->shape, 12);
  f.write((const char*)grid->origin, 24);
  f.write((const char*)grid->delta, 24);
  f.write((const char*)&format, 4);
  f.write((const char*)values, (std::streamsize)(sz * (size_t)count));
  f.close();
  if (!f) return fail(PHX_EINVAL, std::string("svl: writing ") + path + " failed");
  return PHX_OK;
}

int phx_svl_read_header(const char* path, phx_grid* grid, int32_t* format) {
  if (!path) return fail(PHX_EINVAL, "svl: NULL path");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(PHX_ENOTFOUND, std::string("svl: cannot open ") + path);
  phx_grid g;
  int32_t fmt;
  if (int rc = read_header(f, path, &g, &fmt)) return rc;
  if (grid) *grid = g;
  if (format) *format = fmt;
  return PHX_OK;
}

int phx_svl_read(const char* path, int32_t as_format, void* values, int64_t capacity) {
  if (!path || !values) return fail(PHX_EINVAL, "svl: NULL argument");
  const size_t out_sz = type_size(as_format);
  if (!out_sz) return fail(PHX_EINVAL, "svl: unknown value type " + std::to_string(as_format));
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(PHX_ENOTFOUND, std::string("svl: cannot open ") + path);
  phx_grid g;
  int32_t from;
  if (int rc = read_header(f, path, &g, &from)) return rc;
  const int64_t count = (int64_t)g.shape[0] * g.shape[1] * g.shape[2];
  if (count > capacity)
    return fail(PHX_EINVAL, "svl: the grid holds " + std::to_string(count) + " values, room for " +
                                std::to_string(capacity));
  const size_t bytes = type_size(from) * (size_t)count;
  if (from == as_format) {
    if (!f.read((char*)values, (std::streamsize)bytes)) return fail(PHX_EINVAL, std::string("svl: short file ") + path);
    return PHX_OK;
  }
  try {
    std::vector<char> buf(bytes);
    if (!f.read(buf.data(), (std::streamsize)bytes)) return fail(PHX_EINVAL, std::string("svl: short file ") + path);
    switch (as_format) {
      case PHX_SVL_INT8: return convert_all<int8_t>(buf.data(), from, count, values);
      case PHX_SVL_INT16: return convert_all<int16_t>(buf.data(), from, count, values);
      case PHX_SVL_INT32: return convert_all<int32_t>(buf.data(), from, count, values);
      case PHX_SVL_FLOAT: return convert_all<float>(buf.data(), from, count, values);
      default: return convert_all<double>(buf.data(), from, count, values);
    }
  } catch (const std::bad_alloc&) {
    return fail(PHX_ENOMEM, "svl: host memory exhausted");
  }
}

}  // extern "C"
