// Vector files in the format of HODLRnD's storedata::save_vec / load_vec
// (include/myHeaders.hpp:146-170): a cereal PortableBinary archive holding one
// std::vector<double>.  The archive is
//
//   byte 0        1 if the payload is little endian, 0 if big endian
//   bytes 1..8    element count n, unsigned 64-bit, in the payload's byte order
//   bytes 9..     n IEEE-754 binary64 values, in the payload's byte order
//
// which is what cereal's portable binary archive writes for a vector of an
// arithmetic type (a bool endianness tag, a 64-bit size tag, the raw
// elements).  Files are written little endian, as cereal does by default;
// both byte orders are read.  Plain C++ with no cereal dependency.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hodlrnd.h"

namespace hodlr {
void set_thread_error(const std::string& msg);  // engine.cu: hodlr_last_error(NULL)
}

namespace {

bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

template <typename T>
T byte_swapped(T v) {
  unsigned char b[sizeof(T)];
  std::memcpy(b, &v, sizeof(T));
  for (size_t i = 0; i < sizeof(T) / 2; i++) {
    const unsigned char t = b[i];
    b[i] = b[sizeof(T) - 1 - i];
    b[sizeof(T) - 1 - i] = t;
  }
  std::memcpy(&v, b, sizeof(T));
  return v;
}

int fail(int code, const std::string& msg) {
  hodlr::set_thread_error(msg);
  return code;
}

struct File {
  std::FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

// Reads the 9-byte header; leaves the stream at the first value.
int read_header(std::FILE* f, const char* path, bool* swap, int64_t* n) {
  unsigned char tag = 0;
  uint64_t count = 0;
  if (std::fread(&tag, 1, 1, f) != 1 || std::fread(&count, 8, 1, f) != 1)
    return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": shorter than the 9-byte header");
  if (tag > 1) return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": bad endianness tag");
  *swap = (tag == 1) != host_little_endian();
  if (*swap) count = byte_swapped(count);
  // the payload must be exactly n values
  const long here = std::ftell(f);
  if (here < 0 || std::fseek(f, 0, SEEK_END) != 0)
    return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": cannot seek");
  const long end = std::ftell(f);
  if (end < 0 || std::fseek(f, here, SEEK_SET) != 0)
    return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": cannot seek");
  if (count > uint64_t(INT64_MAX / 8) || uint64_t(end - here) != count * 8)
    return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": element count " + std::to_string(count) +
                                  " does not match the file size");
  *n = int64_t(count);
  return HODLR_OK;
}

}  // namespace

extern "C" int hodlr_vec_load(const char* path, double* x, int64_t cap, int64_t* n) {
  if (!path || !n) return fail(HODLR_ERR_INVALID, "hodlr_vec_load: null argument");
  File fh;
  fh.f = std::fopen(path, "rb");
  if (!fh.f) return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: cannot open ") + path);
  bool swap = false;
  int64_t count = 0;
  const int rc = read_header(fh.f, path, &swap, &count);
  if (rc != HODLR_OK) return rc;
  *n = count;
  if (!x) return HODLR_OK;  // size query
  if (cap < count)
    return fail(HODLR_ERR_INVALID, "hodlr_vec_load: the file holds " + std::to_string(count) +
                                       " values, more than cap = " + std::to_string(cap));
  if (count > 0 && std::fread(x, 8, size_t(count), fh.f) != size_t(count))
    return fail(HODLR_ERR_IO, std::string("hodlr_vec_load: ") + path + ": short read");
  if (swap)
    for (int64_t i = 0; i < count; i++) x[i] = byte_swapped(x[i]);
  return HODLR_OK;
}

extern "C" int hodlr_vec_save(const char* path, const double* x, int64_t n) {
  if (!path || (n > 0 && !x) || n < 0) return fail(HODLR_ERR_INVALID, "hodlr_vec_save: bad argument");
  File fh;
  fh.f = std::fopen(path, "wb");
  if (!fh.f) return fail(HODLR_ERR_IO, std::string("hodlr_vec_save: cannot create ") + path);
  const bool swap = !host_little_endian();
  const unsigned char tag = 1;
  uint64_t count = uint64_t(n);
  if (swap) count = byte_swapped(count);
  bool ok = std::fwrite(&tag, 1, 1, fh.f) == 1 && std::fwrite(&count, 8, 1, fh.f) == 1;
  if (ok && !swap) {
    ok = n == 0 || std::fwrite(x, 8, size_t(n), fh.f) == size_t(n);
  } else if (ok) {
    std::vector<double> tmp(x, x + n);
    for (double& v : tmp) v = byte_swapped(v);
    ok = n == 0 || std::fwrite(tmp.data(), 8, size_t(n), fh.f) == size_t(n);
  }
  ok = ok && std::fflush(fh.f) == 0;
  if (!ok) return fail(HODLR_ERR_IO, std::string("hodlr_vec_save: write failed: ") + path);
  return HODLR_OK;
}
