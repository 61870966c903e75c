// mat_io.hpp -- MATLAB Level-5 (uncompressed) writer for the reference's
// result files: matlab_io::mat_save_multi_array
// (libMatlabIO/matlab_io.hpp:64-142) stores a boost::multi_array as one
// numeric variable in Fortran order.  The reference links MATLAB's libmat
// for this; the format (128-byte header, one miMATRIX element holding the
// array flags, dimensions, name and real part) is written here directly.
#ifndef PARTAPP_GPU_MAT_IO_HPP_
#define PARTAPP_GPU_MAT_IO_HPP_

#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace partapp_gpu {

namespace mat_detail {

enum : uint32_t { miINT8 = 1, miINT32 = 5, miUINT32 = 6, miSINGLE = 7, miMATRIX = 14 };
enum : uint32_t { mxSINGLE_CLASS = 7 };

inline size_t pad8(size_t n) { return (n + 7) / 8 * 8; }

inline void put32(std::vector<char> &b, uint32_t v) {
  char c[4];
  std::memcpy(c, &v, 4);
  b.insert(b.end(), c, c + 4);
}

inline void put_bytes(std::vector<char> &b, const void *p, size_t n) {
  const char *c = static_cast<const char *>(p);
  b.insert(b.end(), c, c + n);
  b.resize(b.size() + (pad8(n) - n), 0);
}

}  // namespace mat_detail

// Writes `var` = single-precision array of shape dims (row-major, C order, as
// boost::multi_array stores it) to `path`; MATLAB sees the same shape.
inline bool mat_save_float(const std::string &path, const std::string &var,
                           const std::vector<size_t> &dims, const float *data) {
  using namespace mat_detail;
  size_t n = 1;
  for (size_t d : dims) n *= d;
  // C order -> Fortran order (the copy B = A of matlab_io.hpp:73-75)
  std::vector<float> f(n);
  std::vector<size_t> idx(dims.size(), 0);
  for (size_t i = 0; i < n; ++i) {
    size_t fo = 0, stride = 1;
    for (size_t k = 0; k < dims.size(); ++k) {
      fo += idx[k] * stride;
      stride *= dims[k];
    }
    f[fo] = data[i];
    for (size_t k = dims.size(); k-- > 0;) {  // advance the C-order index
      if (++idx[k] < dims[k]) break;
      idx[k] = 0;
    }
  }
  std::vector<char> body;
  put32(body, miUINT32);  // array flags
  put32(body, 8);
  put32(body, mxSINGLE_CLASS);
  put32(body, 0);
  put32(body, miINT32);  // dimensions
  put32(body, (uint32_t)(4 * dims.size()));
  std::vector<int32_t> d32(dims.begin(), dims.end());
  put_bytes(body, d32.data(), 4 * d32.size());
  put32(body, miINT8);  // array name
  put32(body, (uint32_t)var.size());
  put_bytes(body, var.data(), var.size());
  put32(body, miSINGLE);  // real part
  put32(body, (uint32_t)(4 * n));
  put_bytes(body, f.data(), 4 * n);

  char header[128];
  std::memset(header, ' ', 116);
  const char text[] = "MATLAB 5.0 MAT-file, written by partapp_gb300";
  std::memcpy(header, text, sizeof(text) - 1);
  std::memset(header + 116, 0, 8);  // subsystem data offset
  const uint16_t version = 0x0100;
  std::memcpy(header + 124, &version, 2);
  header[126] = 'I';
  header[127] = 'M';
  std::ofstream out(path, std::ios::binary);
  if (!out) return false;
  out.write(header, 128);
  std::vector<char> tag;
  put32(tag, miMATRIX);
  put32(tag, (uint32_t)body.size());
  out.write(tag.data(), (std::streamsize)tag.size());
  out.write(body.data(), (std::streamsize)body.size());
  return (bool)out;
}

}  // namespace partapp_gpu

#endif  // PARTAPP_GPU_MAT_IO_HPP_
