// mat_io.hpp -- MATLAB Level-5 MAT-files without libmat.
//
// Writer: the reference's result files.  matlab_io::mat_save_multi_array
// (libMatlabIO/matlab_io.hpp:64-142) stores a boost::multi_array as one
// numeric variable in Fortran order; the format (128-byte header, one
// miMATRIX element holding the array flags, dimensions, name and real part)
// is written here directly, uncompressed.
//
// Reader: the files the reference's part detector saves and --find_obj
// loads (partdetect_test.cpp:240-256 writes them with matOpen(..., "wz"),
// i.e. compressed v7 files; PartApp::loadScoreGrid, partapp.cpp:830-903,
// reads them): numeric arrays of any storage type and cell arrays of them,
// plain or inside miCOMPRESSED elements (inflate.hpp).
#ifndef PARTAPP_GPU_MAT_IO_HPP_
#define PARTAPP_GPU_MAT_IO_HPP_

#include <cstdint>
#include <cstring>
#include <fstream>
#include <initializer_list>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "inflate.hpp"

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

// ---------------------------------------------------------------- reader

// One MATLAB variable: a numeric array (values converted to double, Fortran
// order as stored) or a cell array (cells in Fortran order).
struct MatArray {
  std::string name;
  int mx_class = 0;  // 1: cell, 6: double, 7: single, 8-15: integers
  std::vector<size_t> dims;
  std::vector<double> re;
  std::vector<MatArray> cells;
  size_t numel() const {
    size_t n = 1;
    for (size_t d : dims) n *= d;
    return n;
  }
  bool is_cell() const { return mx_class == 1; }
};

namespace mat_detail {

inline uint32_t rd32(const uint8_t *p) {
  uint32_t v;
  std::memcpy(&v, p, 4);
  return v;
}

// Tag of the data element at p (n bytes left): type, payload size, payload
// start, and the offset of the next element.
struct Element {
  uint32_t type;
  size_t size;
  const uint8_t *data;
  size_t next;
};

inline Element element(const uint8_t *p, size_t n) {
  if (n < 8) throw std::runtime_error("MAT: truncated element tag");
  const uint32_t t = rd32(p);
  if (t >> 16) {  // small data element: size and type in one word, data in the next
    const size_t sz = t >> 16;
    if (sz > 4) throw std::runtime_error("MAT: bad small element");
    return {t & 0xFFFFu, sz, p + 4, 8};
  }
  const size_t sz = rd32(p + 4);
  if (sz > n - 8) throw std::runtime_error("MAT: element larger than its container");
  // compressed elements are not padded; the others end on 8-byte boundaries
  const size_t next = t == 15 ? 8 + sz : 8 + pad8(sz);
  return {t, sz, p + 8, next > n ? n : next};
}

template <class T>
void widen(const uint8_t *p, size_t count, std::vector<double> &out) {
  out.resize(count);
  for (size_t i = 0; i < count; ++i) {
    T v;
    std::memcpy(&v, p + i * sizeof(T), sizeof(T));
    out[i] = (double)v;
  }
}

inline void numeric(const Element &e, std::vector<double> &out) {
  switch (e.type) {
    case 1: widen<int8_t>(e.data, e.size, out); break;
    case 2: widen<uint8_t>(e.data, e.size, out); break;
    case 3: widen<int16_t>(e.data, e.size / 2, out); break;
    case 4: widen<uint16_t>(e.data, e.size / 2, out); break;
    case 5: widen<int32_t>(e.data, e.size / 4, out); break;
    case 6: widen<uint32_t>(e.data, e.size / 4, out); break;
    case 7: widen<float>(e.data, e.size / 4, out); break;
    case 9: widen<double>(e.data, e.size / 8, out); break;
    case 12: widen<int64_t>(e.data, e.size / 8, out); break;
    case 13: widen<uint64_t>(e.data, e.size / 8, out); break;
    default: throw std::runtime_error("MAT: unsupported numeric storage type");
  }
}

inline MatArray matrix(const uint8_t *p, size_t n) {
  MatArray a;
  if (n == 0) return a;  // an empty cell element
  size_t off = 0;
  const Element flags = element(p, n);
  if (flags.type != 6 || flags.size < 8) throw std::runtime_error("MAT: bad array flags");
  const uint32_t fw = rd32(flags.data);
  a.mx_class = (int)(fw & 0xFF);
  if (fw & 0x800) throw std::runtime_error("MAT: complex arrays are not supported");
  off += flags.next;
  const Element dims = element(p + off, n - off);
  if (dims.type != 5) throw std::runtime_error("MAT: bad dimensions");
  for (size_t k = 0; k < dims.size / 4; ++k) a.dims.push_back((size_t)(int32_t)rd32(dims.data + 4 * k));
  off += dims.next;
  const Element name = element(p + off, n - off);
  a.name.assign(reinterpret_cast<const char *>(name.data), name.size);
  off += name.next;
  if (a.mx_class == 1) {  // cell: numel miMATRIX elements
    const size_t cnt = a.numel();
    for (size_t k = 0; k < cnt; ++k) {
      const Element c = element(p + off, n - off);
      if (c.type != 14) throw std::runtime_error("MAT: cell element is not a matrix");
      a.cells.push_back(matrix(c.data, c.size));
      off += c.next;
    }
  } else if (a.mx_class >= 6 && a.mx_class <= 15) {
    if (a.numel() > 0) {
      const Element re = element(p + off, n - off);
      numeric(re, a.re);
      if (a.re.size() != a.numel()) throw std::runtime_error("MAT: real part has the wrong length");
    }
  } else {
    throw std::runtime_error("MAT: unsupported array class " + std::to_string(a.mx_class));
  }
  return a;
}

inline void variables(const uint8_t *p, size_t n, std::vector<MatArray> &out) {
  size_t off = 0;
  while (off + 8 <= n) {
    const Element e = element(p + off, n - off);
    if (e.type == 15) {
      const std::vector<uint8_t> raw = inflate_zlib(e.data, e.size);
      variables(raw.data(), raw.size(), out);
    } else if (e.type == 14) {
      out.push_back(matrix(e.data, e.size));
    }
    off += e.next;
  }
}

}  // namespace mat_detail

// Every variable of a little-endian Level-5 MAT-file.
inline std::vector<MatArray> mat_read(const std::string &path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  std::ostringstream ss;
  ss << in.rdbuf();
  const std::string buf = ss.str();
  if (buf.size() < 128 || buf[126] != 'I' || buf[127] != 'M')
    throw std::runtime_error(path + ": not a little-endian Level-5 MAT-file");
  std::vector<MatArray> vars;
  mat_detail::variables(reinterpret_cast<const uint8_t *>(buf.data()) + 128, buf.size() - 128,
                        vars);
  return vars;
}

inline const MatArray &mat_find(const std::vector<MatArray> &vars, const std::string &name) {
  for (const MatArray &v : vars)
    if (v.name == name) return v;
  throw std::runtime_error("MAT: variable " + name + " not found");
}

// Element (i0, i1, ...) of a Fortran-order array.
inline double mat_at(const MatArray &a, std::initializer_list<size_t> idx) {
  size_t o = 0, stride = 1, k = 0;
  for (size_t i : idx) {
    o += i * stride;
    stride *= k < a.dims.size() ? a.dims[k] : 1;
    ++k;
  }
  return a.re.at(o);
}

}  // namespace partapp_gpu

#endif  // PARTAPP_GPU_MAT_IO_HPP_
