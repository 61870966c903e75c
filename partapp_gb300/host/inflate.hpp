// inflate.hpp -- zlib-stream (RFC 1950) / DEFLATE (RFC 1951) decoder for the
// compressed variables of MATLAB v7 MAT-files (miCOMPRESSED elements, which
// the reference writes with matOpen(..., "wz"), partdetect_test.cpp:246).
// Self-contained: the host code has no zlib dependency.  Canonical Huffman
// codes are decoded code length by code length, following the construction
// in RFC 1951 section 3.2.2.
#ifndef PARTAPP_GPU_INFLATE_HPP_
#define PARTAPP_GPU_INFLATE_HPP_

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace partapp_gpu {
namespace inflate_detail {

struct BitReader {
  const uint8_t *p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  BitReader(const uint8_t *data, size_t size) : p(data), n(size) {}
  uint32_t bits(int need) {  // LSB-first, need <= 24
    while (cnt < need) {
      if (pos >= n) throw std::runtime_error("inflate: input ends inside a block");
      buf |= (uint32_t)p[pos++] << cnt;
      cnt += 8;
    }
    const uint32_t v = buf & ((1u << need) - 1u);
    buf >>= need;
    cnt -= need;
    return v;
  }
  void align() {
    buf = 0;
    cnt = 0;
  }
};

// Canonical Huffman code: count[len] codes of each length, symbols in code order.
struct Huffman {
  uint16_t count[16] = {};
  std::vector<uint16_t> symbol;
  void build(const uint8_t *lengths, int n) {
    for (int l = 0; l < 16; ++l) count[l] = 0;
    for (int s = 0; s < n; ++s) ++count[lengths[s]];
    count[0] = 0;
    int left = 1;  // over-subscribed codes are invalid; incomplete ones are allowed
    for (int l = 1; l < 16; ++l) {
      left = 2 * left - count[l];
      if (left < 0) throw std::runtime_error("inflate: over-subscribed Huffman code");
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
    symbol.assign(n, 0);
    for (int s = 0; s < n; ++s)
      if (lengths[s]) symbol[offs[lengths[s]]++] = (uint16_t)s;
  }
  int decode(BitReader &br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= (int)br.bits(1);
      const int c = count[len];
      if (code - first < c) return symbol[index + (code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    throw std::runtime_error("inflate: invalid Huffman code");
  }
};

// Length and distance bases and extra bits (RFC 1951 section 3.2.5).
constexpr uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                   2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                    33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                    1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                    6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

inline void codes(BitReader &br, std::vector<uint8_t> &out, const Huffman &lit,
                  const Huffman &dist) {
  for (;;) {
    int sym = lit.decode(br);
    if (sym < 256) {
      out.push_back((uint8_t)sym);
    } else if (sym == 256) {
      return;
    } else {
      sym -= 257;
      if (sym >= 29) throw std::runtime_error("inflate: invalid length symbol");
      const size_t len = kLenBase[sym] + br.bits(kLenExtra[sym]);
      const int ds = dist.decode(br);
      if (ds >= 30) throw std::runtime_error("inflate: invalid distance symbol");
      const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
      if (d > out.size()) throw std::runtime_error("inflate: distance before the output start");
      const size_t from = out.size() - d;
      for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
  }
}

}  // namespace inflate_detail

// Decompresses a raw DEFLATE stream; returns the number of input bytes used.
inline size_t inflate_raw(const uint8_t *in, size_t n, std::vector<uint8_t> &out) {
  using namespace inflate_detail;
  BitReader br(in, n);
  Huffman fixed_lit, fixed_dist;
  {
    uint8_t l[288];
    for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
    fixed_lit.build(l, 288);
    uint8_t d[30];
    for (int s = 0; s < 30; ++s) d[s] = 5;
    fixed_dist.build(d, 30);
  }
  bool last = false;
  while (!last) {
    last = br.bits(1) != 0;
    const uint32_t type = br.bits(2);
    if (type == 0) {  // stored
      br.align();
      if (br.pos + 4 > n) throw std::runtime_error("inflate: truncated stored block");
      const uint32_t len = in[br.pos] | (in[br.pos + 1] << 8);
      const uint32_t nlen = in[br.pos + 2] | (in[br.pos + 3] << 8);
      if ((len ^ 0xFFFFu) != nlen) throw std::runtime_error("inflate: stored length mismatch");
      br.pos += 4;
      if (br.pos + len > n) throw std::runtime_error("inflate: truncated stored block");
      out.insert(out.end(), in + br.pos, in + br.pos + len);
      br.pos += len;
    } else if (type == 1) {
      codes(br, out, fixed_lit, fixed_dist);
    } else if (type == 2) {
      const int nlit = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
      if (nlit > 286 || ndist > 30) throw std::runtime_error("inflate: bad dynamic header");
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {};
      for (int k = 0; k < ncode; ++k) cl[order[k]] = (uint8_t)br.bits(3);
      Huffman lencode;
      lencode.build(cl, 19);
      uint8_t lengths[320] = {};
      int k = 0;
      while (k < nlit + ndist) {
        const int sym = lencode.decode(br);
        if (sym < 16) {
          lengths[k++] = (uint8_t)sym;
          continue;
        }
        uint8_t v = 0;
        int rep;
        if (sym == 16) {
          if (k == 0) throw std::runtime_error("inflate: repeat with no previous length");
          v = lengths[k - 1];
          rep = 3 + (int)br.bits(2);
        } else if (sym == 17) {
          rep = 3 + (int)br.bits(3);
        } else {
          rep = 11 + (int)br.bits(7);
        }
        if (k + rep > nlit + ndist) throw std::runtime_error("inflate: too many lengths");
        while (rep--) lengths[k++] = v;
      }
      if (lengths[256] == 0) throw std::runtime_error("inflate: no end-of-block code");
      Huffman lit, dist;
      lit.build(lengths, nlit);
      dist.build(lengths + nlit, ndist);
      codes(br, out, lit, dist);
    } else {
      throw std::runtime_error("inflate: invalid block type");
    }
  }
  return br.pos;
}

// Decompresses a zlib stream (2-byte header, DEFLATE data, Adler-32).
inline std::vector<uint8_t> inflate_zlib(const uint8_t *in, size_t n) {
  if (n < 6) throw std::runtime_error("inflate: zlib stream too short");
  const uint8_t cmf = in[0], flg = in[1];
  if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
    throw std::runtime_error("inflate: not a zlib DEFLATE stream (or a preset dictionary)");
  std::vector<uint8_t> out;
  const size_t used = 2 + inflate_raw(in + 2, n - 2, out);
  if (used + 4 > n) throw std::runtime_error("inflate: missing Adler-32");
  uint32_t a = 1, b = 0;
  for (uint8_t c : out) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  const uint32_t want = ((uint32_t)in[used] << 24) | ((uint32_t)in[used + 1] << 16) |
                        ((uint32_t)in[used + 2] << 8) | in[used + 3];
  if (((b << 16) | a) != want) throw std::runtime_error("inflate: Adler-32 mismatch");
  return out;
}

}  // namespace partapp_gpu

#endif  // PARTAPP_GPU_INFLATE_HPP_
