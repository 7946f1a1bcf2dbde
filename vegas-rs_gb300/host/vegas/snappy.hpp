// snappy.hpp -- a Snappy block compressor for the Parquet pages.
//
// The reference's Parquet files are written with Compression::SNAPPY
// (src/output.rs:48, :138).  This is the raw Snappy block format as Google
// publishes it (format_description.txt in google/snappy): the uncompressed
// length as a little-endian base-128 varint, then a sequence of elements,
// each a tag byte whose two low bits give its kind --
//   00 literal: length - 1 in the upper six bits when below 60, else 60..63
//      there and the length - 1 in the next 1..4 bytes (little endian),
//      followed by the literal bytes;
//   01 copy, 1-byte offset: length - 4 (4..11) in bits 2..4, offset bits
//      8..10 in bits 5..7, offset bits 0..7 in the next byte;
//   10 copy, 2-byte offset: length - 1 (1..64) in the upper six bits, the
//      offset in the next two bytes;
//   11 copy, 4-byte offset: as 10 with a four-byte offset.
// A copy repeats `length` bytes starting `offset` bytes back in the output
// (offset >= 1; the ranges may overlap).  Matches are found greedily with a
// hash table of 4-byte sequences; any valid element sequence decodes, so
// the output need not equal another compressor's byte for byte.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace vegas {
namespace snappy {

namespace detail {

inline void varint(std::vector<uint8_t>& o, uint64_t v) {
  while (v >= 0x80) {
    o.push_back((uint8_t)(v | 0x80));
    v >>= 7;
  }
  o.push_back((uint8_t)v);
}

inline uint32_t load32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

inline void literal(std::vector<uint8_t>& o, const uint8_t* p, size_t n) {
  while (n > 0) {  // one element holds at most 2^32 bytes
    const size_t len = n > 0xFFFFFFFFull ? 0xFFFFFFFFull : n;
    const uint64_t m = len - 1;
    if (m < 60) {
      o.push_back((uint8_t)(m << 2));
    } else {
      int bytes = m < (1ull << 8) ? 1 : m < (1ull << 16) ? 2 : m < (1ull << 24) ? 3 : 4;
      o.push_back((uint8_t)((59 + bytes) << 2));
      for (int b = 0; b < bytes; ++b) o.push_back((uint8_t)(m >> (8 * b)));
    }
    o.insert(o.end(), p, p + len);
    p += len;
    n -= len;
  }
}

// One copy element of 1..64 bytes.
inline void copy1(std::vector<uint8_t>& o, size_t offset, size_t len) {
  if (len >= 4 && len <= 11 && offset < 2048) {
    o.push_back((uint8_t)(((offset >> 8) << 5) | ((len - 4) << 2) | 1));
    o.push_back((uint8_t)offset);
  } else if (offset < 65536) {
    o.push_back((uint8_t)(((len - 1) << 2) | 2));
    o.push_back((uint8_t)offset);
    o.push_back((uint8_t)(offset >> 8));
  } else {
    o.push_back((uint8_t)(((len - 1) << 2) | 3));
    for (int b = 0; b < 4; ++b) o.push_back((uint8_t)(offset >> (8 * b)));
  }
}

// A copy of any length >= 4 as elements of at most 64 bytes, none shorter
// than 4 (so that every piece may use the short form when it fits).
inline void copy(std::vector<uint8_t>& o, size_t offset, size_t len) {
  while (len >= 68) {
    copy1(o, offset, 64);
    len -= 64;
  }
  if (len > 64) {
    copy1(o, offset, 60);
    len -= 60;
  }
  copy1(o, offset, len);
}

}  // namespace detail

// Compressed form of in[0, n).
inline std::vector<uint8_t> compress(const uint8_t* in, size_t n) {
  using namespace detail;
  if (n > 0xFFFFFFFFull) throw std::length_error("snappy: a block holds less than 4 GiB");
  std::vector<uint8_t> o;
  o.reserve(n + n / 6 + 32);
  varint(o, n);
  constexpr int kBits = 14;
  std::vector<uint32_t> table(1u << kBits, 0u);  // position + 1 of the last sequence with this hash
  size_t i = 0, lit = 0;
  while (i + 4 <= n) {
    const uint32_t v = load32(in + i);
    const uint32_t h = (v * 0x1E35A7BDu) >> (32 - kBits);
    const size_t cand = table[h];
    table[h] = (uint32_t)(i + 1);
    if (cand > 0 && load32(in + cand - 1) == v) {
      const size_t from = cand - 1;
      size_t len = 4;
      while (i + len < n && in[from + len] == in[i + len]) ++len;
      if (i > lit) literal(o, in + lit, i - lit);
      copy(o, i - from, len);
      i += len;
      lit = i;
    } else {
      ++i;
    }
  }
  if (n > lit) literal(o, in + lit, n - lit);
  return o;
}

inline std::vector<uint8_t> compress(const std::vector<uint8_t>& in) { return compress(in.data(), in.size()); }

// The inverse, for the writer's own checks and tests: throws on malformed input.
inline std::vector<uint8_t> decompress(const uint8_t* p, size_t n) {
  size_t k = 0;
  uint64_t len = 0;
  for (int s = 0;; s += 7) {
    if (k >= n || s > 35) throw std::runtime_error("snappy: bad length");
    const uint8_t b = p[k++];
    len |= (uint64_t)(b & 0x7F) << s;
    if (!(b & 0x80)) break;
  }
  std::vector<uint8_t> o;
  o.reserve(len);
  while (k < n) {
    const uint8_t tag = p[k++];
    const int kind = tag & 3;
    if (kind == 0) {
      uint64_t m = tag >> 2;
      if (m >= 60) {
        const int bytes = (int)m - 59;
        if (k + bytes > n) throw std::runtime_error("snappy: truncated literal length");
        m = 0;
        for (int b = 0; b < bytes; ++b) m |= (uint64_t)p[k++] << (8 * b);
      }
      const uint64_t l = m + 1;
      if (k + l > n) throw std::runtime_error("snappy: truncated literal");
      o.insert(o.end(), p + k, p + k + l);
      k += l;
      continue;
    }
    size_t l, off;
    if (kind == 1) {
      if (k + 1 > n) throw std::runtime_error("snappy: truncated copy");
      l = 4 + ((tag >> 2) & 7);
      off = ((size_t)(tag >> 5) << 8) | p[k++];
    } else {
      const int bytes = kind == 2 ? 2 : 4;
      if (k + bytes > n) throw std::runtime_error("snappy: truncated copy");
      l = 1 + (tag >> 2);
      off = 0;
      for (int b = 0; b < bytes; ++b) off |= (size_t)p[k++] << (8 * b);
    }
    if (off == 0 || off > o.size()) throw std::runtime_error("snappy: bad copy offset");
    const size_t from = o.size() - off;
    for (size_t j = 0; j < l; ++j) o.push_back(o[from + j]);
  }
  if (o.size() != len) throw std::runtime_error("snappy: length mismatch");
  return o;
}

}  // namespace snappy
}  // namespace vegas
