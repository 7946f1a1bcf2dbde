// parquet.hpp -- a minimal Apache Parquet writer for the instruments' files.
//
// The reference writes its observables and state snapshots with arrow's
// ArrowWriter (src/output.rs:26-112, :114-200): flat schemas of required
// BOOLEAN, UINT64 and FLOAT64 columns, row groups of up to 1,048,576 rows,
// written to "<path>.parquet.tmp" (Path::with_extension) and renamed over the
// destination when the writer is dropped.  This writer produces files with
// the same schema, column order and row grouping: PLAIN-encoded values in
// one data page per column chunk, compressed with SNAPPY as the
// reference's pages are (snappy.hpp), and the file metadata in Thrift's compact
// protocol as the Parquet format specifies (parquet.thrift: FileMetaData,
// SchemaElement, RowGroup, ColumnChunk, ColumnMetaData, PageHeader,
// DataPageHeader).
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "error.hpp"
#include "snappy.hpp"

namespace vegas {
namespace parquet {

enum class Type { Bool, UInt64, Float64 };

// Thrift compact protocol, the subset the file metadata needs.
class Compact {
 public:
  std::vector<uint8_t> out;

  void begin_struct() {
    stack_.push_back(last_);
    last_ = 0;
  }
  void end_struct() {
    out.push_back(0);  // stop
    last_ = stack_.back();
    stack_.pop_back();
  }
  void field_i32(int16_t id, int32_t v) {
    header(id, 5);
    varint(zigzag(v));
  }
  void field_i64(int16_t id, int64_t v) {
    header(id, 6);
    varint(zigzag(v));
  }
  void field_bool(int16_t id, bool v) { header(id, v ? 1 : 2); }
  void field_byte(int16_t id, int8_t v) {
    header(id, 3);
    out.push_back((uint8_t)v);
  }
  void field_string(int16_t id, const std::string& s) {
    header(id, 8);
    varint(s.size());
    out.insert(out.end(), s.begin(), s.end());
  }
  void field_struct(int16_t id) {
    header(id, 12);
    begin_struct();
  }
  // list header; elements follow (structs: begin_struct .. end_struct each)
  void field_list(int16_t id, uint8_t elem_type, size_t n) {
    header(id, 9);
    list_header(elem_type, n);
  }
  void list_header(uint8_t elem_type, size_t n) {
    if (n < 15) {
      out.push_back((uint8_t)((n << 4) | elem_type));
    } else {
      out.push_back((uint8_t)(0xF0 | elem_type));
      varint(n);
    }
  }
  void elem_i32(int32_t v) { varint(zigzag(v)); }
  void elem_string(const std::string& s) {
    varint(s.size());
    out.insert(out.end(), s.begin(), s.end());
  }

 private:
  static uint64_t zigzag(int64_t v) { return ((uint64_t)v << 1) ^ (uint64_t)(v >> 63); }
  void varint(uint64_t v) {
    while (v >= 0x80) {
      out.push_back((uint8_t)(v | 0x80));
      v >>= 7;
    }
    out.push_back((uint8_t)v);
  }
  void header(int16_t id, uint8_t type) {
    const int delta = id - last_;
    if (delta > 0 && delta <= 15) {
      out.push_back((uint8_t)((delta << 4) | type));
    } else {
      out.push_back(type);
      varint(zigzag(id));
    }
    last_ = id;
  }
  int16_t last_ = 0;
  std::vector<int16_t> stack_;
};

constexpr uint8_t kI32 = 5, kBinary = 8, kStruct = 12;

struct Column {
  std::string name;
  Type type;
  std::vector<uint8_t> data;  // PLAIN values of the current row group (booleans: one byte each until flushed)
};

class Writer {
 public:
  static constexpr size_t kRowGroupRows = 1024 * 1024;

  // Writes to tmp_path; close() finishes the file and renames it to path.
  Writer(const std::string& path, const std::string& tmp_path, std::vector<std::pair<std::string, Type>> schema,
         size_t row_group_rows = kRowGroupRows)
      : path_(path), tmp_(tmp_path), group_rows_(row_group_rows ? row_group_rows : kRowGroupRows) {
    for (auto& c : schema) cols_.push_back(Column{c.first, c.second, {}});
    f_ = std::fopen(tmp_.c_str(), "wb");
    if (!f_) throw IoError("std io error: cannot create " + tmp_);
    put("PAR1", 4);
  }
  ~Writer() {
    try {
      close();
    } catch (const std::exception& e) {
      std::fprintf(stderr, "error closing parquet writer: %s\n", e.what());
    }
  }
  Writer(const Writer&) = delete;
  Writer& operator=(const Writer&) = delete;

  size_t columns() const { return cols_.size(); }
  void add_bool(size_t c, bool v) { cols_[c].data.push_back(v ? 1 : 0); }
  void add_u64(size_t c, uint64_t v) { append(c, &v, 8); }
  void add_f64(size_t c, double v) { append(c, &v, 8); }
  // One row has been added to every column.
  void end_row() {
    if (++rows_ >= group_rows_) flush();
  }

  void close() {
    if (!f_) return;
    flush();
    Compact m;
    m.begin_struct();
    m.field_i32(1, 1);  // version
    m.field_list(2, kStruct, cols_.size() + 1);
    m.begin_struct();  // root
    m.field_string(4, "arrow_schema");
    m.field_i32(5, (int32_t)cols_.size());
    m.end_struct();
    for (auto& c : cols_) {
      m.begin_struct();
      m.field_i32(1, c.type == Type::Bool ? 0 : c.type == Type::UInt64 ? 2 : 5);  // BOOLEAN / INT64 / DOUBLE
      m.field_i32(3, 0);                                                         // REQUIRED
      m.field_string(4, c.name);
      if (c.type == Type::UInt64) {
        m.field_i32(6, 14);  // ConvertedType UINT_64
        m.field_struct(10);  // LogicalType
        m.field_struct(10);  // INTEGER
        m.field_byte(1, 64);     // bitWidth
        m.field_bool(2, false);  // isSigned
        m.end_struct();
        m.end_struct();
      }
      m.end_struct();
    }
    m.field_i64(3, (int64_t)total_rows_);
    m.field_list(4, kStruct, groups_.size());
    for (auto& g : groups_) {
      m.begin_struct();
      m.field_list(1, kStruct, g.chunks.size());
      int64_t bytes = 0;
      for (size_t k = 0; k < g.chunks.size(); ++k) {
        const Chunk& ch = g.chunks[k];
        bytes += ch.size;
        m.begin_struct();
        m.field_i64(2, ch.offset);  // file_offset
        m.field_struct(3);          // ColumnMetaData
        m.field_i32(1, cols_[k].type == Type::Bool ? 0 : cols_[k].type == Type::UInt64 ? 2 : 5);
        m.field_list(2, kI32, 1);
        m.elem_i32(0);  // PLAIN
        m.field_list(3, kBinary, 1);
        m.elem_string(cols_[k].name);
        m.field_i32(4, 1);  // SNAPPY
        m.field_i64(5, (int64_t)g.rows);
        m.field_i64(6, ch.uncompressed);
        m.field_i64(7, ch.size);
        m.field_i64(9, ch.offset);  // data_page_offset
        m.end_struct();
        m.end_struct();
      }
      m.field_i64(2, bytes);
      m.field_i64(3, (int64_t)g.rows);
      m.end_struct();
    }
    m.field_string(6, "vegas-gb300 parquet writer");
    m.end_struct();
    put(m.out.data(), m.out.size());
    const uint32_t len = (uint32_t)m.out.size();
    const uint8_t le[4] = {(uint8_t)len, (uint8_t)(len >> 8), (uint8_t)(len >> 16), (uint8_t)(len >> 24)};
    put(le, 4);
    put("PAR1", 4);
    const bool ok = std::fclose(f_) == 0;
    f_ = nullptr;
    if (!ok) throw IoError("std io error: cannot write " + tmp_);
    if (std::rename(tmp_.c_str(), path_.c_str()) != 0) std::fprintf(stderr, "error renaming parquet file: %s\n", tmp_.c_str());
  }

 private:
  struct Chunk {
    int64_t offset, size, uncompressed;  // size: page header + compressed values, as written
  };
  struct Group {
    size_t rows;
    std::vector<Chunk> chunks;
  };

  void append(size_t c, const void* p, size_t n) {
    const uint8_t* b = static_cast<const uint8_t*>(p);
    cols_[c].data.insert(cols_[c].data.end(), b, b + n);  // little-endian host (x86-64, aarch64)
  }
  void put(const void* p, size_t n) {
    if (std::fwrite(p, 1, n, f_) != n) throw IoError("std io error: cannot write " + tmp_);
    offset_ += (int64_t)n;
  }
  void flush() {
    if (rows_ == 0) return;
    Group g{rows_, {}};
    for (auto& c : cols_) {
      std::vector<uint8_t> values;
      if (c.type == Type::Bool) {  // PLAIN booleans: bit-packed, least significant bit first
        values.assign((rows_ + 7) / 8, 0);
        for (size_t i = 0; i < rows_; ++i)
          if (c.data[i]) values[i >> 3] |= (uint8_t)(1u << (i & 7));
      } else {
        values.swap(c.data);
      }
      const std::vector<uint8_t> packed = snappy::compress(values);
      Compact h;  // PageHeader
      h.begin_struct();
      h.field_i32(1, 0);  // DATA_PAGE
      h.field_i32(2, (int32_t)values.size());  // uncompressed_page_size
      h.field_i32(3, (int32_t)packed.size());  // compressed_page_size
      h.field_struct(5);  // DataPageHeader
      h.field_i32(1, (int32_t)rows_);
      h.field_i32(2, 0);  // PLAIN
      h.field_i32(3, 3);  // RLE (no levels: every column is required)
      h.field_i32(4, 3);
      h.end_struct();
      h.end_struct();
      const int64_t start = offset_;
      put(h.out.data(), h.out.size());
      put(packed.data(), packed.size());
      g.chunks.push_back(Chunk{start, offset_ - start, (int64_t)(h.out.size() + values.size())});
      c.data.clear();
    }
    total_rows_ += rows_;
    groups_.push_back(std::move(g));
    rows_ = 0;
  }

  std::string path_, tmp_;
  size_t group_rows_;
  FILE* f_ = nullptr;
  std::vector<Column> cols_;
  std::vector<Group> groups_;
  size_t rows_ = 0, total_rows_ = 0;
  int64_t offset_ = 0;
};

// Path::with_extension("parquet.tmp") of the reference: the file name's
// extension (after its last '.') replaced, or appended if it has none.
inline std::string with_extension(const std::string& path, const std::string& ext) {
  const size_t slash = path.find_last_of('/');
  const size_t name = slash == std::string::npos ? 0 : slash + 1;
  const size_t dot = path.find_last_of('.');
  if (dot != std::string::npos && dot > name) return path.substr(0, dot + 1) + ext;
  return path + "." + ext;
}

}  // namespace parquet
}  // namespace vegas
