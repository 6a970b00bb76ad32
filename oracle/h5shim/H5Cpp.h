// H5Cpp.h -- I/O-only stand-in for the HDF5 C++ API subset that the reference
// src/main.cpp uses, so that the unmodified reference compiles in an image
// without libhdf5.  TEST INFRASTRUCTURE ONLY (oracle/_ref is built with it).
//
// Datasets and attributes live in a flat "knng container" file (the same
// format that sisap-2026-task1_gb300/h5container.py and the knng_main CLI read
// and write):
//   magic "KNNGH5S1"
//   records until end of file, each:
//     u32 tag (1 dataset, 2 string attribute, 3 float attribute)
//     u32 name length, name bytes (no leading '/')
//     dataset : u32 type (1 f32, 2 i32, 3 f16, 4 i8), u32 rank, u64 dims[rank],
//               raw little-endian row-major data
//     string  : u64 length, bytes
//     float   : f32
// API surface covered (reference call sites src/main.cpp:101-112, 149-177,
// 465-480): H5File(name, H5F_ACC_RDONLY | H5F_ACC_TRUNC), openDataSet,
// createDataSet, createAttribute, DataSet::getSpace/read/write,
// DataSpace(rank, dims) / DataSpace(H5S_SCALAR), getSimpleExtentDims,
// selectHyperslab(H5S_SELECT_SET, count, offset), StrType(0, H5T_VARIABLE),
// PredType::NATIVE_FLOAT / NATIVE_INT, Attribute::write, Exception.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0x0000u
#define H5F_ACC_TRUNC 0x0002u
#define H5T_VARIABLE ((size_t)(-1))

namespace H5 {

enum H5S_class_t { H5S_SCALAR = 0, H5S_SIMPLE = 1 };
enum H5S_seloper_t { H5S_SELECT_SET = 0 };

class Exception {
 public:
  explicit Exception(std::string m) : msg_(std::move(m)) {}
  std::string getDetailMsg() const { return msg_; }

 private:
  std::string msg_;
};

namespace shim {
enum : uint32_t { kF32 = 1, kI32 = 2, kF16 = 3, kI8 = 4, kStr = 100 };
inline size_t elem_size(uint32_t t) { return t == kF16 ? 2 : (t == kI8 ? 1 : 4); }
inline float half_to_float(uint16_t h) {
  uint32_t s = uint32_t(h >> 15) << 31, e = (h >> 10) & 0x1f, m = h & 0x3ff, bits;
  if (e == 0) {
    if (m == 0) {
      bits = s;
    } else {  // subnormal half: renormalise
      int sh = 0;
      while (!(m & 0x400)) { m <<= 1; ++sh; }
      bits = s | (uint32_t(127 - 15 - sh + 1) << 23) | ((m & 0x3ff) << 13);
    }
  } else if (e == 31) {
    bits = s | 0x7f800000u | (m << 13);
  } else {
    bits = s | ((e + 127 - 15) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}
struct Entry {
  uint32_t type = 0;
  std::vector<hsize_t> dims;
  long offset = 0;  // file offset of the raw data
};
struct FileState {
  std::string name;
  bool writable = false;
  FILE* fp = nullptr;
  std::map<std::string, Entry> index;
  ~FileState() {
    if (fp) std::fclose(fp);
  }
  void put(const void* p, size_t n) {
    if (std::fwrite(p, 1, n, fp) != n) throw Exception("short write to " + name);
  }
  void put_u32(uint32_t v) { put(&v, 4); }
  void put_u64(uint64_t v) { put(&v, 8); }
  void put_name(uint32_t tag, const std::string& nm) {
    put_u32(tag);
    put_u32(uint32_t(nm.size()));
    put(nm.data(), nm.size());
  }
};
inline std::string strip(const std::string& s) { return (!s.empty() && s[0] == '/') ? s.substr(1) : s; }
}  // namespace shim

class DataType {
 public:
  explicit DataType(uint32_t code = 0) : code_(code) {}
  uint32_t code() const { return code_; }

 private:
  uint32_t code_;
};

class PredType : public DataType {
 public:
  explicit PredType(uint32_t code) : DataType(code) {}
  static const PredType NATIVE_FLOAT;
  static const PredType NATIVE_INT;
};
inline const PredType PredType::NATIVE_FLOAT(shim::kF32);
inline const PredType PredType::NATIVE_INT(shim::kI32);

class StrType : public DataType {
 public:
  StrType(int /*dummy*/, size_t /*size*/) : DataType(shim::kStr) {}
};

class DataSpace {
 public:
  DataSpace(H5S_class_t) {}
  DataSpace(int rank, const hsize_t* dims, const hsize_t* = nullptr) : dims_(dims, dims + rank) {}
  int getSimpleExtentDims(hsize_t* dims, hsize_t* maxdims = nullptr) const {
    for (size_t i = 0; i < dims_.size(); ++i) {
      dims[i] = dims_[i];
      if (maxdims) maxdims[i] = dims_[i];
    }
    return int(dims_.size());
  }
  void selectHyperslab(H5S_seloper_t, const hsize_t* count, const hsize_t* start,
                       const hsize_t* = nullptr, const hsize_t* = nullptr) {
    count_.assign(count, count + dims_.size());
    start_.assign(start, start + dims_.size());
  }
  const std::vector<hsize_t>& dims() const { return dims_; }
  const std::vector<hsize_t>& sel_count() const { return count_; }
  const std::vector<hsize_t>& sel_start() const { return start_; }

 private:
  std::vector<hsize_t> dims_, count_, start_;
};

class Attribute {
 public:
  Attribute(std::shared_ptr<shim::FileState> f, std::string name, uint32_t type)
      : f_(std::move(f)), name_(std::move(name)), type_(type) {}
  void write(const DataType&, const std::string& value) {
    f_->put_name(2, name_);
    f_->put_u64(value.size());
    f_->put(value.data(), value.size());
  }
  void write(const DataType& t, const void* buf) {
    if (t.code() != shim::kF32 || type_ != shim::kF32) throw Exception("attribute type not supported");
    f_->put_name(3, name_);
    f_->put(buf, 4);
  }

 private:
  std::shared_ptr<shim::FileState> f_;
  std::string name_;
  uint32_t type_;
};

class DataSet {
 public:
  DataSet(std::shared_ptr<shim::FileState> f, std::string name, shim::Entry e)
      : f_(std::move(f)), name_(std::move(name)), e_(std::move(e)) {}
  DataSpace getSpace() const { return DataSpace(int(e_.dims.size()), e_.dims.data()); }
  // Reads the selected block of file_space (whole extent if none selected),
  // converted to mem_type (float or int32).
  void read(void* buf, const DataType& mem_type, const DataSpace& /*mem_space*/,
            const DataSpace& file_space) const {
    const size_t rank = e_.dims.size();
    std::vector<hsize_t> cnt = file_space.sel_count(), st = file_space.sel_start();
    if (cnt.empty()) { cnt = e_.dims; st.assign(rank, 0); }
    if (rank < 1 || rank > 2) throw Exception("only rank 1-2 datasets are supported");
    const hsize_t cols = rank == 2 ? e_.dims[1] : 1;
    const hsize_t c0 = rank == 2 ? st[1] : 0, nc = rank == 2 ? cnt[1] : 1;
    if (st[0] + cnt[0] > e_.dims[0] || c0 + nc > cols) throw Exception("hyperslab out of range");
    const size_t es = shim::elem_size(e_.type);
    std::vector<unsigned char> row(size_t(nc) * es);
    for (hsize_t r = 0; r < cnt[0]; ++r) {
      long off = e_.offset + long(((st[0] + r) * cols + c0) * es);
      if (std::fseek(f_->fp, off, SEEK_SET) != 0 || std::fread(row.data(), 1, row.size(), f_->fp) != row.size())
        throw Exception("short read from " + f_->name);
      for (hsize_t c = 0; c < nc; ++c) {
        double v;
        const unsigned char* p = row.data() + c * es;
        if (e_.type == shim::kF32) { float f; std::memcpy(&f, p, 4); v = f; }
        else if (e_.type == shim::kI32) { int32_t q; std::memcpy(&q, p, 4); v = q; }
        else if (e_.type == shim::kF16) { uint16_t h; std::memcpy(&h, p, 2); v = shim::half_to_float(h); }
        else { int8_t q; std::memcpy(&q, p, 1); v = q; }
        size_t o = size_t(r * nc + c);
        if (mem_type.code() == shim::kF32) static_cast<float*>(buf)[o] = float(v);
        else if (mem_type.code() == shim::kI32) static_cast<int32_t*>(buf)[o] = int32_t(v);
        else throw Exception("memory type not supported");
      }
    }
  }
  void write(const void* buf, const DataType& mem_type) {
    if (mem_type.code() != e_.type) throw Exception("memory type must match the dataset type");
    size_t n = 1;
    for (hsize_t v : e_.dims) n *= size_t(v);
    f_->put_name(1, name_);
    f_->put_u32(e_.type);
    f_->put_u32(uint32_t(e_.dims.size()));
    for (hsize_t v : e_.dims) f_->put_u64(v);
    f_->put(buf, n * shim::elem_size(e_.type));
  }

 private:
  std::shared_ptr<shim::FileState> f_;
  std::string name_;
  shim::Entry e_;
};

class H5File {
 public:
  H5File(const std::string& name, unsigned int flags) : f_(std::make_shared<shim::FileState>()) {
    f_->name = name;
    if (flags & H5F_ACC_TRUNC) {
      f_->writable = true;
      f_->fp = std::fopen(name.c_str(), "wb");
      if (!f_->fp) throw Exception("unable to create file " + name);
      f_->put("KNNGH5S1", 8);
      return;
    }
    f_->fp = std::fopen(name.c_str(), "rb");
    if (!f_->fp) throw Exception("unable to open file " + name);
    char magic[8];
    if (std::fread(magic, 1, 8, f_->fp) != 8 || std::memcmp(magic, "KNNGH5S1", 8) != 0)
      throw Exception("not a knng container file: " + name);
    for (;;) {
      uint32_t tag, len;
      if (std::fread(&tag, 4, 1, f_->fp) != 1) break;
      if (std::fread(&len, 4, 1, f_->fp) != 1) throw Exception("truncated record");
      std::string nm(len, '\0');
      if (len && std::fread(&nm[0], 1, len, f_->fp) != len) throw Exception("truncated record");
      if (tag == 1) {
        shim::Entry e;
        uint32_t rank;
        if (std::fread(&e.type, 4, 1, f_->fp) != 1 || std::fread(&rank, 4, 1, f_->fp) != 1 || rank > 8)
          throw Exception("bad dataset header");
        e.dims.resize(rank);
        size_t n = 1;
        for (uint32_t r = 0; r < rank; ++r) {
          uint64_t v;
          if (std::fread(&v, 8, 1, f_->fp) != 1) throw Exception("bad dataset header");
          e.dims[r] = v;
          n *= size_t(v);
        }
        e.offset = std::ftell(f_->fp);
        f_->index[nm] = e;
        std::fseek(f_->fp, long(n * shim::elem_size(e.type)), SEEK_CUR);
      } else if (tag == 2) {
        uint64_t n;
        if (std::fread(&n, 8, 1, f_->fp) != 1) throw Exception("bad attribute");
        std::fseek(f_->fp, long(n), SEEK_CUR);
      } else if (tag == 3) {
        std::fseek(f_->fp, 4, SEEK_CUR);
      } else {
        throw Exception("unknown record tag");
      }
    }
  }
  DataSet openDataSet(const std::string& name) const {
    auto it = f_->index.find(shim::strip(name));
    if (it == f_->index.end()) throw Exception("dataset not found: " + name);
    return DataSet(f_, it->first, it->second);
  }
  DataSet createDataSet(const std::string& name, const DataType& t, const DataSpace& sp) {
    if (!f_->writable) throw Exception("file is read-only");
    shim::Entry e;
    e.type = t.code();
    e.dims = sp.dims();
    return DataSet(f_, shim::strip(name), e);
  }
  Attribute createAttribute(const std::string& name, const DataType& t, const DataSpace&) {
    if (!f_->writable) throw Exception("file is read-only");
    return Attribute(f_, name, t.code());
  }

 private:
  std::shared_ptr<shim::FileState> f_;
};

}  // namespace H5
