// hdf5.h -- a small HDF5 reader and writer for the knng_main CLI.
//
// The reference reads /train with the HDF5 C++ library and writes knns/dists
// plus five root attributes (src/main.cpp:149-177, 459-480).  libhdf5 is not
// available in this image, so the CLI carries its own implementation of the
// part of the HDF5 file format (the published "HDF5 File Format
// Specification") that those files use:
//   reading : superblock versions 0-3 (with a user block), object headers v1
//             and v2 with continuation blocks, groups as symbol tables (v1
//             B-tree + local heap) or compact link messages, datasets with
//             contiguous, compact or v1-B-tree chunked layout, deflate and
//             shuffle filters (deflate when built with zlib), fixed-point and
//             IEEE floating-point element types of 1-8 bytes, either byte order;
//   writing : the layout libhdf5 produces with its default ("earliest")
//             settings -- superblock v0, symbol-table groups (the root and one
//             level below it), v1 object headers, contiguous int32 / float32 /
//             float16 datasets, variable-length string and scalar float
//             attributes on the root.
// Dense (fractal-heap) groups, compound/variable-length element types and
// other filters are rejected with a clear error.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace knngio {
namespace h5 {

struct DatasetInfo {
  std::string name;
  int type_class = -1;    // 0 fixed-point, 1 floating-point
  int type_size = 0;      // bytes per element
  bool little_endian = true;
  bool is_signed = true;
  std::vector<uint64_t> dims;
};

bool is_hdf5(const std::string& path);

// Datasets reachable from the root group (paths without the leading '/').
std::vector<DatasetInfo> list_datasets(const std::string& path);

// Reads dataset `name` (leading '/' optional) converted to float32 (or int32),
// row-major.  Throws std::runtime_error with the reason on failure.
std::vector<float> read_float(const std::string& path, const std::string& name, DatasetInfo* info);
std::vector<int32_t> read_int32(const std::string& path, const std::string& name, DatasetInfo* info);

// (name, value) of every attribute of the object at `object` ("/" is the
// root group); strings as text, numbers as comma-separated %.9g values.
std::vector<std::pair<std::string, std::string>> read_attributes(const std::string& path, const std::string& object);

struct WriteDataset {
  std::string name;  // "name" or "group/name" (one group level)
  int type_class;    // 0 int32, 1 float32, 2 float16 (raw IEEE half bits)
  std::vector<uint64_t> dims;
  const void* data;
};
struct WriteAttr {
  std::string name;
  bool is_string;
  std::string s;
  float f;
};
// Writes a new file (truncating) with the datasets in the root group and the
// attributes on the root group.  Throws std::runtime_error on failure.
void write_file(const std::string& path, const std::vector<WriteDataset>& ds, const std::vector<WriteAttr>& attrs);

}  // namespace h5
}  // namespace knngio
