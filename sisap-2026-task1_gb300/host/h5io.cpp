// h5io.cpp -- dataset reader/writer of the knng_main CLI: HDF5 through
// hdf5.h, or the knng container.
#include "h5io.h"

#include "hdf5.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>

namespace knngio {
namespace {

using File = std::unique_ptr<FILE, int (*)(FILE*)>;

float half_to_float(uint16_t h) {
  uint32_t s = uint32_t(h >> 15) << 31, e = (h >> 10) & 0x1f, m = h & 0x3ff, bits;
  if (e == 0) {
    if (m == 0) {
      bits = s;
    } else {
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

void get(FILE* f, void* p, size_t n, const std::string& path) {
  if (std::fread(p, 1, n, f) != n) throw std::runtime_error("truncated file: " + path);
}
void put(FILE* f, const void* p, size_t n, const std::string& path) {
  if (std::fwrite(p, 1, n, f) != n) throw std::runtime_error("short write: " + path);
}
void put_name(FILE* f, uint32_t tag, const std::string& nm, const std::string& path) {
  uint32_t len = uint32_t(nm.size());
  put(f, &tag, 4, path);
  put(f, &len, 4, path);
  put(f, nm.data(), nm.size(), path);
}
size_t elem(uint32_t t) { return t == 3 ? 2 : (t == 4 ? 1 : 4); }

}  // namespace

Matrix read_matrix(const std::string& path, const std::string& name_in) {
  const std::string name = (!name_in.empty() && name_in[0] == '/') ? name_in.substr(1) : name_in;
  File f(std::fopen(path.c_str(), "rb"), &std::fclose);
  if (!f) throw std::runtime_error("unable to open file " + path);
  char magic[8] = {0};
  const bool short_file = std::fread(magic, 1, 8, f.get()) != 8;
  if (short_file || std::memcmp(magic, "KNNGH5S1", 8) != 0) {
    f.reset();
    if (!h5::is_hdf5(path)) throw std::runtime_error("neither an HDF5 nor a knng container file: " + path);
    h5::DatasetInfo info;
    Matrix m;
    m.data = h5::read_float(path, name, &info);
    if (info.dims.size() != 2) throw std::runtime_error("dataset " + name + " is not a matrix");
    m.rows = int64_t(info.dims[0]);
    m.cols = int64_t(info.dims[1]);
    return m;
  }
  for (;;) {
    uint32_t tag, len;
    if (std::fread(&tag, 4, 1, f.get()) != 1) break;
    get(f.get(), &len, 4, path);
    std::string nm(len, '\0');
    if (len) get(f.get(), &nm[0], len, path);
    if (tag == 1) {
      uint32_t type, rank;
      get(f.get(), &type, 4, path);
      get(f.get(), &rank, 4, path);
      if (rank > 8) throw std::runtime_error("bad dataset header in " + path);
      std::vector<uint64_t> dims(rank);
      uint64_t count = 1;
      for (auto& v : dims) {
        get(f.get(), &v, 8, path);
        count *= v;
      }
      if (nm != name) {
        std::fseek(f.get(), long(count * elem(type)), SEEK_CUR);
        continue;
      }
      if (rank != 2) throw std::runtime_error("dataset " + name + " is not a matrix");
      Matrix m;
      m.rows = int64_t(dims[0]);
      m.cols = int64_t(dims[1]);
      m.data.resize(count);
      if (type == 1) {
        get(f.get(), m.data.data(), count * 4, path);
      } else {
        std::vector<unsigned char> raw(count * elem(type));
        get(f.get(), raw.data(), raw.size(), path);
        for (uint64_t i = 0; i < count; ++i) {
          const unsigned char* p = raw.data() + i * elem(type);
          if (type == 2) { int32_t v; std::memcpy(&v, p, 4); m.data[i] = float(v); }
          else if (type == 3) { uint16_t v; std::memcpy(&v, p, 2); m.data[i] = half_to_float(v); }
          else { int8_t v; std::memcpy(&v, p, 1); m.data[i] = float(v); }
        }
      }
      return m;
    } else if (tag == 2) {
      uint64_t n;
      get(f.get(), &n, 8, path);
      std::fseek(f.get(), long(n), SEEK_CUR);
    } else if (tag == 3) {
      std::fseek(f.get(), 4, SEEK_CUR);
    } else {
      throw std::runtime_error("unknown record in " + path);
    }
  }
  throw std::runtime_error("dataset not found: /" + name);
}

Result read_result(const std::string& path) {
  Result r;
  File f(std::fopen(path.c_str(), "rb"), &std::fclose);
  if (!f) throw std::runtime_error("unable to open file " + path);
  char magic[8] = {0};
  if (std::fread(magic, 1, 8, f.get()) != 8 || std::memcmp(magic, "KNNGH5S1", 8) != 0) {
    f.reset();
    if (!h5::is_hdf5(path)) throw std::runtime_error("neither an HDF5 nor a knng container file: " + path);
    h5::DatasetInfo ki, di;
    r.knns = h5::read_int32(path, "knns", &ki);
    r.dists = h5::read_float(path, "dists", &di);
    if (ki.dims.size() != 2 || ki.dims != di.dims) throw std::runtime_error("knns/dists shapes differ in " + path);
    r.rows = int64_t(ki.dims[0]);
    r.cols = int64_t(ki.dims[1]);
    for (const auto& [k, v] : h5::read_attributes(path, "/")) {
      if (k == "algo") r.algo = v;
      else if (k == "task") r.task = v;
      else if (k == "params") r.params = v;
      else if (k == "buildtime") r.buildtime = std::strtof(v.c_str(), nullptr);
      else if (k == "querytime") r.querytime = std::strtof(v.c_str(), nullptr);
    }
    return r;
  }
  std::vector<uint64_t> kd, dd;
  for (;;) {
    uint32_t tag, len;
    if (std::fread(&tag, 4, 1, f.get()) != 1) break;
    get(f.get(), &len, 4, path);
    std::string nm(len, '\0');
    if (len) get(f.get(), &nm[0], len, path);
    if (tag == 1) {
      uint32_t type, rank;
      get(f.get(), &type, 4, path);
      get(f.get(), &rank, 4, path);
      if (rank > 8) throw std::runtime_error("bad dataset header in " + path);
      std::vector<uint64_t> dims(rank);
      uint64_t count = 1;
      for (auto& v : dims) {
        get(f.get(), &v, 8, path);
        count *= v;
      }
      if (nm == "knns" && type == 2) {
        r.knns.resize(count);
        get(f.get(), r.knns.data(), count * 4, path);
        kd = dims;
      } else if (nm == "dists" && type == 1) {
        r.dists.resize(count);
        get(f.get(), r.dists.data(), count * 4, path);
        dd = dims;
      } else {
        std::fseek(f.get(), long(count * elem(type)), SEEK_CUR);
      }
    } else if (tag == 2) {
      uint64_t n;
      get(f.get(), &n, 8, path);
      std::string v(n, '\0');
      if (n) get(f.get(), &v[0], n, path);
      if (nm == "algo") r.algo = v;
      else if (nm == "task") r.task = v;
      else if (nm == "params") r.params = v;
    } else if (tag == 3) {
      float v;
      get(f.get(), &v, 4, path);
      if (nm == "buildtime") r.buildtime = v;
      else if (nm == "querytime") r.querytime = v;
    } else {
      throw std::runtime_error("unknown record in " + path);
    }
  }
  if (kd.size() != 2 || kd != dd) throw std::runtime_error("no knns/dists (i32/f32 matrices of one shape) in " + path);
  r.rows = int64_t(kd[0]);
  r.cols = int64_t(kd[1]);
  return r;
}

void write_result(const std::string& path, const Output& o, Format format) {
  if (format == Format::kHdf5) {
    const std::vector<uint64_t> dims = {uint64_t(o.rows), uint64_t(o.cols)};
    h5::write_file(path, {{"knns", 0, dims, o.knns}, {"dists", 1, dims, o.dists}},
                   {{"algo", true, o.algo, 0.0f},
                    {"task", true, o.task, 0.0f},
                    {"buildtime", false, "", o.buildtime},
                    {"querytime", false, "", o.querytime},
                    {"params", true, o.params, 0.0f}});
    return;
  }
  File f(std::fopen(path.c_str(), "wb"), &std::fclose);
  if (!f) throw std::runtime_error("unable to create file " + path);
  put(f.get(), "KNNGH5S1", 8, path);
  const uint64_t dims[2] = {uint64_t(o.rows), uint64_t(o.cols)};
  const uint32_t rank = 2;
  auto dataset = [&](const char* nm, uint32_t type, const void* p) {
    put_name(f.get(), 1, nm, path);
    put(f.get(), &type, 4, path);
    put(f.get(), &rank, 4, path);
    put(f.get(), dims, 16, path);
    put(f.get(), p, size_t(o.rows) * size_t(o.cols) * 4, path);
  };
  dataset("knns", 2, o.knns);
  dataset("dists", 1, o.dists);
  auto sattr = [&](const char* nm, const std::string& v) {
    put_name(f.get(), 2, nm, path);
    uint64_t n = v.size();
    put(f.get(), &n, 8, path);
    put(f.get(), v.data(), v.size(), path);
  };
  auto fattr = [&](const char* nm, float v) {
    put_name(f.get(), 3, nm, path);
    put(f.get(), &v, 4, path);
  };
  sattr("algo", o.algo);
  sattr("task", o.task);
  fattr("buildtime", o.buildtime);
  fattr("querytime", o.querytime);
  sattr("params", o.params);
}

}  // namespace knngio
