// No-op stand-in for the HDF5 C++ API header.
//
// Test infrastructure only. The reference's microphysics headers include
// <H5Cpp.h> through src/utilitites/pch.h:49, src/utilitites/utils.h:624-1380
// (struct Output) writes HDF5 files and src/utilitites/H5Easy.h reads them
// (pulled in by the blastwave and EATS headers). None of that is on the paths
// the oracle harnesses drive, so these declarations only need to let the
// headers compile. Datasets and scalar attributes live in an in-memory store
// keyed by "file//group/name" (pbag_h5): what the reference writes is kept
// there instead of in a file (its dynamics and spectrum writers, read back by
// a harness), and what a harness puts there is what the reference's loaders
// read (e.g. the ejecta initial data of ejecta_id.h), without HDF5.
#ifndef PBAG_ORACLE_SHIM_H5CPP_H
#define PBAG_ORACLE_SHIM_H5CPP_H

#include <unistd.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

typedef unsigned long long hsize_t;
typedef long long hid_t;
typedef std::string H5std_string;
enum H5T_class_t { H5T_NO_CLASS = -1, H5T_INTEGER = 0, H5T_FLOAT = 1 };
enum H5T_order_t { H5T_ORDER_ERROR = -1, H5T_ORDER_LE = 0, H5T_ORDER_BE = 1 };
enum H5S_class_t { H5S_SCALAR = 0, H5S_SIMPLE = 1 };
#define H5F_ACC_TRUNC 2u
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_RDWR 1u
#define H5P_DEFAULT 0

namespace pbag_h5 {
struct Entry {
  std::vector<double> data;
  std::vector<unsigned long long> dims;
};
inline std::map<std::string, Entry>& datasets() {
  static std::map<std::string, Entry> m;
  return m;
}
inline std::map<std::string, double>& attributes() {
  static std::map<std::string, double> m;
  return m;
}
inline void put(const std::string& file, const std::string& name, const std::vector<double>& data,
                const std::vector<unsigned long long>& dims) {
  datasets()[file + "//" + name] = Entry{data, dims};
}
inline void put_attr(const std::string& file, const std::string& name, double v) {
  attributes()[file + "//" + name] = v;
}
inline const Entry* find(const std::string& key) {
  auto it = datasets().find(key);
  return it == datasets().end() ? nullptr : &it->second;
}
// Optional write-through log of what the program writes (a file descriptor,
// -1: off): per dataset 'D', key, rank, dims, count, values; per attribute 'A',
// key, value. Written with write(2) as each write happens, so that it holds
// everything written before the program's exit path misbehaves.
inline int& log_fd() {
  static int fd = -1;
  return fd;
}
inline void log_bytes(const void* p, size_t n) {
  const char* c = static_cast<const char*>(p);
  while (n > 0 && log_fd() >= 0) {
    const long w = (long)::write(log_fd(), c, n);
    if (w <= 0) return;
    c += w;
    n -= (size_t)w;
  }
}
inline void log_key(char tag, const std::string& key) {
  const uint32_t n = (uint32_t)key.size();
  log_bytes(&tag, 1);
  log_bytes(&n, sizeof n);
  log_bytes(key.data(), n);
}
inline void log_dataset(const std::string& key, const std::vector<unsigned long long>& dims, const double* v,
                        uint64_t n) {
  if (log_fd() < 0) return;
  log_key('D', key);
  const uint32_t r = (uint32_t)dims.size();
  log_bytes(&r, sizeof r);
  log_bytes(dims.data(), sizeof(unsigned long long) * r);
  log_bytes(&n, sizeof n);
  log_bytes(v, sizeof(double) * n);
}
inline void log_attr(const std::string& key, double v) {
  if (log_fd() < 0) return;
  log_key('A', key);
  log_bytes(&v, sizeof v);
}
}  // namespace pbag_h5

namespace H5 {
struct PredType {
  static const PredType NATIVE_DOUBLE, NATIVE_INT, IEEE_F32LE, IEEE_F64LE, IEEE_F32BE, IEEE_F64BE, STD_I8LE,
      STD_I8BE, STD_I16LE, STD_I16BE, STD_I32LE, STD_I32BE, STD_I64LE, STD_I64BE, STD_U32LE;
  bool operator==(const PredType&) const { return false; }
};
inline const PredType PredType::NATIVE_DOUBLE{}, PredType::NATIVE_INT{}, PredType::IEEE_F32LE{},
    PredType::IEEE_F64LE{}, PredType::IEEE_F32BE{}, PredType::IEEE_F64BE{}, PredType::STD_I8LE{},
    PredType::STD_I8BE{}, PredType::STD_I16LE{}, PredType::STD_I16BE{}, PredType::STD_I32LE{},
    PredType::STD_I32BE{}, PredType::STD_I64LE{}, PredType::STD_I64BE{}, PredType::STD_U32LE{};
struct Exception {
  static void dontPrint() {}
  void printErrorStack() const {}
  std::string getDetailMsg() const { return {}; }
};
struct FileIException : Exception {};
struct GroupIException : Exception {};
struct DataSetIException : Exception {};
struct DataSpaceIException : Exception {};
struct AttributeIException : Exception {};
struct DataTypeIException : Exception {};

struct DataType {
  DataType() {}
  DataType(const PredType&) {}
  H5T_class_t getClass() const { return H5T_FLOAT; }
  unsigned long getSize() const { return 8; }
  void close() {}
};
struct IntType : DataType {
  IntType() {}
  IntType(const PredType&) {}
  H5T_order_t getOrder(H5std_string&) const { return H5T_ORDER_LE; }
  H5T_order_t getOrder() const { return H5T_ORDER_LE; }
};
struct FloatType : DataType {
  H5T_order_t getOrder(H5std_string&) const { return H5T_ORDER_LE; }
};
struct DataSpace {
  std::vector<unsigned long long> dims;
  DataSpace() {}
  DataSpace(int) {}
  DataSpace(int rank, const hsize_t* d) : dims(d, d + rank) {}
  DataSpace(H5S_class_t) {}
  int getSimpleExtentNdims() const { return (int)dims.size(); }
  int getSimpleExtentDims(hsize_t* d, hsize_t* = nullptr) const {
    for (size_t i = 0; i < dims.size(); ++i) d[i] = dims[i];
    return (int)dims.size();
  }
  long getSimpleExtentNpoints() const {
    long n = dims.empty() ? 0 : 1;
    for (unsigned long long d : dims) n *= (long)d;
    return n;
  }
  void close() {}
};
struct Attribute {
  std::string key;
  void write(const DataType&, const void* v) {
    if (key.empty()) return;
    pbag_h5::attributes()[key] = *static_cast<const double*>(v);
    pbag_h5::log_attr(key, *static_cast<const double*>(v));
  }
  void read(const DataType&, void* v) const {
    auto it = pbag_h5::attributes().find(key);
    *static_cast<double*>(v) = it == pbag_h5::attributes().end() ? -1. : it->second;
  }
  DataType getDataType() const { return {}; }
  unsigned long long getStorageSize() const { return 0; }
};
struct DataSet {
  std::string key;
  std::vector<unsigned long long> dims;
  void write(const void* buf, const PredType&) {
    if (key.empty()) return;
    size_t n = dims.empty() ? 0 : 1;
    for (unsigned long long d : dims) n *= (size_t)d;
    const double* in = static_cast<const double*>(buf);
    pbag_h5::datasets()[key] = pbag_h5::Entry{std::vector<double>(in, in + n), dims};
    pbag_h5::log_dataset(key, dims, in, n);
  }
  void read(void* buf, const PredType&) const {
    if (const pbag_h5::Entry* e = pbag_h5::find(key)) {
      double* out = static_cast<double*>(buf);
      for (size_t i = 0; i < e->data.size(); ++i) out[i] = e->data[i];
    }
  }
  void close() {}
  DataType getDataType() const { return {}; }
  DataSpace getSpace() const {
    DataSpace s;
    if (const pbag_h5::Entry* e = pbag_h5::find(key)) s.dims = e->dims;
    return s;
  }
  FloatType getFloatType() const { return {}; }
  IntType getIntType() const { return {}; }
};
struct Group {
  std::string path;
  Group() {}
  explicit Group(const std::string& p) : path(p) {}
  DataSet createDataSet(const std::string& n, const DataType&, const DataSpace& sp) {
    return DataSet{path + "/" + n, sp.dims};
  }
  DataSet createDataSet(const std::string& n, const PredType&, const DataSpace& sp) {
    return DataSet{path + "/" + n, sp.dims};
  }
  Attribute createAttribute(const std::string& n, const DataType&, const DataSpace&) {
    return Attribute{path + "/" + n};
  }
  DataSet openDataSet(const std::string& n) const { return DataSet{path + "/" + n}; }
  long getId() const { return 0; }
  void close() {}
};
struct H5File {
  std::string name;
  H5File() {}
  H5File(const std::string& n, unsigned) : name(n) {}
  DataSet createDataSet(const std::string& n, const DataType&, const DataSpace& sp) {
    return DataSet{name + "//" + n, sp.dims};
  }
  DataSet createDataSet(const std::string& n, const PredType&, const DataSpace& sp) {
    return DataSet{name + "//" + n, sp.dims};
  }
  Attribute createAttribute(const std::string& n, const DataType&, const DataSpace&) {
    return Attribute{name + "//" + n};
  }
  Group createGroup(const std::string& g) { return Group(name + "//" + g); }
  Group openGroup(const std::string& g) { return Group(name + "//" + g); }
  DataSet openDataSet(const std::string& v) const { return DataSet{name + "//" + v}; }
  Attribute openAttribute(const std::string& k) const { return Attribute{name + "//" + k}; }
  bool attrExists(const std::string& k) const { return pbag_h5::attributes().count(name + "//" + k) > 0; }
  hid_t getId() const { return 0; }
  void close() {}
};
}  // namespace H5
inline int H5Lexists(hid_t, const char*, int) { return 0; }

#endif
