// No-op stand-in for the HDF5 C++ API header.
//
// Test infrastructure only. The reference's microphysics headers include
// <H5Cpp.h> through src/utilitites/pch.h:49, src/utilitites/utils.h:624-1380
// (struct Output) writes HDF5 files and src/utilitites/H5Easy.h reads them
// (pulled in by the blastwave and EATS headers). None of that is on the paths
// the oracle harnesses drive, so these declarations only need to let the
// headers compile; every method is an empty inline body that is never called.
#ifndef PBAG_ORACLE_SHIM_H5CPP_H
#define PBAG_ORACLE_SHIM_H5CPP_H

#include <string>

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
  DataSpace() {}
  DataSpace(int) {}
  DataSpace(int, const hsize_t*) {}
  DataSpace(H5S_class_t) {}
  int getSimpleExtentNdims() const { return 0; }
  int getSimpleExtentDims(hsize_t*, hsize_t* = nullptr) const { return 0; }
  long getSimpleExtentNpoints() const { return 0; }
  void close() {}
};
struct Attribute {
  template <typename... A> void write(A&&...) {}
  template <typename... A> void read(A&&...) const {}
  DataType getDataType() const { return {}; }
  unsigned long long getStorageSize() const { return 0; }
};
struct DataSet {
  void write(const void*, const PredType&) {}
  void read(void*, const PredType&) const {}
  void close() {}
  DataType getDataType() const { return {}; }
  DataSpace getSpace() const { return {}; }
  FloatType getFloatType() const { return {}; }
  IntType getIntType() const { return {}; }
};
struct Group {
  Group() {}
  template <typename... A> DataSet createDataSet(A&&...) { return {}; }
  template <typename... A> Attribute createAttribute(A&&...) { return {}; }
  DataSet openDataSet(const std::string&) const { return {}; }
  long getId() const { return 0; }
  void close() {}
};
struct H5File {
  H5File() {}
  H5File(const std::string&, unsigned) {}
  template <typename... A> DataSet createDataSet(A&&...) { return {}; }
  template <typename... A> Attribute createAttribute(A&&...) { return {}; }
  Group createGroup(const std::string&) { return {}; }
  Group openGroup(const std::string&) { return {}; }
  DataSet openDataSet(const std::string&) const { return {}; }
  Attribute openAttribute(const std::string&) const { return {}; }
  bool attrExists(const std::string&) const { return false; }
  hid_t getId() const { return 0; }
  void close() {}
};
}  // namespace H5
inline int H5Lexists(hid_t, const char*, int) { return 0; }

#endif
