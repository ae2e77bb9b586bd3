// Stand-in for the HDF5 C++ API (H5Cpp.h).  The reference's hdf5_interface.h, included by
// its mri_data.h, declares HDF5 wrappers and defines templates over these classes;
// oracle/_ref compiles those headers but never calls into HDF5, so every member aborts.
#ifndef ORACLE_REFSHIM_H5CPP_H
#define ORACLE_REFSHIM_H5CPP_H

#include <cstdio>
#include <cstdlib>
#include <string>

typedef unsigned long long hsize_t;

namespace H5 {

[[noreturn]] inline void h5_unavailable() {
  std::fprintf(stderr, "HDF5 stand-in: HDF5 is not available in this build\n");
  std::abort();
}

class Exception {
 public:
  static void dontPrint() {}
};
class FileIException : public Exception {};
class GroupIException : public Exception {};

class DataType {
 public:
  DataType() {}
  DataType(const DataType &) = default;
};
class PredType : public DataType {
 public:
  static const PredType NATIVE_DOUBLE, NATIVE_FLOAT, NATIVE_SHORT, NATIVE_UINT64, NATIVE_INT;
};
inline const PredType PredType::NATIVE_DOUBLE{}, PredType::NATIVE_FLOAT{}, PredType::NATIVE_SHORT{},
    PredType::NATIVE_UINT64{}, PredType::NATIVE_INT{};
class CompType : public DataType {
 public:
  explicit CompType(size_t) {}
  void insertMember(const std::string &, size_t, const DataType &) { h5_unavailable(); }
};
class DataSpace {
 public:
  DataSpace() {}
  DataSpace(int, const hsize_t *) {}
  int getSimpleExtentNdims() const { h5_unavailable(); }
  int getSimpleExtentDims(hsize_t *, hsize_t *) const { h5_unavailable(); }
  long getSelectNpoints() const { h5_unavailable(); }
};
class DataSet {
 public:
  DataSet() {}
  DataSpace getSpace() const { h5_unavailable(); }
  DataType getDataType() const { h5_unavailable(); }
  void read(void *, const DataType &) const { h5_unavailable(); }
  void write(const void *, const DataType &, const DataSpace &) const { h5_unavailable(); }
};
class Group {
 public:
  Group() {}
  DataSet openDataSet(const std::string &) const { h5_unavailable(); }
  DataSet createDataSet(const std::string &, const DataType &, const DataSpace &) const { h5_unavailable(); }
};
class H5File {
 public:
  H5File() {}
};

}  // namespace H5

#endif
