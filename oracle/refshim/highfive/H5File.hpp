// TEST INFRASTRUCTURE (oracle build of the reference).  Minimal stand-in for
// the HighFive API surface that demonstrator/src/Particles.cpp uses for its
// snapshot writers (dump2file, dumpNNL).  HDF5 is not installed here and the
// harness never writes snapshots, so every call is a no-op.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

namespace HighFive {
class DataSpace {
public:
    DataSpace(std::size_t) {}
    DataSpace(const std::vector<std::size_t> &) {}
};
class DataSet {
public:
    template <class T> void write(const T &) {}
    template <class T> void read(T &) const {}
};
class File {
public:
    enum { ReadOnly = 1, ReadWrite = 2, Create = 4, Truncate = 8 };
    File(const std::string &, int) {}
    template <class T> DataSet createDataSet(const std::string &, const DataSpace &) { return DataSet(); }
    DataSet getDataSet(const std::string &) const { return DataSet(); }
};
}  // namespace HighFive
