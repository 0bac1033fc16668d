// Minimal NetCDF classic-format (CDF-1 / CDF-2, 64-bit offsets) writer and
// reader for the reference's Snapshot and Probability files, written from the
// public format specification: big-endian header (magic, numrecs, dimension,
// global-attribute and variable lists), fixed-size variables followed by the
// record section in which every record holds each record variable's slab in
// variable order.  Only NC_DOUBLE variables and attributes are used.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace xf {
namespace nc {

struct Attr {
    std::string name;
    std::vector<double> values;
};

struct Var {
    std::string name;
    std::vector<int> dims;  // dimension ids
    std::vector<Attr> atts;
    // derived
    bool record = false;
    uint64_t vsize = 0;   // bytes of one record (record vars) or of the whole variable
    uint64_t begin = 0;
};

struct Dim {
    std::string name;
    uint64_t len;  // 0 = the unlimited (record) dimension
};

class Writer {
public:
    ~Writer() { close(); }
    // Creates (clobbers) a file; version 1 (CDF-1) or 2 (CDF-2, 64-bit offsets).
    bool create(const std::string& path, const std::vector<Dim>& dims, const std::vector<Var>& vars, int version = 2);
    // Appends one record: data[i] holds the slab of the i-th record variable.
    bool append(const std::vector<const double*>& data);
    // The same with some slabs already in the file's big-endian encoding
    // (be[i] set): those are written as given, without conversion.
    bool append(const std::vector<const void*>& data, const std::vector<bool>& be);
    bool sync();
    void close();
    uint64_t records() const { return numrecs_; }
    bool is_open() const { return f_ != nullptr; }

private:
    FILE* f_ = nullptr;
    std::vector<Dim> dims_;
    std::vector<Var> vars_;
    uint64_t numrecs_ = 0, recsize_ = 0, rec_begin_ = 0;
};

class Reader {
public:
    ~Reader() { close(); }
    bool open(const std::string& path);
    void close();
    int find_var(const std::string& name) const;
    uint64_t records() const { return numrecs_; }
    const std::vector<Dim>& dims() const { return dims_; }
    const std::vector<Var>& vars() const { return vars_; }
    // Values of one record of a record variable (or all of a fixed variable, rec ignored).
    bool read(int var, uint64_t rec, std::vector<double>& out);
    uint64_t count(int var) const;  // values per record (or total for fixed variables)

private:
    FILE* f_ = nullptr;
    int version_ = 1;
    std::vector<Dim> dims_;
    std::vector<Var> vars_;
    uint64_t numrecs_ = 0, recsize_ = 0;
};

}  // namespace nc
}  // namespace xf
