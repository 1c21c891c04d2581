// NetCDF classic-format file writer, host only: CDF-2 ("64-bit offset") and CDF-5
// ("64-bit data"), after the published netCDF classic format specification.
//
// The reference writes its snapshots and sanity records through the netCDF-4 C++ API
// (include/io/netCDF_writer.cpp:29-149, include/io/sanity_checks_netcdf_writer.cpp:25-71).
// Its data model (dimensions, one unlimited record dimension, typed variables, text,
// int and double attributes) is written here in the classic encoding, which every
// netCDF reader opens, without the netCDF or HDF5 libraries.
//
// Layout of a file: the header, then each fixed-size variable's data in definition
// order, then the records; record r holds every record variable's slab of that record,
// again in definition order.  All values are big-endian.  The header is laid out once
// (enddef) with spare room after it, so that global attributes added later (the
// reference adds its run metadata at the first snapshot) and the record count are
// rewritten in place without moving any data.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

namespace swe {
namespace nc {

enum Type : int {
    NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6,
    NC_UBYTE = 7, NC_USHORT = 8, NC_UINT = 9, NC_INT64 = 10, NC_UINT64 = 11,
};

// Size in bytes of one value of a type, 0 for an unknown type.
size_t type_size(int type);

// The netCDF default fill value of NC_DOUBLE (9.9692099683868690e+36).
constexpr double kFillDouble = 9.9692099683868690e+36;

// Byte-reverses n 8-byte values from src into dst (host order -> big-endian on a
// little-endian host; the copy is plain on a big-endian host).
void store_be64(void *dst, const void *src, size_t n);

class ClassicFile {
  public:
    ClassicFile() = default;
    ~ClassicFile();
    ClassicFile(const ClassicFile &) = delete;
    ClassicFile &operator=(const ClassicFile &) = delete;

    // Creates (truncates) the file, making missing parent directories; version 2 or 5.
    bool create(const std::string &path, int version);

    // Define phase.  len 0 makes the record (unlimited) dimension; at most one.
    int add_dim(const std::string &name, uint64_t len);
    int add_var(const std::string &name, int type, const std::vector<int> &dims);
    // var -1 = global.  Allowed before enddef, and for globals after it while the
    // header still fits its reserved room.
    bool put_att_text(int var, const std::string &name, const std::string &value);
    bool put_att_int(int var, const std::string &name, int32_t value);
    bool put_att_double(int var, const std::string &name, double value);

    // Lays out the data (fixed variables from the first multiple of 4096 after the
    // header plus `reserve` bytes) and writes the header.
    bool enddef(size_t reserve);

    // Writes big-endian bytes into a fixed variable at a byte offset within it.
    bool write_fixed(int var, const void *be, size_t nbytes, uint64_t offset = 0);
    // Writes big-endian bytes into record `rec` of a record variable.
    bool write_record(int var, uint64_t rec, const void *be, size_t nbytes,
                      uint64_t offset = 0);
    // Byte offset in the file of record `rec` of a record variable (of a fixed one: rec 0).
    uint64_t data_offset(int var, uint64_t rec) const;
    // Raises the header's record count to n (never lowers it).
    bool set_numrecs(uint64_t n);
    uint64_t numrecs() const { return numrecs_; }
    uint64_t var_bytes(int var) const;  // one record's (or the fixed variable's) bytes

    bool close();
    bool is_open() const { return fd_ >= 0; }
    int version() const { return version_; }
    std::string error() const {
        std::lock_guard<std::mutex> lk(err_mu_);
        return err_;
    }

    // Largest variable (per record) the CDF-2 encoding can describe, bytes.
    static constexpr uint64_t kCdf2VarLimit = 4294967292ull;  // 2^32 - 4

  private:
    struct Att {
        std::string name;
        int type;
        uint64_t nelems;
        std::vector<unsigned char> be;  // values, big-endian, unpadded
    };
    struct Dim {
        std::string name;
        uint64_t len;
    };
    struct Var {
        std::string name;
        int type;
        std::vector<int> dims;
        std::vector<Att> atts;
        bool record = false;
        uint64_t vsize = 0;  // bytes, padded to 4 (per record for record variables)
        uint64_t begin = 0;
    };

    std::vector<unsigned char> encode_header() const;
    bool write_header_locked();
    bool put_att(int var, Att a);
    bool pwrite_all(const void *p, size_t n, uint64_t off);
    bool fail(const std::string &m);

    int fd_ = -1;
    int version_ = 2;
    bool defined_ = false;
    std::vector<Dim> dims_;
    std::vector<Att> gatts_;
    std::vector<Var> vars_;
    uint64_t header_room_ = 0;  // bytes before the first data byte
    uint64_t recsize_ = 0;
    uint64_t numrecs_ = 0;
    mutable std::mutex mu_;  // header rewrites (record count, late attributes)
    mutable std::mutex err_mu_;
    std::string err_;
};

}  // namespace nc
}  // namespace swe
