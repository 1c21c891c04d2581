// NetCDF classic-format writer (CDF-2 and CDF-5); see swe_ncfile.h for the layout.
#include "swe_ncfile.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstring>
#include <filesystem>

namespace swe {
namespace nc {

namespace {

constexpr uint32_t TAG_DIMENSION = 0x0A, TAG_VARIABLE = 0x0B, TAG_ATTRIBUTE = 0x0C;

uint64_t pad4(uint64_t n) { return (n + 3) & ~uint64_t(3); }
uint64_t round_up(uint64_t n, uint64_t a) { return (n + a - 1) / a * a; }

void put_be(std::vector<unsigned char> &h, uint64_t v, int bytes) {
    for (int b = bytes - 1; b >= 0; --b) h.push_back((unsigned char)(v >> (8 * b)));
}

}  // namespace

size_t type_size(int type) {
    switch (type) {
        case NC_BYTE: case NC_CHAR: case NC_UBYTE: return 1;
        case NC_SHORT: case NC_USHORT: return 2;
        case NC_INT: case NC_FLOAT: case NC_UINT: return 4;
        case NC_DOUBLE: case NC_INT64: case NC_UINT64: return 8;
        default: return 0;
    }
}

void store_be64(void *dst, const void *src, size_t n) {
    const unsigned char *s = static_cast<const unsigned char *>(src);
    unsigned char *d = static_cast<unsigned char *>(dst);
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
    std::memmove(d, s, 8 * n);
#else
    for (size_t i = 0; i < n; ++i) {
        uint64_t v;
        std::memcpy(&v, s + 8 * i, 8);
        v = __builtin_bswap64(v);
        std::memcpy(d + 8 * i, &v, 8);
    }
#endif
}

ClassicFile::~ClassicFile() {
    if (fd_ >= 0) ::close(fd_);
}

bool ClassicFile::fail(const std::string &m) {
    std::lock_guard<std::mutex> lk(err_mu_);
    if (err_.empty()) err_ = m;
    return false;
}

bool ClassicFile::create(const std::string &path, int version) {
    if (version != 2 && version != 5) return fail("netCDF: version must be 2 or 5");
    std::error_code ec;
    const std::filesystem::path p(path);
    if (p.has_parent_path()) std::filesystem::create_directories(p.parent_path(), ec);
    fd_ = ::open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC | O_CLOEXEC, 0644);
    if (fd_ < 0) return fail("netCDF: cannot create " + path + ": " + std::strerror(errno));
    version_ = version;
    return true;
}

int ClassicFile::add_dim(const std::string &name, uint64_t len) {
    if (defined_ || name.empty()) return -1;
    for (const Dim &d : dims_)
        if (d.name == name || (len == 0 && d.len == 0)) return -1;
    dims_.push_back({name, len});
    return (int)dims_.size() - 1;
}

int ClassicFile::add_var(const std::string &name, int type, const std::vector<int> &dims) {
    if (defined_ || name.empty() || type_size(type) == 0) return -1;
    if (version_ != 5 && type > NC_DOUBLE) return -1;  // the extended types need CDF-5
    for (size_t k = 0; k < dims.size(); ++k) {
        if (dims[k] < 0 || dims[k] >= (int)dims_.size()) return -1;
        if (dims_[dims[k]].len == 0 && k != 0) return -1;  // record dimension first only
    }
    for (const Var &v : vars_)
        if (v.name == name) return -1;
    Var v;
    v.name = name;
    v.type = type;
    v.dims = dims;
    v.record = !dims.empty() && dims_[dims[0]].len == 0;
    vars_.push_back(std::move(v));
    return (int)vars_.size() - 1;
}

bool ClassicFile::put_att(int var, Att a) {
    if (var < -1 || var >= (int)vars_.size()) return fail("netCDF: bad variable id");
    if (defined_ && var != -1) return fail("netCDF: variable attribute after enddef");
    if (version_ != 5 && a.type > NC_DOUBLE) return fail("netCDF: attribute type needs CDF-5");
    std::vector<Att> &list = var == -1 ? gatts_ : vars_[var].atts;
    std::lock_guard<std::mutex> lk(mu_);
    size_t slot = list.size();
    Att old;
    bool replaced = false;
    for (size_t k = 0; k < list.size(); ++k)
        if (list[k].name == a.name) {
            slot = k;
            old = list[k];
            replaced = true;
        }
    if (replaced)
        list[slot] = std::move(a);
    else
        list.push_back(std::move(a));
    if (!defined_) return true;
    if (encode_header().size() > header_room_) {
        if (replaced)
            list[slot] = std::move(old);
        else
            list.pop_back();
        return fail("netCDF: header room exhausted by a late attribute");
    }
    return write_header_locked();
}

bool ClassicFile::put_att_text(int var, const std::string &name, const std::string &value) {
    Att a{name, NC_CHAR, value.size(), std::vector<unsigned char>(value.begin(), value.end())};
    return put_att(var, std::move(a));
}

bool ClassicFile::put_att_int(int var, const std::string &name, int32_t value) {
    Att a{name, NC_INT, 1, {}};
    put_be(a.be, (uint32_t)value, 4);
    return put_att(var, std::move(a));
}

bool ClassicFile::put_att_double(int var, const std::string &name, double value) {
    Att a{name, NC_DOUBLE, 1, std::vector<unsigned char>(8)};
    store_be64(a.be.data(), &value, 1);
    return put_att(var, std::move(a));
}

std::vector<unsigned char> ClassicFile::encode_header() const {
    std::vector<unsigned char> h;
    const int nn = version_ == 5 ? 8 : 4;  // NON_NEG width
    auto name = [&](const std::string &s) {
        put_be(h, s.size(), nn);
        h.insert(h.end(), s.begin(), s.end());
        while (h.size() % 4) h.push_back(0);
    };
    auto att_list = [&](const std::vector<Att> &atts) {
        if (atts.empty()) {  // ABSENT
            put_be(h, 0, 4);
            put_be(h, 0, nn);
            return;
        }
        put_be(h, TAG_ATTRIBUTE, 4);
        put_be(h, atts.size(), nn);
        for (const Att &a : atts) {
            name(a.name);
            put_be(h, (uint32_t)a.type, 4);
            put_be(h, a.nelems, nn);
            h.insert(h.end(), a.be.begin(), a.be.end());
            while (h.size() % 4) h.push_back(0);
        }
    };
    h.push_back('C');
    h.push_back('D');
    h.push_back('F');
    h.push_back((unsigned char)version_);
    put_be(h, numrecs_, nn);
    if (dims_.empty()) {
        put_be(h, 0, 4);
        put_be(h, 0, nn);
    } else {
        put_be(h, TAG_DIMENSION, 4);
        put_be(h, dims_.size(), nn);
        for (const Dim &d : dims_) {
            name(d.name);
            put_be(h, d.len, nn);
        }
    }
    att_list(gatts_);
    if (vars_.empty()) {
        put_be(h, 0, 4);
        put_be(h, 0, nn);
    } else {
        put_be(h, TAG_VARIABLE, 4);
        put_be(h, vars_.size(), nn);
        for (const Var &v : vars_) {
            name(v.name);
            put_be(h, v.dims.size(), nn);
            for (int d : v.dims) put_be(h, (uint64_t)d, nn);
            att_list(v.atts);
            put_be(h, (uint32_t)v.type, 4);
            put_be(h, v.vsize, nn);
            put_be(h, v.begin, 8);  // OFFSET is 64-bit in CDF-2 and CDF-5
        }
    }
    return h;
}

bool ClassicFile::enddef(size_t reserve) {
    if (fd_ < 0) return fail("netCDF: file not open");
    if (defined_) return fail("netCDF: enddef called twice");
    for (const Dim &d : dims_)
        if (version_ != 5 && d.len > 0x7fffffffull) return fail("netCDF: dimension too long for CDF-2");
    for (Var &v : vars_) {
        uint64_t n = type_size(v.type);
        for (size_t k = v.record ? 1 : 0; k < v.dims.size(); ++k) n *= dims_[v.dims[k]].len;
        v.vsize = pad4(n);
        if (version_ != 5 && v.vsize > kCdf2VarLimit)
            return fail("netCDF: variable " + v.name + " too large for CDF-2 (use CDF-5)");
    }
    const uint64_t hsize = encode_header().size();
    header_room_ = round_up(hsize + reserve, 4096);
    uint64_t off = header_room_;
    for (Var &v : vars_)
        if (!v.record) {
            v.begin = off;
            off += v.vsize;
        }
    off = round_up(off, 4096);
    recsize_ = 0;
    for (Var &v : vars_)
        if (v.record) {
            v.begin = off + recsize_;
            recsize_ += v.vsize;
        }
    defined_ = true;
    std::lock_guard<std::mutex> lk(mu_);
    return write_header_locked();
}

bool ClassicFile::write_header_locked() {
    const std::vector<unsigned char> h = encode_header();
    return pwrite_all(h.data(), h.size(), 0);
}

bool ClassicFile::pwrite_all(const void *p, size_t n, uint64_t off) {
    const char *c = static_cast<const char *>(p);
    while (n > 0) {
        const ssize_t w = ::pwrite(fd_, c, n, (off_t)off);
        if (w < 0) {
            if (errno == EINTR) continue;
            return fail(std::string("netCDF: write failed: ") + std::strerror(errno));
        }
        if (w == 0) return fail("netCDF: write made no progress");
        c += w;
        n -= (size_t)w;
        off += (uint64_t)w;
    }
    return true;
}

uint64_t ClassicFile::var_bytes(int var) const {
    if (var < 0 || var >= (int)vars_.size()) return 0;
    const Var &v = vars_[var];
    uint64_t n = type_size(v.type);
    for (size_t k = v.record ? 1 : 0; k < v.dims.size(); ++k) n *= dims_[v.dims[k]].len;
    return n;
}

uint64_t ClassicFile::data_offset(int var, uint64_t rec) const {
    const Var &v = vars_[var];
    return v.begin + (v.record ? rec * recsize_ : 0);
}

bool ClassicFile::write_fixed(int var, const void *be, size_t nbytes, uint64_t offset) {
    if (!defined_ || var < 0 || var >= (int)vars_.size() || vars_[var].record)
        return fail("netCDF: bad fixed-variable write");
    if (offset + nbytes > var_bytes(var)) return fail("netCDF: write past a variable's end");
    return pwrite_all(be, nbytes, data_offset(var, 0) + offset);
}

bool ClassicFile::write_record(int var, uint64_t rec, const void *be, size_t nbytes,
                               uint64_t offset) {
    if (!defined_ || var < 0 || var >= (int)vars_.size() || !vars_[var].record)
        return fail("netCDF: bad record-variable write");
    if (offset + nbytes > var_bytes(var)) return fail("netCDF: write past a record's end");
    return pwrite_all(be, nbytes, data_offset(var, rec) + offset);
}

bool ClassicFile::set_numrecs(uint64_t n) {
    std::lock_guard<std::mutex> lk(mu_);
    if (n <= numrecs_) return true;
    numrecs_ = n;
    std::vector<unsigned char> f;
    put_be(f, n, version_ == 5 ? 8 : 4);
    return pwrite_all(f.data(), f.size(), 4);
}

bool ClassicFile::close() {
    if (fd_ < 0) return error().empty();
    bool ok = error().empty();
    if (defined_) {
        std::lock_guard<std::mutex> lk(mu_);
        ok = write_header_locked() && ok;
    }
    if (::close(fd_) != 0) ok = fail(std::string("netCDF: close failed: ") + std::strerror(errno));
    fd_ = -1;
    return ok;
}

}  // namespace nc
}  // namespace swe
