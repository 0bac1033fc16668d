// NetCDF classic-format writer and reader (see xf_netcdf.h).
#include "xf_netcdf.h"

#include <cstring>

namespace xf {
namespace nc {

namespace {

constexpr uint32_t kDimTag = 0x0000000A;
constexpr uint32_t kVarTag = 0x0000000B;
constexpr uint32_t kAttTag = 0x0000000C;
constexpr uint32_t kDouble = 6;

void put32(std::vector<uint8_t>& b, uint32_t v)
{
    for (int i = 3; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
}

void put64(std::vector<uint8_t>& b, uint64_t v)
{
    for (int i = 7; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
}

void put_name(std::vector<uint8_t>& b, const std::string& s)
{
    put32(b, (uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    while (b.size() % 4) b.push_back(0);
}

void put_double_be(uint8_t* p, double v)
{
    uint64_t u;
    std::memcpy(&u, &v, 8);
    for (int i = 7; i >= 0; --i) *p++ = (uint8_t)(u >> (8 * i));
}

double get_double_be(const uint8_t* p)
{
    uint64_t u = 0;
    for (int i = 0; i < 8; ++i) u = (u << 8) | p[i];
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

uint64_t round4(uint64_t x) { return (x + 3) & ~uint64_t(3); }

void put_atts(std::vector<uint8_t>& b, const std::vector<Attr>& atts)
{
    if (atts.empty()) {
        put32(b, 0);
        put32(b, 0);
        return;
    }
    put32(b, kAttTag);
    put32(b, (uint32_t)atts.size());
    for (const auto& a : atts) {
        put_name(b, a.name);
        put32(b, kDouble);
        put32(b, (uint32_t)a.values.size());
        for (double v : a.values) {
            uint8_t t[8];
            put_double_be(t, v);
            b.insert(b.end(), t, t + 8);
        }
    }
}

std::vector<uint8_t> header(const std::vector<Dim>& dims, const std::vector<Var>& vars, int version, uint64_t numrecs)
{
    std::vector<uint8_t> b;
    b.push_back('C');
    b.push_back('D');
    b.push_back('F');
    b.push_back((uint8_t)version);
    put32(b, (uint32_t)numrecs);
    if (dims.empty()) {
        put32(b, 0);
        put32(b, 0);
    } else {
        put32(b, kDimTag);
        put32(b, (uint32_t)dims.size());
        for (const auto& d : dims) {
            put_name(b, d.name);
            put32(b, (uint32_t)d.len);
        }
    }
    put32(b, 0);  // no global attributes
    put32(b, 0);
    if (vars.empty()) {
        put32(b, 0);
        put32(b, 0);
    } else {
        put32(b, kVarTag);
        put32(b, (uint32_t)vars.size());
        for (const auto& v : vars) {
            put_name(b, v.name);
            put32(b, (uint32_t)v.dims.size());
            for (int d : v.dims) put32(b, (uint32_t)d);
            put_atts(b, v.atts);
            put32(b, kDouble);
            put32(b, v.vsize > 0xFFFFFFFCull ? 0xFFFFFFFFu : (uint32_t)v.vsize);
            if (version == 2) put64(b, v.begin);
            else put32(b, (uint32_t)v.begin);
        }
    }
    return b;
}

// vsize and record flags of every variable (the record dimension has length 0).
void layout(const std::vector<Dim>& dims, std::vector<Var>& vars, uint64_t& recsize)
{
    int nrec = 0;
    for (auto& v : vars) {
        uint64_t n = 8;
        v.record = !v.dims.empty() && dims[v.dims[0]].len == 0;
        for (size_t i = v.record ? 1 : 0; i < v.dims.size(); ++i) n *= dims[v.dims[i]].len;
        v.vsize = round4(n);
        if (v.record) ++nrec;
    }
    recsize = 0;
    for (auto& v : vars)
        if (v.record) recsize += v.vsize;
    // a single record variable is stored without padding between records
    if (nrec == 1)
        for (auto& v : vars)
            if (v.record) {
                uint64_t n = 8;
                for (size_t i = 1; i < v.dims.size(); ++i) n *= dims[v.dims[i]].len;
                recsize = n;
            }
}

}  // namespace

bool Writer::create(const std::string& path, const std::vector<Dim>& dims, const std::vector<Var>& vars, int version)
{
    close();
    dims_ = dims;
    vars_ = vars;
    layout(dims_, vars_, recsize_);
    const uint64_t hlen = header(dims_, vars_, version, 0).size();
    uint64_t off = round4(hlen);
    for (auto& v : vars_)
        if (!v.record) {
            v.begin = off;
            off += v.vsize;
        }
    rec_begin_ = off;
    for (auto& v : vars_)
        if (v.record) {
            v.begin = off;
            off += v.vsize;
        }
    if (version == 1 && off > 0x7FFFFFFFull) return false;
    f_ = std::fopen(path.c_str(), "wb+");
    if (!f_) return false;
    std::vector<uint8_t> h = header(dims_, vars_, version, 0);
    h.resize(round4(hlen), 0);
    if (std::fwrite(h.data(), 1, h.size(), f_) != h.size()) return false;
    // fixed-size variables are written as zeros (none are used by the snapshot files)
    std::vector<uint8_t> zero(4096, 0);
    for (const auto& v : vars_)
        if (!v.record)
            for (uint64_t done = 0; done < v.vsize; done += zero.size())
                std::fwrite(zero.data(), 1, (size_t)std::min<uint64_t>(zero.size(), v.vsize - done), f_);
    numrecs_ = 0;
    return true;
}

bool Writer::append(const std::vector<const double*>& data)
{
    return append(std::vector<const void*>(data.begin(), data.end()), std::vector<bool>(data.size(), false));
}

bool Writer::append(const std::vector<const void*>& data, const std::vector<bool>& be)
{
    if (!f_) return false;
    std::vector<uint8_t> buf;
    size_t k = 0;
    for (const auto& v : vars_) {
        if (!v.record) continue;
        if (k >= data.size()) return false;
        uint64_t n = 1;
        for (size_t i = 1; i < v.dims.size(); ++i) n *= dims_[v.dims[i]].len;
        const uint64_t off = v.begin + numrecs_ * recsize_;
        if (std::fseek(f_, (long)off, SEEK_SET) != 0) return false;
        // a lone record variable is not padded to 4 bytes in the record (the format's special case)
        const size_t len = (recsize_ < v.vsize) ? (size_t)recsize_ : (size_t)v.vsize;
        if (k < be.size() && be[k]) {
            // doubles are 8 bytes, so the slab has no padding: n * 8 == vsize
            if (std::fwrite(data[k], 1, len, f_) != len) return false;
        } else {
            buf.assign((size_t)v.vsize, 0);
            const double* d = static_cast<const double*>(data[k]);
            for (uint64_t i = 0; i < n; ++i) put_double_be(&buf[8 * i], d[i]);
            if (std::fwrite(buf.data(), 1, len, f_) != len) return false;
        }
        ++k;
    }
    ++numrecs_;
    uint8_t nr[4] = {(uint8_t)(numrecs_ >> 24), (uint8_t)(numrecs_ >> 16), (uint8_t)(numrecs_ >> 8), (uint8_t)numrecs_};
    if (std::fseek(f_, 4, SEEK_SET) != 0) return false;
    return std::fwrite(nr, 1, 4, f_) == 4;
}

bool Writer::sync() { return f_ && std::fflush(f_) == 0; }

void Writer::close()
{
    if (f_) std::fclose(f_);
    f_ = nullptr;
}

// ------------------------------------------------------------------ reader

namespace {

struct Cursor {
    const std::vector<uint8_t>& b;
    size_t p = 0;
    bool ok = true;
    uint32_t u32()
    {
        if (p + 4 > b.size()) {
            ok = false;
            return 0;
        }
        uint32_t v = ((uint32_t)b[p] << 24) | ((uint32_t)b[p + 1] << 16) | ((uint32_t)b[p + 2] << 8) | b[p + 3];
        p += 4;
        return v;
    }
    uint64_t u64()
    {
        uint64_t hi = u32();
        return (hi << 32) | u32();
    }
    std::string name()
    {
        const uint32_t n = u32();
        if (!ok || p + n > b.size()) {
            ok = false;
            return std::string();
        }
        std::string s((const char*)&b[p], n);
        p = round4(p + n);
        return s;
    }
};

}  // namespace

bool Reader::open(const std::string& path)
{
    close();
    f_ = std::fopen(path.c_str(), "rb");
    if (!f_) return false;
    // the header of these files is small: read the first 64 KiB
    std::vector<uint8_t> b(65536);
    b.resize(std::fread(b.data(), 1, b.size(), f_));
    if (b.size() < 8 || b[0] != 'C' || b[1] != 'D' || b[2] != 'F' || (b[3] != 1 && b[3] != 2)) return false;
    version_ = b[3];
    Cursor c{b, 4};
    numrecs_ = c.u32();
    dims_.clear();
    vars_.clear();
    uint32_t tag = c.u32(), n = c.u32();
    if (tag == kDimTag)
        for (uint32_t i = 0; i < n && c.ok; ++i) {
            Dim d;
            d.name = c.name();
            d.len = c.u32();
            dims_.push_back(d);
        }
    tag = c.u32();
    n = c.u32();
    if (tag == kAttTag) return false;  // global attributes are not written by this implementation
    tag = c.u32();
    n = c.u32();
    if (tag == kVarTag)
        for (uint32_t i = 0; i < n && c.ok; ++i) {
            Var v;
            v.name = c.name();
            const uint32_t nd = c.u32();
            for (uint32_t k = 0; k < nd; ++k) v.dims.push_back((int)c.u32());
            const uint32_t at = c.u32(), na = c.u32();
            if (at == kAttTag)
                for (uint32_t k = 0; k < na && c.ok; ++k) {
                    Attr a;
                    a.name = c.name();
                    const uint32_t ty = c.u32(), cnt = c.u32();
                    if (ty != kDouble) return false;
                    for (uint32_t j = 0; j < cnt; ++j) {
                        a.values.push_back(get_double_be(&b[c.p]));
                        c.p += 8;
                    }
                    v.atts.push_back(a);
                }
            if (c.u32() != kDouble) return false;
            v.vsize = c.u32();
            v.begin = version_ == 2 ? c.u64() : c.u32();
            vars_.push_back(v);
        }
    if (!c.ok) return false;
    for (const auto& v : vars_)
        for (int d : v.dims)
            if (d < 0 || d >= (int)dims_.size()) return false;
    std::vector<Var> tmp = vars_;
    layout(dims_, tmp, recsize_);
    for (size_t i = 0; i < vars_.size(); ++i) vars_[i].record = tmp[i].record;
    return true;
}

void Reader::close()
{
    if (f_) std::fclose(f_);
    f_ = nullptr;
}

int Reader::find_var(const std::string& name) const
{
    for (size_t i = 0; i < vars_.size(); ++i)
        if (vars_[i].name == name) return (int)i;
    return -1;
}

uint64_t Reader::count(int var) const
{
    const Var& v = vars_[var];
    uint64_t n = 1;
    for (size_t i = v.record ? 1 : 0; i < v.dims.size(); ++i) n *= dims_[v.dims[i]].len;
    return n;
}

bool Reader::read(int var, uint64_t rec, std::vector<double>& out)
{
    if (!f_ || var < 0 || var >= (int)vars_.size()) return false;
    const Var& v = vars_[var];
    if (v.record && rec >= numrecs_) return false;
    const uint64_t n = count(var);
    const uint64_t off = v.begin + (v.record ? rec * recsize_ : 0);
    std::vector<uint8_t> b((size_t)(8 * n));
    if (std::fseek(f_, (long)off, SEEK_SET) != 0) return false;
    if (std::fread(b.data(), 1, b.size(), f_) != b.size()) return false;
    out.resize((size_t)n);
    for (uint64_t i = 0; i < n; ++i) out[i] = get_double_be(&b[8 * i]);
    return true;
}

}  // namespace nc
}  // namespace xf
