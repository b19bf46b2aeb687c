// ESMF weight files: EsmfWeightIO::write_esmf / read_esmf
// (src/io/esmf_weight_io.cpp:66-183). The reference writes, through
// libnetcdf, one dimension num_wgts, variables S (double), col_idx and
// row_idx (int, 1-based) on it, and global int attributes n_a (source cells)
// and n_b (destination cells); it reads those back, whatever format
// libnetcdf opens.
//
// Here the file is written in the NetCDF-3 64-bit-offset format (CDF-2),
// from the published classic-format grammar: big-endian, a header of
// dimension, global attribute and variable lists (names and values padded
// to 4 bytes), then each fixed-size variable's data at its `begin` offset.
// libnetcdf opens such files, so the reference's read_esmf takes them.
// The reader takes CDF-1 and CDF-2 files, fixed-size or record (unlimited)
// num_wgts, and converts numeric variable types as nc_get_var_* does.
// NETCDF4 files (HDF5 containers, what the reference itself writes) and
// CDF-5 are refused with AXGB_ERR_UNSUPPORTED.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "internal.hpp"

namespace axgb {
namespace {

constexpr std::uint32_t kNcDimension = 0x0A, kNcVariable = 0x0B, kNcAttribute = 0x0C;
enum NcType { kByte = 1, kChar = 2, kShort = 3, kInt = 4, kFloat = 5, kDouble = 6 };

int type_size(int t) {
    switch (t) {
        case kByte:
        case kChar: return 1;
        case kShort: return 2;
        case kInt:
        case kFloat: return 4;
        case kDouble: return 8;
        default: return 0;
    }
}

inline std::size_t pad4(std::size_t n) { return (n + 3) & ~std::size_t(3); }

// ─── writer ────────────────────────────────────────────────────────────────
struct Out {
    std::vector<std::uint8_t> b;
    void u32(std::uint32_t v) {
        for (int s = 24; s >= 0; s -= 8) b.push_back(static_cast<std::uint8_t>(v >> s));
    }
    void u64(std::uint64_t v) {
        for (int s = 56; s >= 0; s -= 8) b.push_back(static_cast<std::uint8_t>(v >> s));
    }
    void name(const char *s) {
        const std::size_t n = std::strlen(s);
        u32(static_cast<std::uint32_t>(n));
        b.insert(b.end(), s, s + n);
        b.resize(b.size() + (pad4(n) - n), 0);
    }
};

struct FileCloser {
    void operator()(std::FILE *f) const {
        if (f) std::fclose(f);
    }
};
using File = std::unique_ptr<std::FILE, FileCloser>;

// ─── reader ────────────────────────────────────────────────────────────────
struct In {
    const std::uint8_t *p;
    std::size_t n, at = 0;
    int version;
    void need(std::size_t k) const {
        if (at + k > n || at + k < at) throw Error(AXGB_ERR_INVALID, "read_esmf: truncated NetCDF header");
    }
    std::uint32_t u32() {
        need(4);
        std::uint32_t v = 0;
        for (int i = 0; i < 4; ++i) v = (v << 8) | p[at++];
        return v;
    }
    std::uint64_t u64() {
        need(8);
        std::uint64_t v = 0;
        for (int i = 0; i < 8; ++i) v = (v << 8) | p[at++];
        return v;
    }
    std::uint64_t non_neg() {
        const std::uint32_t v = u32();
        if (v > 0x7fffffffu) throw Error(AXGB_ERR_INVALID, "read_esmf: negative count in NetCDF header");
        return v;
    }
    std::uint64_t offset() { return version == 1 ? u32() : u64(); }
    std::string name() {
        const std::uint64_t len = non_neg();
        need(pad4(len));
        std::string s(reinterpret_cast<const char *>(p + at), len);
        at += pad4(len);
        return s;
    }
    // list header: tag + count; ABSENT is two zero words
    std::uint64_t list(std::uint32_t tag) {
        const std::uint32_t t = u32();
        const std::uint64_t cnt = non_neg();
        if (t == 0 && cnt == 0) return 0;
        if (t != tag) throw Error(AXGB_ERR_INVALID, "read_esmf: malformed NetCDF header list");
        return cnt;
    }
};

struct NcAtt {
    std::string name;
    int type = 0;
    std::uint64_t count = 0;
    std::size_t value_at = 0;  // offset of the values in the header
};
struct NcVar {
    std::string name;
    std::vector<std::uint64_t> dims;
    int type = 0;
    std::uint64_t vsize = 0, begin = 0;
};

std::vector<NcAtt> read_atts(In &in) {
    std::vector<NcAtt> atts(in.list(kNcAttribute));
    for (auto &a : atts) {
        a.name = in.name();
        a.type = static_cast<int>(in.u32());
        a.count = in.non_neg();
        const int ts = type_size(a.type);
        if (!ts) throw Error(AXGB_ERR_INVALID, "read_esmf: unknown attribute type " + std::to_string(a.type));
        a.value_at = in.at;
        const std::uint64_t bytes = pad4(static_cast<std::size_t>(a.count) * ts);
        in.need(bytes);
        in.at += bytes;
    }
    return atts;
}

double get_num(const std::uint8_t *q, int type) {
    std::uint64_t v = 0;
    for (int i = 0; i < type_size(type); ++i) v = (v << 8) | q[i];
    switch (type) {
        case kByte: return static_cast<double>(static_cast<std::int8_t>(v));
        case kShort: return static_cast<double>(static_cast<std::int16_t>(v));
        case kInt: return static_cast<double>(static_cast<std::int32_t>(v));
        case kFloat: {
            const std::uint32_t u = static_cast<std::uint32_t>(v);
            float f;
            std::memcpy(&f, &u, 4);
            return f;
        }
        case kDouble: {
            double d;
            std::memcpy(&d, &v, 8);
            return d;
        }
        default: throw Error(AXGB_ERR_INVALID, "read_esmf: variable is not numeric");
    }
}

}  // namespace

void esmf_write(const std::string &path, std::int64_t n_a, std::int64_t n_b, std::int64_t nnz, const double *S,
                const std::int32_t *col1, const std::int32_t *row1) {
    AXGB_REQUIRE(nnz >= 0 && (nnz == 0 || (S && col1 && row1)), "write_esmf: NULL weight arrays");
    AXGB_REQUIRE(n_a >= 0 && n_a <= 0x7fffffff && n_b >= 0 && n_b <= 0x7fffffff,
                 "write_esmf: n_a / n_b do not fit the int attributes");
    // every variable's vsize must fit the format's 32-bit field
    AXGB_REQUIRE(nnz <= (std::int64_t(0xfffffffc) / 8), "write_esmf: more than 536,870,911 weights");
    Out h;
    h.b.insert(h.b.end(), {'C', 'D', 'F', 2});
    h.u32(0);  // numrecs (num_wgts is a record dimension only when it is empty)
    h.u32(kNcDimension);
    h.u32(1);
    h.name("num_wgts");
    h.u32(static_cast<std::uint32_t>(nnz));  // 0 makes it the unlimited dimension
    h.u32(kNcAttribute);
    h.u32(2);
    h.name("n_a");
    h.u32(kInt);
    h.u32(1);
    h.u32(static_cast<std::uint32_t>(n_a));
    h.name("n_b");
    h.u32(kInt);
    h.u32(1);
    h.u32(static_cast<std::uint32_t>(n_b));
    h.u32(kNcVariable);
    h.u32(3);
    const char *names[3] = {"S", "col_idx", "row_idx"};
    const int types[3] = {kDouble, kInt, kInt};
    std::size_t begin_at[3];
    const std::uint64_t n = static_cast<std::uint64_t>(nnz);
    for (int v = 0; v < 3; ++v) {
        h.name(names[v]);
        h.u32(1);  // rank
        h.u32(0);  // dimension id of num_wgts
        h.u32(0);  // no variable attributes (ABSENT)
        h.u32(0);
        h.u32(static_cast<std::uint32_t>(types[v]));
        // vsize: the whole variable, or one record's worth for a record variable
        h.u32(static_cast<std::uint32_t>(pad4((nnz ? n : 1) * type_size(types[v]))));
        begin_at[v] = h.b.size();
        h.u64(0);  // begin, patched below
    }
    std::uint64_t off = h.b.size();
    for (int v = 0; v < 3; ++v) {
        for (int s = 0; s < 8; ++s) h.b[begin_at[v] + s] = static_cast<std::uint8_t>(off >> (56 - 8 * s));
        off += nnz ? pad4(n * type_size(types[v])) : 0;
    }
    File f(std::fopen(path.c_str(), "wb"));
    if (!f) throw Error(AXGB_ERR_INVALID, "write_esmf: cannot open " + path + " for writing");
    auto put = [&](const void *p, std::size_t k) {
        if (k && std::fwrite(p, 1, k, f.get()) != k) throw Error(AXGB_ERR_INVALID, "write_esmf: write failed: " + path);
    };
    put(h.b.data(), h.b.size());
    std::vector<std::uint8_t> buf;
    const std::int64_t kChunk = 1 << 20;
    for (std::int64_t b0 = 0; b0 < nnz; b0 += kChunk) {  // S, big-endian
        const std::int64_t e = std::min(nnz, b0 + kChunk);
        buf.resize(8 * (e - b0));
        for (std::int64_t k = b0; k < e; ++k) {
            std::uint64_t u;
            std::memcpy(&u, S + k, 8);
            for (int s = 0; s < 8; ++s) buf[8 * (k - b0) + s] = static_cast<std::uint8_t>(u >> (56 - 8 * s));
        }
        put(buf.data(), buf.size());
    }
    for (const std::int32_t *a : {col1, row1})
        for (std::int64_t b0 = 0; b0 < nnz; b0 += kChunk) {
            const std::int64_t e = std::min(nnz, b0 + kChunk);
            buf.resize(4 * (e - b0));
            for (std::int64_t k = b0; k < e; ++k) {
                const std::uint32_t u = static_cast<std::uint32_t>(a[k]);
                for (int s = 0; s < 4; ++s) buf[4 * (k - b0) + s] = static_cast<std::uint8_t>(u >> (24 - 8 * s));
            }
            put(buf.data(), buf.size());
        }
    if (std::fflush(f.get()) != 0) throw Error(AXGB_ERR_INVALID, "write_esmf: write failed: " + path);
}

EsmfWeights esmf_read(const std::string &path) {
    File f(std::fopen(path.c_str(), "rb"));
    if (!f) throw Error(AXGB_ERR_INVALID, "read_esmf: cannot open " + path);
    std::vector<std::uint8_t> data;
    {
        std::uint8_t chunk[1 << 16];
        std::size_t k;
        while ((k = std::fread(chunk, 1, sizeof(chunk), f.get())) > 0) data.insert(data.end(), chunk, chunk + k);
    }
    static const std::uint8_t kHdf5[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (data.size() >= 8 && std::memcmp(data.data(), kHdf5, 8) == 0)
        throw Error(AXGB_ERR_UNSUPPORTED, "read_esmf: " + path + " is a NETCDF4 (HDF5) file; only NetCDF-3 classic "
                                          "and 64-bit-offset files are read here");
    AXGB_REQUIRE(data.size() >= 4 && data[0] == 'C' && data[1] == 'D' && data[2] == 'F',
                 "read_esmf: " + path + " is not a NetCDF file");
    if (data[3] == 5) throw Error(AXGB_ERR_UNSUPPORTED, "read_esmf: CDF-5 (64-bit data) files are not read here");
    AXGB_REQUIRE(data[3] == 1 || data[3] == 2, "read_esmf: unknown NetCDF format version");
    In in{data.data(), data.size()};
    in.at = 4;
    in.version = data[3];
    const std::uint32_t numrecs_raw = in.u32();
    const std::uint64_t numrecs = numrecs_raw == 0xffffffffu ? 0 : numrecs_raw;  // streaming: treat as empty
    std::vector<std::string> dim_name;
    std::vector<std::uint64_t> dim_len;
    const std::uint64_t nd = in.list(kNcDimension);
    for (std::uint64_t d = 0; d < nd; ++d) {
        dim_name.push_back(in.name());
        dim_len.push_back(in.non_neg());
    }
    const std::vector<NcAtt> gatts = read_atts(in);
    std::vector<NcVar> vars(in.list(kNcVariable));
    std::uint64_t recsize = 0;
    int n_rec_vars = 0;
    for (auto &v : vars) {
        v.name = in.name();
        v.dims.resize(in.non_neg());
        for (auto &d : v.dims) {
            d = in.non_neg();
            AXGB_REQUIRE(d < dim_len.size(), "read_esmf: variable refers to a missing dimension");
        }
        read_atts(in);
        v.type = static_cast<int>(in.u32());
        AXGB_REQUIRE(type_size(v.type) > 0, "read_esmf: unknown variable type");
        v.vsize = in.u32();
        v.begin = in.offset();
        if (!v.dims.empty() && dim_len[v.dims[0]] == 0) {
            recsize += v.vsize;
            ++n_rec_vars;
        }
    }
    auto att_int = [&](const char *name) -> std::int64_t {
        for (const auto &a : gatts)
            if (a.name == name) {
                AXGB_REQUIRE(a.count >= 1 && a.type != kChar, std::string("read_esmf: attribute ") + name + " is not numeric");
                return static_cast<std::int64_t>(get_num(data.data() + a.value_at, a.type));
            }
        throw Error(AXGB_ERR_INVALID, std::string("read_esmf: global attribute ") + name + " not found");
    };
    auto find = [&](const char *name) -> const NcVar & {
        for (const auto &v : vars)
            if (v.name == name) return v;
        throw Error(AXGB_ERR_INVALID, std::string("read_esmf: variable ") + name + " not found");
    };
    EsmfWeights w;
    w.n_a = att_int("n_a");
    w.n_b = att_int("n_b");
    const NcVar &vs = find("S"), &vc = find("col_idx"), &vr = find("row_idx");
    auto length = [&](const NcVar &v) -> std::uint64_t {
        AXGB_REQUIRE(v.dims.size() == 1, "read_esmf: " + v.name + " is not one-dimensional");
        const std::uint64_t len = dim_len[v.dims[0]];
        return len == 0 ? numrecs : len;
    };
    const std::uint64_t nnz = length(vs);
    AXGB_REQUIRE(length(vc) == nnz && length(vr) == nnz, "read_esmf: S, col_idx and row_idx differ in length");
    // element k of a variable: contiguous, or one per record (a lone record
    // variable's records are not padded)
    auto fetch = [&](const NcVar &v, std::uint64_t k) -> double {
        const int ts = type_size(v.type);
        const bool rec = dim_len[v.dims[0]] == 0;
        const std::uint64_t stride = rec ? (n_rec_vars == 1 ? static_cast<std::uint64_t>(ts) : recsize) : ts;
        const std::uint64_t at = v.begin + k * stride;
        AXGB_REQUIRE(at + ts <= data.size() && at >= v.begin, "read_esmf: variable data beyond the end of the file");
        return get_num(data.data() + at, v.type);
    };
    w.S.resize(nnz);
    w.col1.resize(nnz);
    w.row1.resize(nnz);
    for (std::uint64_t k = 0; k < nnz; ++k) {
        w.S[k] = fetch(vs, k);
        w.col1[k] = static_cast<std::int32_t>(fetch(vc, k));
        w.row1[k] = static_cast<std::int32_t>(fetch(vr, k));
    }
    return w;
}

}  // namespace axgb
