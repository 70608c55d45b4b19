// netCDF classic format (see ncfile.h): header layout per Unidata's
// published format specification; all integers and values big-endian,
// names and values padded to 4-byte boundaries.
#include "ncfile.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace ibm {
namespace {

constexpr uint32_t TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C;

int type_size(int t) { return t == NCT_CHAR ? 1 : t == NCT_DOUBLE ? 8 : 4; }

struct Out {
    std::vector<unsigned char> b;
    void u32(uint32_t v) {
        for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
    }
    void u64(uint64_t v) {
        for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
    }
    void pad() {
        while (b.size() % 4) b.push_back(0);
    }
    void name(const std::string &s) {
        u32((uint32_t)s.size());
        b.insert(b.end(), s.begin(), s.end());
        pad();
    }
};

// Element count of a variable.
long long nelems(const NcFile &f, const NcVar &v) {
    long long n = 1;
    for (int d : v.dims) n *= f.dims[d].second;
    return n;
}

long long vsize(const NcFile &f, const NcVar &v) {
    long long s = nelems(f, v) * type_size(v.type);
    return (s + 3) / 4 * 4;
}

// Header bytes for the given version (1: 32-bit offsets, 2: 64-bit) and
// the variables' begins.
std::vector<unsigned char> header(const NcFile &f, int version, const std::vector<long long> &begin) {
    Out o;
    o.b = {'C', 'D', 'F', (unsigned char)version};
    o.u32(0);  // numrecs: no record dimension
    if (f.dims.empty()) {
        o.u32(0);
        o.u32(0);
    } else {
        o.u32(TAG_DIM);
        o.u32((uint32_t)f.dims.size());
        for (auto &d : f.dims) {
            o.name(d.first);
            o.u32((uint32_t)d.second);
        }
    }
    o.u32(0);  // no global attributes
    o.u32(0);
    o.u32(TAG_VAR);
    o.u32((uint32_t)f.vars.size());
    for (size_t q = 0; q < f.vars.size(); q++) {
        const NcVar &v = f.vars[q];
        o.name(v.name);
        o.u32((uint32_t)v.dims.size());
        for (int d : v.dims) o.u32((uint32_t)d);
        if (v.atts.empty()) {
            o.u32(0);
            o.u32(0);
        } else {
            o.u32(TAG_ATT);
            o.u32((uint32_t)v.atts.size());
            for (auto &a : v.atts) {
                o.name(a.first);
                o.u32(NCT_CHAR);
                o.u32((uint32_t)a.second.size());
                o.b.insert(o.b.end(), a.second.begin(), a.second.end());
                o.pad();
            }
        }
        o.u32((uint32_t)v.type);
        const long long vs = vsize(f, v);
        o.u32((uint32_t)(vs > 0xFFFFFFFFll ? 0xFFFFFFFFu : vs));
        if (version == 1) o.u32((uint32_t)begin[q]);
        else o.u64((uint64_t)begin[q]);
    }
    return o.b;
}

// Writes n values of tsize bytes each from a little-endian host (x86-64
// and aarch64 both are), byte-swapped to big-endian.
void put_be(FILE *fp, const void *data, long long n, int tsize) {
    const unsigned char *p = (const unsigned char *)data;
    std::vector<unsigned char> buf;
    const long long chunk = 1 << 20;
    for (long long i = 0; i < n; i += chunk) {
        const long long m = std::min(chunk, n - i);
        buf.resize((size_t)(m * tsize));
        for (long long e = 0; e < m; e++)
            for (int c = 0; c < tsize; c++) buf[(size_t)(e * tsize + c)] = p[(i + e) * tsize + (tsize - 1 - c)];
        fwrite(buf.data(), 1, buf.size(), fp);
    }
}

uint32_t get_u32(const unsigned char *&p) {
    const uint32_t v = (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3];
    p += 4;
    return v;
}

uint64_t get_u64(const unsigned char *&p) {
    const uint64_t hi = get_u32(p);
    return hi << 32 | get_u32(p);
}

bool get_name(const unsigned char *&p, const unsigned char *end, std::string &s) {
    if (end - p < 4) return false;
    const uint32_t n = get_u32(p);
    const size_t padded = ((size_t)n + 3) / 4 * 4;
    if ((size_t)(end - p) < padded) return false;
    s.assign((const char *)p, n);
    p += padded;
    return true;
}

}  // namespace

bool nc_write(const std::string &path, const NcFile &f) {
    // The header size depends on the offset width: lay out with CDF-1
    // and switch to CDF-2 when an offset passes 2^31.
    int version = 1;
    std::vector<long long> begin(f.vars.size(), 0);
    for (;;) {
        long long off = (long long)header(f, version, begin).size();
        for (size_t q = 0; q < f.vars.size(); q++) {
            begin[q] = off;
            off += vsize(f, f.vars[q]);
        }
        if (version == 1 && !f.vars.empty() && begin.back() > 0x7FFFFFFFll) {
            version = 2;
            continue;
        }
        break;
    }
    const std::vector<unsigned char> h = header(f, version, begin);
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return false;
    bool ok = fwrite(h.data(), 1, h.size(), fp) == h.size();
    for (size_t q = 0; ok && q < f.vars.size(); q++) {
        const NcVar &v = f.vars[q];
        const long long n = nelems(f, v);
        put_be(fp, v.data, n, type_size(v.type));
        const long long padb = vsize(f, v) - n * type_size(v.type);
        for (long long e = 0; e < padb; e++) fputc(0, fp);
    }
    ok = ok && !ferror(fp);
    return fclose(fp) == 0 && ok;
}

bool nc_read_header(const std::string &path, NcFile &f) {
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return false;
    std::vector<unsigned char> b(1 << 16);
    const size_t got = fread(b.data(), 1, b.size(), fp);
    fclose(fp);
    b.resize(got);
    if (got < 16 || b[0] != 'C' || b[1] != 'D' || b[2] != 'F' || (b[3] != 1 && b[3] != 2)) return false;
    const int version = b[3];
    const unsigned char *p = b.data() + 4, *end = b.data() + got;
    f = NcFile();
    get_u32(p);  // numrecs
    uint32_t tag = get_u32(p), n = get_u32(p);
    if (tag == TAG_DIM)
        for (uint32_t q = 0; q < n; q++) {
            std::string s;
            if (!get_name(p, end, s) || end - p < 4) return false;
            f.dims.push_back({s, (long long)get_u32(p)});
        }
    if (end - p < 8) return false;
    tag = get_u32(p);
    n = get_u32(p);
    if (tag == TAG_ATT)  // global attributes: skipped
        for (uint32_t q = 0; q < n; q++) {
            std::string s;
            if (!get_name(p, end, s) || end - p < 8) return false;
            const int t = (int)get_u32(p);
            const uint32_t m = get_u32(p);
            const size_t len = ((size_t)m * type_size(t) + 3) / 4 * 4;
            if ((size_t)(end - p) < len) return false;
            p += len;
        }
    if (end - p < 8) return false;
    tag = get_u32(p);
    n = get_u32(p);
    if (tag != TAG_VAR) return n == 0;
    for (uint32_t q = 0; q < n; q++) {
        NcVar v;
        if (!get_name(p, end, v.name) || end - p < 4) return false;
        const uint32_t nd = get_u32(p);
        if ((size_t)(end - p) < (size_t)nd * 4 + 8) return false;
        for (uint32_t d = 0; d < nd; d++) {
            const uint32_t id = get_u32(p);
            if (id >= f.dims.size()) return false;
            v.dims.push_back((int)id);
        }
        tag = get_u32(p);
        const uint32_t na = get_u32(p);
        for (uint32_t a = 0; a < na && tag == TAG_ATT; a++) {
            std::string s;
            if (!get_name(p, end, s) || end - p < 8) return false;
            const int t = (int)get_u32(p);
            const uint32_t m = get_u32(p);
            const size_t len = ((size_t)m * type_size(t) + 3) / 4 * 4;
            if ((size_t)(end - p) < len) return false;
            std::string val;
            if (t == NCT_CHAR) val.assign((const char *)p, m);
            p += len;
            v.atts.push_back({s, val});
        }
        if (end - p < (version == 1 ? 12 : 16)) return false;
        v.type = (int)get_u32(p);
        get_u32(p);  // vsize
        v.begin = version == 1 ? (long long)get_u32(p) : (long long)get_u64(p);
        f.vars.push_back(v);
    }
    return true;
}

bool nc_read_var(const std::string &path, const NcFile &f, const std::string &name, std::vector<double> &out) {
    const NcVar *v = nullptr;
    for (auto &x : f.vars)
        if (x.name == name) v = &x;
    if (!v || (v->type != NCT_FLOAT && v->type != NCT_DOUBLE && v->type != NCT_INT)) return false;
    const long long n = nelems(f, *v);
    const int ts = type_size(v->type);
    std::vector<unsigned char> raw((size_t)(n * ts));
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return false;
    bool ok = fseeko(fp, (off_t)v->begin, SEEK_SET) == 0 && fread(raw.data(), 1, raw.size(), fp) == raw.size();
    fclose(fp);
    if (!ok) return false;
    out.resize((size_t)n);
    for (long long e = 0; e < n; e++) {
        unsigned char le[8];
        for (int c = 0; c < ts; c++) le[c] = raw[(size_t)(e * ts + ts - 1 - c)];
        if (v->type == NCT_FLOAT) {
            float x;
            memcpy(&x, le, 4);
            out[(size_t)e] = x;
        } else if (v->type == NCT_DOUBLE) {
            double x;
            memcpy(&x, le, 8);
            out[(size_t)e] = x;
        } else {
            int32_t x;
            memcpy(&x, le, 4);
            out[(size_t)e] = x;
        }
    }
    return true;
}

}  // namespace ibm
