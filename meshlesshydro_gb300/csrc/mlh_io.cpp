// Host-side input and output of the reference's run (include/mlh_io.h):
// config.info and parameter.h readers, and a minimal HDF5 reader and writer
// written from the HDF5 file-format specification (superblock versions 0/1,
// version-1 object headers, symbol-table groups, version-1 B-trees, local
// heaps, contiguous and compact dataset storage).
#include "../../include/mlh_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace mlh {
void set_last_error(const char *msg);
}

namespace {

int fail(int code, const std::string &msg) {
    mlh::set_last_error(msg.c_str());
    return code;
}

// ---------------------------------------------------------------- config.info

// One node of a Boost INFO tree: key -> value, key -> child block.
struct InfoNode {
    std::map<std::string, std::string> values;
    std::map<std::string, std::shared_ptr<InfoNode>> children;
};

// Tokens of the INFO syntax: words, quoted strings, '{', '}', and line ends;
// ';' starts a comment that runs to the end of the line.
std::vector<std::string> info_tokens(const std::string &text) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < text.size()) {
        char ch = text[i];
        if (ch == '\n') { out.push_back("\n"); ++i; continue; }
        if (std::isspace((unsigned char)ch)) { ++i; continue; }
        if (ch == ';') { while (i < text.size() && text[i] != '\n') ++i; continue; }
        if (ch == '{' || ch == '}') { out.push_back(std::string(1, ch)); ++i; continue; }
        if (ch == '"') {
            std::string s;
            ++i;
            while (i < text.size() && text[i] != '"') {
                if (text[i] == '\\' && i + 1 < text.size()) ++i;
                s += text[i++];
            }
            ++i;
            out.push_back("\"" + s);   // marked as a quoted word
            continue;
        }
        std::string s;
        while (i < text.size() && !std::isspace((unsigned char)text[i]) && text[i] != ';' && text[i] != '{' &&
               text[i] != '}')
            s += text[i++];
        out.push_back(s);
    }
    return out;
}

std::string unquote(const std::string &t) { return (!t.empty() && t[0] == '"') ? t.substr(1) : t; }

// key [value] [{ ... }] per line; a '{' may also open on the next line.
bool info_parse(const std::vector<std::string> &tok, size_t &p, InfoNode &node, int depth, std::string &err) {
    while (p < tok.size()) {
        if (tok[p] == "\n") { ++p; continue; }
        if (tok[p] == "}") {
            if (depth == 0) { err = "unbalanced '}'"; return false; }
            ++p;
            return true;
        }
        if (tok[p] == "{") { err = "'{' without a key"; return false; }
        const std::string key = unquote(tok[p++]);
        std::string value;
        if (p < tok.size() && tok[p] != "\n" && tok[p] != "{" && tok[p] != "}") value = unquote(tok[p++]);
        size_t q = p;
        while (q < tok.size() && tok[q] == "\n") ++q;
        if (q < tok.size() && tok[q] == "{") {
            p = q + 1;
            auto child = std::make_shared<InfoNode>();
            if (!info_parse(tok, p, *child, depth + 1, err)) return false;
            node.children[key] = child;
            if (!value.empty()) node.values[key] = value;
        } else {
            node.values[key] = value;
        }
    }
    if (depth != 0) { err = "missing '}'"; return false; }
    return true;
}

bool to_double(const std::string &s, double &v) {
    if (s.empty()) return false;
    char *end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

bool to_int(const std::string &s, int &v) {
    double d;
    if (!to_double(s, d) || d != std::floor(d) || std::fabs(d) > 2147483647.) return false;
    v = (int)d;
    return true;
}

void copy_str(char *dst, size_t cap, const std::string &s) {
    std::snprintf(dst, cap, "%s", s.c_str());
}

// ---------------------------------------------------------------- HDF5 bytes

constexpr uint64_t UNDEF = ~0ull;
const unsigned char H5_SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

struct Reader {
    std::ifstream f;
    uint64_t size = 0, base = 0;
    int so = 8, sl = 8;   // sizes of offsets and lengths
    std::string err;

    bool open(const char *path) {
        f.open(path, std::ios::binary);
        if (!f) { err = std::string("cannot open ") + path; return false; }
        f.seekg(0, std::ios::end);
        size = (uint64_t)f.tellg();
        return true;
    }
    bool read(uint64_t off, size_t n, std::vector<unsigned char> &out) {
        if (off > size || n > size - off) { err = "read beyond the end of the file"; return false; }
        out.resize(n);
        f.seekg((std::streamoff)off);
        f.read((char *)out.data(), (std::streamsize)n);
        if (!f) { err = "read error"; return false; }
        return true;
    }
    static uint64_t le(const unsigned char *p, int n) {
        uint64_t v = 0;
        for (int k = n - 1; k >= 0; --k) v = (v << 8) | p[k];
        return v;
    }
    uint64_t addr(const unsigned char *p) const {
        uint64_t v = le(p, so);
        if (so < 8 && v == ((1ull << (8 * so)) - 1)) return UNDEF;
        if (v == UNDEF) return UNDEF;
        return v + base;
    }
};

struct Message {
    unsigned type;
    std::vector<unsigned char> data;
};

// Messages of a version-1 object header, following continuation messages.
bool object_header(Reader &r, uint64_t addr, std::vector<Message> &msgs) {
    std::vector<unsigned char> pre;
    if (!r.read(addr, 16, pre)) return false;
    if (std::memcmp(pre.data(), "OHDR", 4) == 0) {
        r.err = "version-2 object headers are not supported (file written with libver 'latest')";
        return false;
    }
    if (pre[0] != 1) { r.err = "unknown object header version"; return false; }
    const unsigned nmsgs = (unsigned)Reader::le(&pre[2], 2);
    const uint64_t hsize = Reader::le(&pre[8], 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks = {{addr + 16, hsize}};
    unsigned seen = 0;
    for (size_t b = 0; b < blocks.size() && seen < nmsgs; ++b) {
        std::vector<unsigned char> blk;
        if (!r.read(blocks[b].first, (size_t)blocks[b].second, blk)) return false;
        size_t p = 0;
        while (p + 8 <= blk.size() && seen < nmsgs) {
            const unsigned type = (unsigned)Reader::le(&blk[p], 2);
            const size_t sz = (size_t)Reader::le(&blk[p + 2], 2);
            if (p + 8 + sz > blk.size()) { r.err = "object header message runs past its block"; return false; }
            Message m;
            m.type = type;
            m.data.assign(blk.begin() + p + 8, blk.begin() + p + 8 + sz);
            ++seen;
            if (type == 0x10) {   // continuation: address + length of the next block
                if (sz < (size_t)(r.so + r.sl)) { r.err = "short continuation message"; return false; }
                blocks.push_back({r.addr(m.data.data()), Reader::le(m.data.data() + r.so, r.sl)});
            } else {
                msgs.push_back(std::move(m));
            }
            p += 8 + sz;
        }
    }
    return true;
}

struct Superblock {
    uint64_t root_oh = UNDEF, btree = UNDEF, heap = UNDEF;
};

bool superblock(Reader &r, Superblock &sb) {
    std::vector<unsigned char> b;
    uint64_t at = 0;
    for (;; at = at ? at * 2 : 512) {   // the signature may follow a user block
        if (at + 8 > r.size) { r.err = "not an HDF5 file"; return false; }
        if (!r.read(at, 8, b)) return false;
        if (std::memcmp(b.data(), H5_SIG, 8) == 0) break;
    }
    if (!r.read(at, std::min<uint64_t>(r.size - at, 128), b)) return false;
    const int ver = b[8];
    if (ver > 1) {
        r.err = "superblock version " + std::to_string(ver) + " is not supported (file written with libver 'latest')";
        return false;
    }
    r.so = b[13];
    r.sl = b[14];
    if ((r.so != 4 && r.so != 8) || (r.sl != 4 && r.sl != 8)) { r.err = "unsupported offset/length size"; return false; }
    size_t p = 24 + (ver == 1 ? 4 : 0);
    r.base = Reader::le(&b[p], r.so);
    p += 4 * r.so;   // base, free space, end of file, driver info
    if (p + 2 * r.so + 24 > b.size()) { r.err = "truncated superblock"; return false; }
    sb.root_oh = r.addr(&b[p + r.so]);
    const uint32_t cache = (uint32_t)Reader::le(&b[p + 2 * r.so], 4);
    if (cache == 1) {
        sb.btree = r.addr(&b[p + 2 * r.so + 8]);
        sb.heap = r.addr(&b[p + 2 * r.so + 8 + r.so]);
    }
    return true;
}

// name -> object header address of every link in the root group
bool root_links(Reader &r, std::map<std::string, uint64_t> &links) {
    Superblock sb;
    if (!superblock(r, sb)) return false;
    std::vector<Message> msgs;
    if (!object_header(r, sb.root_oh, msgs)) return false;
    uint64_t btree = UNDEF, heap = UNDEF;
    for (const Message &m : msgs) {
        if (m.type == 0x11 && m.data.size() >= (size_t)(2 * r.so)) {
            btree = r.addr(m.data.data());
            heap = r.addr(m.data.data() + r.so);
        } else if (m.type == 0x06) {   // link message (compact new-style group)
            const unsigned char *d = m.data.data();
            size_t p = 2;
            const unsigned fl = d[1];
            unsigned ltype = 0;
            if (fl & 0x08) ltype = d[p++];
            if (fl & 0x04) p += 8;
            if (fl & 0x10) p += 1;
            const int lsz = 1 << (fl & 3);
            const size_t nlen = (size_t)Reader::le(d + p, lsz);
            p += lsz;
            if (p + nlen > m.data.size()) continue;
            std::string name((const char *)d + p, nlen);
            p += nlen;
            if (ltype == 0 && p + r.so <= m.data.size()) links[name] = r.addr(d + p);
        }
    }
    if (btree == UNDEF) {
        if (!links.empty()) return true;
        r.err = "root group without a symbol table";
        return false;
    }
    std::vector<unsigned char> hh;
    if (!r.read(heap, 8 + 2 * r.sl + r.so, hh)) return false;
    if (std::memcmp(hh.data(), "HEAP", 4) != 0) { r.err = "bad local heap"; return false; }
    const uint64_t hsize = Reader::le(&hh[8], r.sl);
    const uint64_t hdata = r.addr(&hh[8 + 2 * r.sl]);
    std::vector<unsigned char> names;
    if (!r.read(hdata, (size_t)hsize, names)) return false;
    // depth-first walk of the group B-tree
    std::vector<std::pair<uint64_t, int>> stack = {{btree, 64}};
    while (!stack.empty()) {
        const uint64_t a = stack.back().first;
        const int budget = stack.back().second;
        stack.pop_back();
        if (budget <= 0) { r.err = "group B-tree too deep"; return false; }
        std::vector<unsigned char> hd;
        if (!r.read(a, 8 + 2 * r.so, hd)) return false;
        if (std::memcmp(hd.data(), "TREE", 4) != 0 || hd[4] != 0) { r.err = "bad group B-tree node"; return false; }
        const int level = hd[5];
        const unsigned used = (unsigned)Reader::le(&hd[6], 2);
        std::vector<unsigned char> kc;
        if (!r.read(a + 8 + 2 * r.so, (size_t)used * (r.sl + r.so) + r.sl, kc)) return false;
        for (unsigned k = 0; k < used; ++k) {
            const uint64_t child = r.addr(&kc[(size_t)k * (r.sl + r.so) + r.sl]);
            if (level > 0) { stack.push_back({child, budget - 1}); continue; }
            std::vector<unsigned char> sn;
            if (!r.read(child, 8, sn)) return false;
            if (std::memcmp(sn.data(), "SNOD", 4) != 0) { r.err = "bad symbol table node"; return false; }
            const unsigned nsym = (unsigned)Reader::le(&sn[6], 2);
            const size_t esz = 2 * r.so + 24;
            std::vector<unsigned char> ent;
            if (!r.read(child + 8, nsym * esz, ent)) return false;
            for (unsigned e = 0; e < nsym; ++e) {
                const uint64_t noff = Reader::le(&ent[e * esz], r.so);
                const uint64_t oh = r.addr(&ent[e * esz + r.so]);
                if (noff >= names.size()) { r.err = "bad link name offset"; return false; }
                const char *nm = (const char *)names.data() + noff;
                links[std::string(nm, strnlen(nm, names.size() - noff))] = oh;
            }
        }
    }
    return true;
}

struct DatasetInfo {
    int rank = 0;
    uint64_t dims[2] = {0, 0};
    int cls = -1;          // 0 float, 1 integer
    int size = 0;
    bool big_endian = false, is_signed = true;
    int layout = -1;       // 0 compact, 1 contiguous
    uint64_t addr = UNDEF, nbytes = 0;
    std::vector<unsigned char> compact;
};

bool dataset(Reader &r, const char *file, const char *name, DatasetInfo &di) {
    if (!r.open(file)) return false;
    std::map<std::string, uint64_t> links;
    if (!root_links(r, links)) return false;
    std::string nm = name;
    if (!nm.empty() && nm[0] == '/') nm = nm.substr(1);
    if (nm.find('/') != std::string::npos) { r.err = "only datasets of the root group are supported"; return false; }
    auto it = links.find(nm);
    if (it == links.end()) { r.err = "no dataset /" + nm; return false; }
    std::vector<Message> msgs;
    if (!object_header(r, it->second, msgs)) return false;
    bool space = false, type = false;
    for (const Message &m : msgs) {
        const unsigned char *d = m.data.data();
        if (m.type == 0x01) {
            const int ver = d[0];
            di.rank = d[1];
            if (di.rank < 1 || di.rank > 2) { r.err = "/" + nm + ": rank " + std::to_string(di.rank) + " not supported"; return false; }
            const size_t p = ver == 1 ? 8 : 4;
            for (int k = 0; k < di.rank; ++k) di.dims[k] = Reader::le(d + p + (size_t)k * r.sl, r.sl);
            space = true;
        } else if (m.type == 0x03) {
            const int cls = d[0] & 0x0f;
            di.size = (int)Reader::le(d + 4, 4);
            if (cls == 0) {
                di.cls = 1;
                di.big_endian = d[1] & 1;
                di.is_signed = (d[1] >> 3) & 1;
                if (di.size != 1 && di.size != 2 && di.size != 4 && di.size != 8) { r.err = "integer size"; return false; }
            } else if (cls == 1) {
                di.cls = 0;
                if (d[1] & 0x40) { r.err = "VAX floating point is not supported"; return false; }
                di.big_endian = d[1] & 1;
                if (di.size != 4 && di.size != 8) { r.err = "floating-point size"; return false; }
            } else {
                r.err = "/" + nm + ": datatype class " + std::to_string(cls) + " is not supported";
                return false;
            }
            type = true;
        } else if (m.type == 0x0b) {
            r.err = "/" + nm + ": filtered (compressed) datasets are not supported";
            return false;
        } else if (m.type == 0x08) {
            const int ver = d[0];
            if (ver >= 3) {
                di.layout = d[1];
                if (di.layout == 0) {
                    const size_t n = (size_t)Reader::le(d + 2, 2);
                    di.compact.assign(d + 4, d + 4 + std::min(n, m.data.size() - 4));
                } else if (di.layout == 1) {
                    di.addr = r.addr(d + 2);
                    di.nbytes = Reader::le(d + 2 + r.so, r.sl);
                } else {
                    r.err = "/" + nm + ": chunked or virtual storage is not supported";
                    return false;
                }
            } else {   // versions 1 and 2
                const int ndims = d[1];
                di.layout = d[2];
                if (di.layout == 1) {
                    di.addr = r.addr(d + 8);
                    di.nbytes = UNDEF;
                } else if (di.layout == 0) {
                    const size_t p = 8 + (size_t)ndims * 4;
                    const size_t n = (size_t)Reader::le(d + p, 4);
                    di.compact.assign(d + p + 4, d + p + 4 + n);
                } else {
                    r.err = "/" + nm + ": chunked storage is not supported";
                    return false;
                }
            }
        }
    }
    if (!space || !type || di.layout < 0) { r.err = "/" + nm + ": incomplete dataset header"; return false; }
    return true;
}

uint64_t elements(const DatasetInfo &di) { return di.rank == 1 ? di.dims[0] : di.dims[0] * di.dims[1]; }

template <class T>
bool read_as(const char *file, const char *name, T *out, long long count) {
    Reader r;
    DatasetInfo di;
    if (!dataset(r, file, name, di)) { mlh::set_last_error(r.err.c_str()); return false; }
    const uint64_t n = elements(di);
    if ((long long)n != count) {
        mlh::set_last_error((std::string(name) + ": element count mismatch").c_str());
        return false;
    }
    const uint64_t bytes = n * (uint64_t)di.size;
    std::vector<unsigned char> raw;
    if (di.layout == 0) {
        if (di.compact.size() < bytes) { mlh::set_last_error("short compact dataset"); return false; }
        raw.assign(di.compact.begin(), di.compact.begin() + bytes);
    } else if (di.addr == UNDEF) {
        raw.assign(bytes, 0);   // never written: the default fill value
    } else if (!r.read(di.addr, (size_t)bytes, raw)) {
        mlh::set_last_error(r.err.c_str());
        return false;
    }
    for (uint64_t k = 0; k < n; ++k) {
        unsigned char e[8];
        for (int b = 0; b < di.size; ++b) e[b] = raw[k * di.size + (di.big_endian ? di.size - 1 - b : b)];
        double v;
        if (di.cls == 0) {
            if (di.size == 8) { double d; std::memcpy(&d, e, 8); v = d; }
            else { float f; std::memcpy(&f, e, 4); v = f; }
            out[k] = (T)v;
        } else {
            uint64_t u = Reader::le(e, di.size);
            if (di.is_signed && di.size < 8 && (u >> (8 * di.size - 1)) & 1) u |= ~0ull << (8 * di.size);
            out[k] = di.is_signed ? (T)(int64_t)u : (T)u;
        }
    }
    return true;
}

}  // namespace

// ---------------------------------------------------------------- writer

struct mlh_h5_writer {
    struct Set {
        std::string name;
        int rank;
        uint64_t dims[2];
        bool is_float;
        std::vector<unsigned char> data;
    };
    std::string path;
    std::vector<Set> sets;
};

namespace {

struct Out {
    std::vector<unsigned char> b;
    void u8(unsigned v) { b.push_back((unsigned char)v); }
    void le(uint64_t v, int n) { for (int k = 0; k < n; ++k) b.push_back((unsigned char)(v >> (8 * k))); }
    void bytes(const void *p, size_t n) { b.insert(b.end(), (const unsigned char *)p, (const unsigned char *)p + n); }
    void pad8() { while (b.size() % 8) b.push_back(0); }
    void at(size_t off, uint64_t v, int n) { for (int k = 0; k < n; ++k) b[off + k] = (unsigned char)(v >> (8 * k)); }
    size_t size() const { return b.size(); }
};

constexpr int LEAF_K = 16;       // symbol table nodes hold up to 2K links
constexpr int INTERNAL_K = 16;   // group B-tree nodes hold up to 2K children
constexpr size_t BTREE_BYTES = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8;
constexpr size_t SNOD_BYTES = 8 + 2 * LEAF_K * 40;

// header of one message of a version-1 object header (8-byte aligned data)
void msg_header(Out &o, unsigned type, size_t size, unsigned flags) {
    o.le(type, 2);
    o.le(size, 2);
    o.u8(flags);
    o.le(0, 3);
}

std::vector<unsigned char> dataset_header(const mlh_h5_writer::Set &s, uint64_t data_addr) {
    Out o;
    const size_t space_sz = 8 + 8 * (size_t)s.rank;
    const size_t type_sz = s.is_float ? 24 : 16;
    const size_t fill_sz = 8, layout_sz = 24;
    const size_t total = 4 * 8 + space_sz + type_sz + fill_sz + layout_sz;
    o.u8(1); o.u8(0); o.le(4, 2); o.le(1, 4); o.le(total, 4); o.le(0, 4);
    // dataspace, version 1
    msg_header(o, 0x0001, space_sz, 0);
    o.u8(1); o.u8((unsigned)s.rank); o.u8(0); o.u8(0); o.le(0, 4);
    for (int k = 0; k < s.rank; ++k) o.le(s.dims[k], 8);
    // datatype, version 1 (constant message)
    msg_header(o, 0x0003, type_sz, 1);
    if (s.is_float) {
        // IEEE binary64, little endian: sign bit 63, exponent 52..62 (bias
        // 1023), mantissa 0..51 with an implied leading one
        o.u8(0x11); o.u8(0x20); o.u8(63); o.u8(0); o.le(8, 4);
        o.le(0, 2); o.le(64, 2); o.u8(52); o.u8(11); o.u8(0); o.u8(52); o.le(1023, 4);
        o.le(0, 4);
    } else {
        // signed 32-bit two's complement, little endian
        o.u8(0x10); o.u8(0x08); o.u8(0); o.u8(0); o.le(4, 4);
        o.le(0, 2); o.le(32, 2);
        o.le(0, 4);
    }
    // fill value, version 2: late allocation, written if set, undefined
    msg_header(o, 0x0005, fill_sz, 1);
    o.u8(2); o.u8(2); o.u8(2); o.u8(0); o.le(0, 4);
    // data layout, version 3: contiguous
    msg_header(o, 0x0008, layout_sz, 0);
    o.u8(3); o.u8(1); o.le(data_addr, 8); o.le(s.data.size(), 8); o.le(0, 6);
    return o.b;
}

int write_file(mlh_h5_writer *w) {
    std::vector<mlh_h5_writer::Set> &sets = w->sets;
    std::sort(sets.begin(), sets.end(), [](const mlh_h5_writer::Set &a, const mlh_h5_writer::Set &b) {
        return std::strcmp(a.name.c_str(), b.name.c_str()) < 0;
    });
    for (size_t k = 1; k < sets.size(); ++k)
        if (sets[k].name == sets[k - 1].name) return fail(MLH_ERR_INVALID, "duplicate dataset /" + sets[k].name);
    if (sets.size() > (size_t)(2 * LEAF_K)) return fail(MLH_ERR_CAPACITY, "at most 32 datasets per file");
    // local heap data: "" at offset 0, then the names, each padded to 8 bytes
    std::vector<uint64_t> name_off;
    Out heap;
    heap.le(0, 8);
    for (const auto &s : sets) {
        name_off.push_back(heap.size());
        heap.bytes(s.name.c_str(), s.name.size() + 1);
        heap.pad8();
    }
    const uint64_t sb_at = 0, root_at = 96, heap_at = root_at + 40, heapdata_at = heap_at + 32;
    const uint64_t btree_at = heapdata_at + heap.size();
    const uint64_t snod_at = btree_at + BTREE_BYTES;
    uint64_t at = snod_at + SNOD_BYTES;
    std::vector<uint64_t> oh_at, data_at;
    std::vector<std::vector<unsigned char>> headers;
    for (const auto &s : sets) {
        oh_at.push_back(at);
        const size_t hsz = dataset_header(s, 0).size();
        data_at.push_back((at + hsz + 7) / 8 * 8);
        headers.push_back(dataset_header(s, data_at.back()));
        at = (data_at.back() + s.data.size() + 7) / 8 * 8;
    }
    const uint64_t eof = at;
    Out o;
    // superblock version 0 (8-byte offsets and lengths)
    o.bytes(H5_SIG, 8);
    o.u8(0); o.u8(0); o.u8(0); o.u8(0); o.u8(0); o.u8(8); o.u8(8); o.u8(0);
    o.le(LEAF_K, 2); o.le(INTERNAL_K, 2); o.le(0, 4);
    o.le(0, 8); o.le(UNDEF, 8); o.le(eof, 8); o.le(UNDEF, 8);
    // root group symbol table entry (cache type 1: B-tree and heap)
    o.le(0, 8); o.le(root_at, 8); o.le(1, 4); o.le(0, 4); o.le(btree_at, 8); o.le(heap_at, 8);
    (void)sb_at;
    // root object header: one symbol table message
    o.u8(1); o.u8(0); o.le(1, 2); o.le(1, 4); o.le(24, 4); o.le(0, 4);
    msg_header(o, 0x0011, 16, 0);
    o.le(btree_at, 8); o.le(heap_at, 8);
    // local heap (no free block: offset 1 ends the free list)
    o.bytes("HEAP", 4); o.u8(0); o.le(0, 3); o.le(heap.size(), 8); o.le(1, 8); o.le(heapdata_at, 8);
    o.bytes(heap.b.data(), heap.size());
    // group B-tree: one leaf with one symbol table node
    const size_t bt = o.size();
    o.bytes("TREE", 4); o.u8(0); o.u8(0); o.le(sets.empty() ? 0 : 1, 2); o.le(UNDEF, 8); o.le(UNDEF, 8);
    o.le(0, 8); o.le(snod_at, 8); o.le(sets.empty() ? 0 : name_off.back(), 8);
    while (o.size() < bt + BTREE_BYTES) o.u8(0);
    // symbol table node, links sorted by name
    const size_t sn = o.size();
    o.bytes("SNOD", 4); o.u8(1); o.u8(0); o.le(sets.size(), 2);
    for (size_t k = 0; k < sets.size(); ++k) { o.le(name_off[k], 8); o.le(oh_at[k], 8); o.le(0, 4); o.le(0, 4); o.le(0, 16); }
    while (o.size() < sn + SNOD_BYTES) o.u8(0);
    for (size_t k = 0; k < sets.size(); ++k) {
        while (o.size() < oh_at[k]) o.u8(0);
        o.bytes(headers[k].data(), headers[k].size());
        while (o.size() < data_at[k]) o.u8(0);
        o.bytes(sets[k].data.data(), sets[k].data.size());
    }
    while (o.size() < eof) o.u8(0);
    std::ofstream f(w->path, std::ios::binary | std::ios::trunc);
    if (!f) return fail(MLH_ERR_INVALID, "cannot create " + w->path);
    f.write((const char *)o.b.data(), (std::streamsize)o.size());
    if (!f) return fail(MLH_ERR_INVALID, "write error on " + w->path);
    return 0;
}

template <class T>
int add_set(mlh_h5_writer *w, const char *name, int rank, const long long *dims, const T *data, bool is_float) {
    if (!w || !name || !dims || rank < 1 || rank > 2) return fail(MLH_ERR_INVALID, "invalid dataset");
    std::string nm = name;
    if (!nm.empty() && nm[0] == '/') nm = nm.substr(1);
    if (nm.empty() || nm.find('/') != std::string::npos) return fail(MLH_ERR_INVALID, "datasets live in the root group");
    mlh_h5_writer::Set s;
    s.name = nm;
    s.rank = rank;
    uint64_t n = 1;
    for (int k = 0; k < rank; ++k) {
        if (dims[k] < 0) return fail(MLH_ERR_INVALID, "negative dimension");
        s.dims[k] = (uint64_t)dims[k];
        n *= s.dims[k];
    }
    if (n > 0 && !data) return fail(MLH_ERR_INVALID, "no data");
    s.is_float = is_float;
    s.data.resize(n * sizeof(T));
    // the host is little endian (x86-64 and aarch64), as the file
    if (n) std::memcpy(s.data.data(), data, n * sizeof(T));
    w->sets.push_back(std::move(s));
    return 0;
}

}  // namespace

extern "C" {

void mlh_default_run_config(mlh_run_config *run) {
    std::memset(run, 0, sizeof(*run));
    mlh_config &c = run->cfg;
    c.dim = 2;
    c.periodic = 1;
    c.adaptive_timestep = 1;
    c.slope_limiting = 1;
    c.pairwise_limiter = 1;
    c.meshless_finite_mass = 0;
    c.move_particles = 1;
    c.first_order_quad_point = 1;
    c.riemann_max_iter = 100;
    c.kernel_size = .025;
    c.gamma = 5. / 3.;
    c.cfl = .2;
    c.time_step = .005;
    c.beta = 4.;
    c.psi1 = .5;
    c.psi2 = .25;
    c.riemann_tol = 1e-10;
    c.box_hi[0] = 1.;
    c.box_hi[1] = 1.;
    run->time_end = 1.;
    run->h5_dump_interval = 10;
    run->debug_lvl = 1;
    copy_str(run->out_dir, sizeof(run->out_dir), "output");
}

int mlh_read_parameter_header(const char *path, mlh_run_config *run) {
    if (!path || !run) return fail(MLH_ERR_INVALID, "null argument");
    std::ifstream f(path);
    if (!f) return fail(MLH_ERR_INVALID, std::string("cannot open ") + path);
    std::map<std::string, std::string> defs;
    std::string line;
    bool in_comment = false;
    while (std::getline(f, line)) {
        // drop /* */ and // comments
        std::string s;
        for (size_t i = 0; i < line.size(); ++i) {
            if (in_comment) {
                if (line.compare(i, 2, "*/") == 0) { in_comment = false; ++i; }
                continue;
            }
            if (line.compare(i, 2, "/*") == 0) { in_comment = true; ++i; continue; }
            if (line.compare(i, 2, "//") == 0) break;
            s += line[i];
        }
        std::istringstream is(s);
        std::string hash, name, value;
        is >> hash;
        if (hash == "#") is >> hash, hash = "#" + hash;
        if (hash != "#define") continue;
        is >> name;
        std::getline(is, value);
        value.erase(0, value.find_first_not_of(" \t"));
        value.erase(value.find_last_not_of(" \t\r") + 1);
        defs[name] = value;
    }
    auto num = [&](const char *k, double &v) -> int {
        auto it = defs.find(k);
        if (it == defs.end()) return 0;
        if (!to_double(it->second, v)) return fail(MLH_ERR_INVALID, std::string(k) + ": not a number: " + it->second);
        return 0;
    };
    // a switch: an undefined macro reads as 0 in #if; an empty one is an
    // error there, as it is here
    auto flag = [&](const char *k, int &v) -> int {
        double d = 0.;
        auto it = defs.find(k);
        if (it != defs.end() && !to_double(it->second, d))
            return fail(MLH_ERR_INVALID, std::string(k) + ": not a number: '" + it->second + "'");
        v = d != 0.;
        return 0;
    };
    mlh_config &c = run->cfg;
    double d;
    int rc = 0;
    d = c.dim;
    if ((rc = num("DIM", d))) return rc;
    if (d != 2. && d != 3.) return fail(MLH_ERR_INVALID, "DIM must be 2 or 3");
    c.dim = (int)d;
    if ((rc = flag("PERIODIC_BOUNDARIES", c.periodic))) return rc;
    if ((rc = flag("ADAPTIVE_TIMESTEP", c.adaptive_timestep))) return rc;
    if ((rc = flag("SLOPE_LIMITING", c.slope_limiting))) return rc;
    if ((rc = flag("PAIRWISE_LIMITER", c.pairwise_limiter))) return rc;
    if ((rc = flag("MESHLESS_FINITE_MASS", c.meshless_finite_mass))) return rc;
    if ((rc = flag("MOVE_PARTICLES", c.move_particles))) return rc;
    if ((rc = flag("FIRST_ORDER_QUAD_POINT", c.first_order_quad_point))) return rc;
    if ((rc = num("CFL", c.cfl))) return rc;
    if ((rc = num("BETA", c.beta))) return rc;
    if ((rc = num("PSI_1", c.psi1))) return rc;
    if ((rc = num("PSI_2", c.psi2))) return rc;
    d = 0.;
    if ((rc = num("MAX_NUM_INTERACTIONS", d))) return rc;
    if (d > 0.) c.max_neighbours = (int)d;
    d = run->debug_lvl;
    if ((rc = num("DEBUG_LVL", d))) return rc;
    run->debug_lvl = (int)d;
    int sph = 0, sym = 1;
    if ((rc = flag("RUNSPH", sph))) return rc;
    if (sph) return fail(MLH_ERR_INVALID, "RUNSPH: the SPH path is not the MFV step");
    if (defs.count("ENFORCE_FLUX_SYM")) {
        if ((rc = flag("ENFORCE_FLUX_SYM", sym))) return rc;
        if (!sym) return fail(MLH_ERR_INVALID, "ENFORCE_FLUX_SYM 0 is not supported: faces are solved once");
    }
    if (c.adaptive_timestep && !defs.count("CFL"))
        return fail(MLH_ERR_INVALID, "ADAPTIVE_TIMESTEP needs CFL");
    return 0;
}

int mlh_read_config_info(const char *path, mlh_run_config *run) {
    if (!path || !run) return fail(MLH_ERR_INVALID, "null argument");
    std::ifstream f(path);
    if (!f) return fail(MLH_ERR_INVALID, std::string("cannot open ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    InfoNode root;
    std::string err;
    size_t p = 0;
    const std::vector<std::string> tok = info_tokens(ss.str());
    if (!info_parse(tok, p, root, 0, err)) return fail(MLH_ERR_INVALID, std::string(path) + ": " + err);
    auto get = [&](const InfoNode &n, const char *k, std::string &v) -> int {
        auto it = n.values.find(k);
        if (it == n.values.end()) return fail(MLH_ERR_INVALID, std::string("config.info: no key '") + k + "'");
        v = it->second;
        return 0;
    };
    auto getd = [&](const InfoNode &n, const char *k, double &v) -> int {
        std::string s;
        if (int rc = get(n, k, s)) return rc;
        if (!to_double(s, v)) return fail(MLH_ERR_INVALID, std::string("config.info: ") + k + " is not a number");
        return 0;
    };
    std::string s;
    int rc;
    if ((rc = get(root, "initFile", s))) return rc;
    copy_str(run->init_file, sizeof(run->init_file), s);
    if ((rc = get(root, "outDir", s))) return rc;
    copy_str(run->out_dir, sizeof(run->out_dir), s);
    if ((rc = getd(root, "timeStep", run->cfg.time_step))) return rc;
    if ((rc = getd(root, "timeEnd", run->time_end))) return rc;
    if ((rc = get(root, "h5DumpInterval", s))) return rc;
    if (!to_int(s, run->h5_dump_interval)) return fail(MLH_ERR_INVALID, "config.info: h5DumpInterval is not an integer");
    if ((rc = getd(root, "kernelSize", run->cfg.kernel_size))) return rc;
    if ((rc = getd(root, "gamma", run->cfg.gamma))) return rc;
    if (run->cfg.periodic) {
        auto it = root.children.find("periodicBoxLimits");
        if (it == root.children.end()) return fail(MLH_ERR_INVALID, "config.info: no block 'periodicBoxLimits'");
        const InfoNode &b = *it->second;
        const char *lo[3] = {"lowerX", "lowerY", "lowerZ"}, *hi[3] = {"upperX", "upperY", "upperZ"};
        for (int a = 0; a < 3; ++a) { run->cfg.box_lo[a] = 0.; run->cfg.box_hi[a] = 0.; }
        for (int a = 0; a < run->cfg.dim; ++a) {
            if ((rc = getd(b, lo[a], run->cfg.box_lo[a]))) return rc;
            if ((rc = getd(b, hi[a], run->cfg.box_hi[a]))) return rc;
        }
    }
    if (run->h5_dump_interval < 1) return fail(MLH_ERR_INVALID, "config.info: h5DumpInterval must be positive");
    return 0;
}

int mlh_info_get(const char *file, const char *key_path, char *out, int cap) {
    if (!file || !key_path || !out || cap < 1) return fail(MLH_ERR_INVALID, "null argument");
    std::ifstream f(file);
    if (!f) return fail(MLH_ERR_INVALID, std::string("cannot open ") + file);
    std::stringstream ss;
    ss << f.rdbuf();
    InfoNode root;
    std::string err;
    size_t p = 0;
    if (!info_parse(info_tokens(ss.str()), p, root, 0, err)) return fail(MLH_ERR_INVALID, std::string(file) + ": " + err);
    const InfoNode *node = &root;
    std::string path = key_path;
    size_t dot;
    while ((dot = path.find('.')) != std::string::npos) {
        auto it = node->children.find(path.substr(0, dot));
        if (it == node->children.end()) return fail(MLH_ERR_INVALID, std::string("config.info: no block '") + path.substr(0, dot) + "'");
        node = it->second.get();
        path = path.substr(dot + 1);
    }
    auto it = node->values.find(path);
    if (it == node->values.end()) return fail(MLH_ERR_INVALID, std::string("config.info: no key '") + key_path + "'");
    copy_str(out, (size_t)cap, it->second);
    return 0;
}

int mlh_h5_dataset_info(const char *file, const char *name, int *rank, long long dims[2], int *elem_class,
                        int *elem_size) {
    if (!file || !name) return fail(MLH_ERR_INVALID, "null argument");
    Reader r;
    DatasetInfo di;
    if (!dataset(r, file, name, di)) return fail(MLH_ERR_INVALID, std::string(file) + ": " + r.err);
    if (rank) *rank = di.rank;
    if (dims) { dims[0] = (long long)di.dims[0]; dims[1] = di.rank > 1 ? (long long)di.dims[1] : 1; }
    if (elem_class) *elem_class = di.cls;
    if (elem_size) *elem_size = di.size;
    return 0;
}

int mlh_h5_read_f64(const char *file, const char *name, double *out, long long count) {
    if (!file || !name || (count > 0 && !out)) return fail(MLH_ERR_INVALID, "null argument");
    return read_as<double>(file, name, out, count) ? 0 : MLH_ERR_INVALID;
}

int mlh_h5_read_i32(const char *file, const char *name, int *out, long long count) {
    if (!file || !name || (count > 0 && !out)) return fail(MLH_ERR_INVALID, "null argument");
    return read_as<int>(file, name, out, count) ? 0 : MLH_ERR_INVALID;
}

int mlh_h5_create(const char *file, mlh_h5_writer **out) {
    if (!file || !out) return fail(MLH_ERR_INVALID, "null argument");
    *out = new mlh_h5_writer();
    (*out)->path = file;
    return 0;
}

int mlh_h5_add_f64(mlh_h5_writer *w, const char *name, int rank, const long long *dims, const double *data) {
    return add_set(w, name, rank, dims, data, true);
}

int mlh_h5_add_i32(mlh_h5_writer *w, const char *name, int rank, const long long *dims, const int *data) {
    return add_set(w, name, rank, dims, data, false);
}

int mlh_h5_close(mlh_h5_writer *w) {
    if (!w) return fail(MLH_ERR_INVALID, "null writer");
    const int rc = write_file(w);
    delete w;
    return rc;
}

int mlh_read_initial_count(const char *file, int *n) {
    if (!file || !n) return fail(MLH_ERR_INVALID, "null argument");
    const char *names[5] = {"m", "x", "v", "u", "materialId"};
    long long len[5];
    for (int k = 0; k < 5; ++k) {
        int rank;
        long long dims[2];
        if (int rc = mlh_h5_dataset_info(file, names[k], &rank, dims, nullptr, nullptr)) return rc;
        len[k] = dims[0];
    }
    for (int k = 1; k < 5; ++k)
        if (len[k] != len[0]) return fail(MLH_ERR_INVALID, "Length mismatch between mass, position and/or velocity vectors.");
    if (len[0] < 1 || len[0] > 0x7fffffff) return fail(MLH_ERR_INVALID, "bad particle count");
    *n = (int)len[0];
    return 0;
}

int mlh_read_initial_distribution(const char *file, int dim, mlh_particles_view *v, int *material_id) {
    if (!file || !v || (dim != 2 && dim != 3)) return fail(MLH_ERR_INVALID, "invalid argument");
    int n = 0;
    if (int rc = mlh_read_initial_count(file, &n)) return rc;
    if (n != v->n) return fail(MLH_ERR_INVALID, "particle view size does not match the file");
    double *X[3] = {v->x, v->y, v->z}, *V[3] = {v->vx, v->vy, v->vz};
    const char *vec[2] = {"x", "v"};
    for (int q = 0; q < 2; ++q) {
        int rank;
        long long dims[2];
        if (int rc = mlh_h5_dataset_info(file, vec[q], &rank, dims, nullptr, nullptr)) return rc;
        if (rank != 2 || dims[1] < dim) return fail(MLH_ERR_INVALID, std::string("/") + vec[q] + " must be N x DIM");
        std::vector<double> buf((size_t)dims[0] * dims[1]);
        if (int rc = mlh_h5_read_f64(file, vec[q], buf.data(), (long long)buf.size())) return rc;
        double **dst = q == 0 ? X : V;
        for (int a = 0; a < dim; ++a) {
            if (!dst[a]) return fail(MLH_ERR_INVALID, "missing array in the particle view");
            for (int i = 0; i < n; ++i) dst[a][i] = buf[(size_t)i * dims[1] + a];
        }
    }
    if (!v->m || !v->u) return fail(MLH_ERR_INVALID, "missing array in the particle view");
    if (int rc = mlh_h5_read_f64(file, "m", v->m, n)) return rc;
    if (int rc = mlh_h5_read_f64(file, "u", v->u, n)) return rc;
    if (material_id)
        if (int rc = mlh_h5_read_i32(file, "materialId", material_id, n)) return rc;
    return 0;
}

int mlh_write_snapshot(const char *file, int dim, const mlh_particles_view *v, const double *rho, const double *P,
                       const double *rho_grad, const int *noi, const int *material_id, double time) {
    if (!file || !v || (dim != 2 && dim != 3) || v->n < 0) return fail(MLH_ERR_INVALID, "invalid argument");
    const int n = v->n;
    const double *vx = v->vx, *vy = v->vy, *vz = v->vz, *m = v->m, *u = v->u;
    if (!v->x || !v->y || !vx || !vy || !m || !u || (dim == 3 && (!v->z || !vz)))
        return fail(MLH_ERR_INVALID, "missing array in the particle view");
    // Particles::sumMass / sumEnergy / sumMomentumX/Y/Z (Particles.cpp:2839-2886)
    double M = 0., E = 0., px = 0., py = 0., pz = 0.;
    for (int i = 0; i < n; ++i) M += m[i];
    for (int i = 0; i < n; ++i) {
        if (dim == 2) E += m[i] * (u[i] + .5 * (vx[i] * vx[i] + vy[i] * vy[i]));
        else E += m[i] * (u[i] + .5 * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]));
    }
    for (int i = 0; i < n; ++i) px += m[i] * vx[i];
    for (int i = 0; i < n; ++i) py += m[i] * vy[i];
    if (dim == 3) for (int i = 0; i < n; ++i) pz += m[i] * vz[i];
    mlh_h5_writer *w = nullptr;
    if (int rc = mlh_h5_create(file, &w)) return rc;
    const long long one = 1, nn = n, nd[2] = {n, dim};
    int rc = 0;
    auto scalar = [&](const char *k, double val) { if (!rc) rc = mlh_h5_add_f64(w, k, 1, &one, &val); };
    scalar("time", time);
    scalar("totalMass", M);
    scalar("energy", E);
    scalar("xMomentum", px);
    scalar("yMomentum", py);
    if (dim == 3) scalar("zMomentum", pz);
    std::vector<double> zeros;
    auto vecN = [&](const char *k, const double *a) {
        if (rc) return;
        if (!a) { zeros.assign(n, 0.); a = zeros.data(); }
        rc = mlh_h5_add_f64(w, k, 1, &nn, a);
    };
    vecN("rho", rho);
    vecN("m", m);
    vecN("u", u);
    vecN("P", P);
    std::vector<double> buf((size_t)n * dim);
    auto vecND = [&](const char *k, const double *const *cols, const double *stride3) {
        if (rc) return;
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < dim; ++a)
                buf[(size_t)i * dim + a] = stride3 ? stride3[(size_t)i * 3 + a] : (cols ? cols[a][i] : 0.);
        rc = mlh_h5_add_f64(w, k, 2, nd, buf.data());
    };
    const double *xs[3] = {v->x, v->y, v->z}, *vs[3] = {vx, vy, vz};
    vecND("x", xs, nullptr);
    vecND("v", vs, nullptr);
    vecND("rhoGrad", nullptr, rho_grad);
    std::vector<int> izero;
    if (!rc) {
        if (!noi) izero.assign(n, 0);
        rc = mlh_h5_add_i32(w, "noi", 1, &nn, noi ? noi : izero.data());
    }
    if (!rc && material_id) rc = mlh_h5_add_i32(w, "materialId", 1, &nn, material_id);
    if (rc) {
        delete w;
        return rc;
    }
    return mlh_h5_close(w);
}

}  // extern "C"
