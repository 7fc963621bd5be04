// HDF5 classic-format subset: writer and reader (see h5.hpp for the scope).
//
// Layout written, per group: a version-1 object header holding a symbol-table message (and
// any attributes), a local heap with the member names ("" at offset 0, names padded to
// 8 bytes, a free block at the end as libhdf5 leaves it), symbol-table nodes of 2*4 entries
// and a v1 B-tree of 2*16 children per node, levels added as the member count requires.
// Per dataset: dataspace (v1, with maximum dims), datatype (IEEE float32 LE, or a v2 array
// of 3 of them), fill value (v2, default), contiguous layout (v3), modification time and
// attributes (v1).  Byte layouts follow the HDF5 file-format specification, version 0
// superblock, 8-byte offsets and lengths.
#include "h5.hpp"
#include "error.hpp"
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <map>

namespace spn {
namespace h5 {

namespace {

constexpr int kLeafK = 4;       // symbols per symbol-table node: 2 * kLeafK
constexpr int kInternalK = 16;  // children per B-tree node: 2 * kInternalK
constexpr int kSnodEntries = 2 * kLeafK;
constexpr int kTreeChildren = 2 * kInternalK;
constexpr uint64_t kSnodBytes = 8 + 40 * kSnodEntries;
constexpr uint64_t kTreeBytes = 24 + 8 * kTreeChildren + 8 * (kTreeChildren + 1);
constexpr uint64_t kSuperblockBytes = 96;
const char kSignature[8] = {'\x89', 'H', 'D', 'F', '\r', '\n', '\x1a', '\n'};

[[noreturn]] void fail(const std::string &m) { throw Error(ErrorType::IO, "HDF5: " + m); }
[[noreturn]] void unsupported(const std::string &m) { throw Error(ErrorType::Unsupported, "HDF5: " + m); }

uint64_t pad8(uint64_t x) { return (x + 7) & ~uint64_t(7); }

void put_le(std::string &s, uint64_t v, int n) {
    for (int i = 0; i < n; ++i) s.push_back(char((v >> (8 * i)) & 0xff));
}

// ---------------------------------------------------------------- encoders
std::string float_type() {
    std::string s;
    s.push_back(char(0x11));  // version 1, class 1 (floating point)
    s.push_back(char(0x20));  // little endian, mantissa normalisation "implied msb"
    s.push_back(char(31));    // sign bit position
    s.push_back(char(0));
    put_le(s, 4, 4);          // size
    put_le(s, 0, 2);          // bit offset
    put_le(s, 32, 2);         // bit precision
    s.push_back(char(23));    // exponent location
    s.push_back(char(8));     // exponent size
    s.push_back(char(0));     // mantissa location
    s.push_back(char(23));    // mantissa size
    put_le(s, 127, 4);        // exponent bias
    return s;                 // 20 bytes
}

std::string array3_type() {
    std::string s;
    s.push_back(char(0x2a));  // version 2, class 10 (array)
    s.append(3, '\0');
    put_le(s, 12, 4);         // 3 x float32
    s.push_back(char(1));     // rank
    s.append(3, '\0');
    put_le(s, 3, 4);          // dimension
    put_le(s, 0, 4);          // permutation index
    s += float_type();
    return s;                 // 40 bytes
}

std::string dataspace(const std::vector<uint64_t> &dims) {
    if (dims.empty()) unsupported("scalar dataspaces are not written");
    std::string s;
    s.push_back(char(1));
    s.push_back(char(dims.size()));
    s.push_back(char(1));  // maximum dimensions present
    s.append(5, '\0');
    for (uint64_t d : dims) put_le(s, d, 8);
    for (uint64_t d : dims) put_le(s, d, 8);
    return s;
}

struct Messages {
    std::string bytes;
    int n = 0;
    void add(uint16_t type, uint8_t flags, const std::string &body) {
        uint64_t len = pad8(body.size());
        put_le(bytes, type, 2);
        put_le(bytes, len, 2);
        bytes.push_back(char(flags));
        bytes.append(3, '\0');
        bytes += body;
        bytes.append(len - body.size(), '\0');
        ++n;
    }
};

std::string attribute_body(const Attribute &a) {
    uint64_t count = 1;
    for (uint64_t d : a.dims) count *= d;
    if (count != a.data.size()) throw Error(ErrorType::Internal, "HDF5: attribute '" + a.name + "' size mismatch");
    std::string t = float_type(), sp = dataspace(a.dims);
    std::string s;
    s.push_back(char(1));
    s.push_back(char(0));
    put_le(s, a.name.size() + 1, 2);
    put_le(s, t.size(), 2);
    put_le(s, sp.size(), 2);
    std::string name = a.name;
    name.push_back('\0');
    name.append(pad8(name.size()) - name.size(), '\0');
    s += name;
    s += t;
    s.append(pad8(t.size()) - t.size(), '\0');
    s += sp;
    s.append(pad8(sp.size()) - sp.size(), '\0');
    s.append(reinterpret_cast<const char *>(a.data.data()), a.data.size() * sizeof(float));
    return s;
}

// ---------------------------------------------------------------- image builder
struct Image {
    uint64_t base;
    std::string b;
    explicit Image(uint64_t base_) : base(base_) {}
    uint64_t end() const { return base + b.size(); }
    uint64_t alloc(uint64_t n) {
        uint64_t a = pad8(end());
        b.append(a - end() + n, '\0');
        return a;
    }
    char *at(uint64_t addr) { return &b[addr - base]; }
    void w(uint64_t addr, uint64_t v, int n) {
        char *p = at(addr);
        for (int i = 0; i < n; ++i) p[i] = char((v >> (8 * i)) & 0xff);
    }
    void wbytes(uint64_t addr, const std::string &s) { std::memcpy(at(addr), s.data(), s.size()); }
};

uint64_t write_header(Image &img, const Messages &m) {
    uint64_t a = img.alloc(16 + m.bytes.size());
    img.w(a, 1, 1);                 // version
    img.w(a + 2, m.n, 2);           // messages
    img.w(a + 4, 1, 4);             // reference count
    img.w(a + 8, m.bytes.size(), 4);
    img.wbytes(a + 16, m.bytes);
    return a;
}

uint32_t now_seconds() { return uint32_t(std::time(nullptr)); }

struct Member {
    std::string name;
    const Group *g = nullptr;
    const Dataset *d = nullptr;
};

struct Written {
    uint64_t header = 0, btree = kUndef, heap = kUndef;
};

Written write_group(Image &img, const Group &g, bool reuse);

uint64_t write_dataset(Image &img, const Dataset &d) {
    uint64_t count = d.count();
    uint64_t nbytes = count * sizeof(float);
    uint64_t addr;
    if (!d.data.empty()) {
        if (d.data.size() != count) throw Error(ErrorType::Internal, "HDF5: dataset '" + d.name + "' size mismatch");
        addr = img.alloc(nbytes);
        std::memcpy(img.at(addr), d.data.data(), nbytes);
    } else if (count == 0) {
        addr = kUndef;
    } else if (d.addr != kUndef && !d.compact && d.nbytes == nbytes) {
        addr = d.addr;  // storage already in the file this image is appended to
    } else {
        throw Error(ErrorType::Internal, "HDF5: dataset '" + d.name + "' has no values to write");
    }
    Messages m;
    m.add(0x0001, 0, dataspace(d.dims));
    m.add(0x0003, 1, d.array3 ? array3_type() : float_type());
    m.add(0x0005, 1, std::string("\x02\x02\x02\x01\x00\x00\x00\x00", 8));
    std::string layout;
    layout.push_back(char(3));
    layout.push_back(char(1));  // contiguous
    put_le(layout, addr, 8);
    put_le(layout, nbytes, 8);
    m.add(0x0008, 0, layout);
    std::string mtime;
    mtime.push_back(char(1));
    mtime.append(3, '\0');
    put_le(mtime, now_seconds(), 4);
    m.add(0x0012, 0, mtime);
    for (const Attribute &a : d.attrs) m.add(0x000C, 0, attribute_body(a));
    return write_header(img, m);
}

// reuse: objects of unchanged subgroups that already exist in the file are referenced.
Written write_group(Image &img, const Group &g, bool reuse) {
    std::vector<Member> mem;
    for (const Group &c : g.groups) mem.push_back({c.name, &c, nullptr});
    for (const Dataset &c : g.datasets) mem.push_back({c.name, nullptr, &c});
    std::sort(mem.begin(), mem.end(), [](const Member &a, const Member &b) { return a.name < b.name; });
    for (size_t i = 0; i < mem.size(); ++i) {
        if (mem[i].name.empty() || mem[i].name.find('/') != std::string::npos)
            throw Error(ErrorType::Argument, "HDF5: invalid member name '" + mem[i].name + "'");
        if (i > 0 && mem[i].name == mem[i - 1].name) throw Error(ErrorType::Argument, "HDF5: duplicate member '" + mem[i].name + "'");
    }

    // local heap: "" at 0, then the names
    std::vector<uint64_t> name_off(mem.size());
    uint64_t used = 8;
    for (size_t i = 0; i < mem.size(); ++i) {
        name_off[i] = used;
        used += pad8(mem[i].name.size() + 1);
    }
    uint64_t dsize = 88;
    while (dsize < used + 16) dsize *= 2;

    // symbol-table nodes and B-tree levels
    size_t n_snod = (mem.size() + kSnodEntries - 1) / kSnodEntries;
    std::vector<uint64_t> snod(n_snod);
    std::vector<size_t> snod_last(n_snod);  // index of the last member in each node
    for (size_t k = 0; k < n_snod; ++k) snod_last[k] = std::min(mem.size(), (k + 1) * kSnodEntries) - 1;

    Written out;
    Messages hm;
    hm.add(0x0011, 0, std::string(16, '\0'));  // patched below
    for (const Attribute &a : g.attrs) hm.add(0x000C, 0, attribute_body(a));
    out.header = write_header(img, hm);

    out.heap = img.alloc(32 + dsize);
    uint64_t heap_data = out.heap + 32;
    std::memcpy(img.at(out.heap), "HEAP", 4);
    img.w(out.heap + 8, dsize, 8);
    img.w(out.heap + 16, used, 8);  // free list head: the free block at the end
    img.w(out.heap + 24, heap_data, 8);
    for (size_t i = 0; i < mem.size(); ++i) std::memcpy(img.at(heap_data + name_off[i]), mem[i].name.data(), mem[i].name.size());
    img.w(heap_data + used, 1, 8);  // next free block: none
    img.w(heap_data + used + 8, dsize - used, 8);

    for (size_t k = 0; k < n_snod; ++k) snod[k] = img.alloc(kSnodBytes);

    // B-tree: level 0 points at symbol-table nodes; higher levels at B-tree nodes.  Each
    // child carries the heap offset of the largest name below it.
    struct Child { uint64_t addr; uint64_t max_key; };
    std::vector<Child> level;
    for (size_t k = 0; k < n_snod; ++k) level.push_back({snod[k], name_off[snod_last[k]]});
    int depth = 0;
    uint64_t root = kUndef;
    do {
        size_t n_nodes = std::max<size_t>(1, (level.size() + kTreeChildren - 1) / kTreeChildren);
        std::vector<uint64_t> nodes(n_nodes);
        for (size_t i = 0; i < n_nodes; ++i) nodes[i] = img.alloc(kTreeBytes);
        std::vector<Child> up;
        uint64_t left_key = 0;
        for (size_t i = 0; i < n_nodes; ++i) {
            uint64_t a = nodes[i];
            size_t lo = i * kTreeChildren, hi = std::min(level.size(), lo + kTreeChildren);
            std::memcpy(img.at(a), "TREE", 4);
            img.w(a + 4, 0, 1);  // group node
            img.w(a + 5, depth, 1);
            img.w(a + 6, hi - lo, 2);
            img.w(a + 8, i > 0 ? nodes[i - 1] : kUndef, 8);
            img.w(a + 16, i + 1 < n_nodes ? nodes[i + 1] : kUndef, 8);
            uint64_t p = a + 24;
            img.w(p, left_key, 8);
            for (size_t c = lo; c < hi; ++c) {
                img.w(p + 8, level[c].addr, 8);
                img.w(p + 16, level[c].max_key, 8);
                p += 16;
            }
            if (hi > lo) left_key = level[hi - 1].max_key;
            up.push_back({a, hi > lo ? level[hi - 1].max_key : 0});
        }
        level.swap(up);
        ++depth;
        if (level.size() == 1) root = level[0].addr;
    } while (level.size() > 1);
    out.btree = root;
    img.w(out.header + 16 + 8, out.btree, 8);
    img.w(out.header + 16 + 16, out.heap, 8);

    for (size_t k = 0; k < n_snod; ++k) {
        uint64_t a = snod[k];
        size_t lo = k * kSnodEntries, hi = snod_last[k] + 1;
        std::memcpy(img.at(a), "SNOD", 4);
        img.w(a + 4, 1, 1);
        img.w(a + 6, hi - lo, 2);
        for (size_t i = lo; i < hi; ++i) {
            uint64_t e = a + 8 + 40 * (i - lo);
            img.w(e, name_off[i], 8);
            if (mem[i].g) {
                const Group &cg = *mem[i].g;
                Written c = (reuse && cg.header != kUndef) ? Written{cg.header, cg.btree, cg.heap} : write_group(img, cg, reuse);
                img.w(e + 8, c.header, 8);
                img.w(e + 16, 1, 4);
                img.w(e + 24, c.btree, 8);
                img.w(e + 32, c.heap, 8);
            } else {
                img.w(e + 8, write_dataset(img, *mem[i].d), 8);
            }
        }
    }
    return out;
}

void write_superblock(char *p, uint64_t eof, const Written &root) {
    std::string s(kSignature, 8);
    s.append(5, '\0');        // superblock, free-space, root-entry, reserved, shared-header versions
    s.push_back(char(8));     // size of offsets
    s.push_back(char(8));     // size of lengths
    s.push_back(char(0));
    put_le(s, kLeafK, 2);
    put_le(s, kInternalK, 2);
    put_le(s, 0, 4);          // consistency flags
    put_le(s, 0, 8);          // base address
    put_le(s, kUndef, 8);     // free-space info
    put_le(s, eof, 8);
    put_le(s, kUndef, 8);     // driver info
    put_le(s, 0, 8);          // root entry: name offset
    put_le(s, root.header, 8);
    put_le(s, 1, 4);          // cache type: symbol table
    put_le(s, 0, 4);
    put_le(s, root.btree, 8);
    put_le(s, root.heap, 8);
    std::memcpy(p, s.data(), s.size());
}

// ---------------------------------------------------------------- reader
class Reader {
public:
    explicit Reader(const std::string &path) : path_(path) {
        f_ = std::fopen(path.c_str(), "rb");
        if (!f_) fail("cannot open '" + path + "' for reading");
        std::fseek(f_, 0, SEEK_END);
        size_ = uint64_t(ftello(f_));
    }
    ~Reader() {
        if (f_) std::fclose(f_);
    }
    Reader(const Reader &) = delete;
    Reader &operator=(const Reader &) = delete;
    uint64_t size() const { return size_; }
    std::string bytes(uint64_t off, uint64_t n) const {
        if (off > size_ || n > size_ - off) fail("'" + path_ + "' is truncated or corrupt (read past end)");
        std::string s(n, '\0');
        if (n) {
            fseeko(f_, off_t(off), SEEK_SET);
            if (std::fread(&s[0], 1, n, f_) != n) fail("read error on '" + path_ + "'");
        }
        return s;
    }
    uint64_t u(uint64_t off, int n) const {
        std::string s = bytes(off, n);
        uint64_t v = 0;
        for (int i = n - 1; i >= 0; --i) v = (v << 8) | uint8_t(s[i]);
        return v;
    }

private:
    std::string path_;
    FILE *f_ = nullptr;
    uint64_t size_ = 0;
};

uint64_t ule(const std::string &s, size_t off, int n) {
    if (off + n > s.size()) fail("message too short");
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | uint8_t(s[off + i]);
    return v;
}

struct TypeInfo {
    int array3 = 0;
    size_t len = 0;  // encoded length
};

TypeInfo decode_type(const std::string &s, size_t off) {
    uint8_t cv = uint8_t(s.at(off));
    int cls = cv & 0x0f, ver = cv >> 4;
    uint64_t size = ule(s, off + 4, 4);
    if (cls == 1) {
        if (size != 4 || (uint8_t(s.at(off + 1)) & 1)) unsupported("only little-endian float32 data is supported");
        return {0, 20};
    }
    if (cls == 10) {
        int rank = uint8_t(s.at(off + 8));
        size_t p;
        std::vector<uint64_t> dims;
        if (ver == 2) {
            for (int i = 0; i < rank; ++i) dims.push_back(ule(s, off + 12 + 4 * i, 4));
            p = off + 12 + 8 * rank;
        } else {
            for (int i = 0; i < rank; ++i) dims.push_back(ule(s, off + 9 + 4 * i, 4));
            p = off + 9 + 4 * rank;
        }
        TypeInfo base = decode_type(s, p);
        if (base.array3 || dims.size() != 1 || dims[0] != 3) unsupported("only float32[3] array types are supported");
        return {1, p - off + base.len};
    }
    unsupported("datatype class " + std::to_string(cls) + " is not supported");
}

std::vector<uint64_t> decode_space(const std::string &s, size_t off) {
    int ver = uint8_t(s.at(off)), rank = uint8_t(s.at(off + 1));
    size_t p;
    if (ver == 1) p = off + 8;
    else if (ver == 2) p = off + 4;
    else unsupported("dataspace version " + std::to_string(ver));
    std::vector<uint64_t> dims;
    for (int i = 0; i < rank; ++i) dims.push_back(ule(s, p + 8 * i, 8));
    return dims;
}

Attribute decode_attribute(const std::string &s) {
    int ver = uint8_t(s.at(0));
    uint64_t nlen = ule(s, 2, 2), tlen = ule(s, 4, 2), slen = ule(s, 6, 2);
    auto pad = [&](uint64_t x) { return ver == 1 ? pad8(x) : x; };
    size_t p = (ver == 3) ? 9 : 8;
    Attribute a;
    a.name = std::string(s.c_str() + p);
    p += pad(nlen);
    TypeInfo t = decode_type(s, p);
    p += pad(tlen);
    a.dims = decode_space(s, p);
    p += pad(slen);
    uint64_t count = 1;
    for (uint64_t d : a.dims) count *= d;
    count *= t.array3 ? 3 : 1;
    if (p + count * 4 > s.size()) fail("attribute '" + a.name + "' is truncated");
    a.data.resize(count);
    std::memcpy(a.data.data(), s.data() + p, count * 4);
    return a;
}

struct Node {
    bool is_group = false;
    uint64_t btree = 0, heap = 0;
    Dataset d;
    std::vector<Attribute> attrs;
};

Node read_node(const Reader &r, uint64_t addr) {
    if (r.u(addr, 1) != 1) unsupported("object header version " + std::to_string(r.u(addr, 1)) + " (only version 1 is read)");
    uint64_t nmsg = r.u(addr + 2, 2), size = r.u(addr + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, size}};
    Node n;
    bool have_space = false, have_type = false, have_layout = false;
    uint64_t seen = 0;
    for (size_t bi = 0; bi < blocks.size() && seen < nmsg; ++bi) {
        std::string blk = r.bytes(blocks[bi].first, blocks[bi].second);
        size_t p = 0;
        while (p + 8 <= blk.size() && seen < nmsg) {
            uint64_t type = ule(blk, p, 2), len = ule(blk, p + 2, 2);
            if (p + 8 + len > blk.size()) fail("object header message overruns its block");
            std::string body = blk.substr(p + 8, len);
            switch (type) {
                case 0x10: blocks.push_back({ule(body, 0, 8), ule(body, 8, 8)}); break;
                case 0x11:
                    n.is_group = true;
                    n.btree = ule(body, 0, 8);
                    n.heap = ule(body, 8, 8);
                    break;
                case 0x01: n.d.dims = decode_space(body, 0); have_space = true; break;
                case 0x03: n.d.array3 = decode_type(body, 0).array3; have_type = true; break;
                case 0x08: {
                    int ver = uint8_t(body.at(0));
                    if (ver == 3) {
                        int cls = uint8_t(body.at(1));
                        if (cls == 1) {
                            n.d.addr = ule(body, 2, 8);
                            n.d.nbytes = ule(body, 10, 8);
                        } else if (cls == 0) {
                            uint64_t sz = ule(body, 2, 2);
                            n.d.compact = true;
                            n.d.nbytes = sz;
                            n.d.data.resize(sz / 4);
                            std::memcpy(n.d.data.data(), body.data() + 4, (sz / 4) * 4);
                        } else {
                            unsupported("chunked dataset layout");
                        }
                    } else if (ver == 1 || ver == 2) {
                        if (uint8_t(body.at(2)) != 1) unsupported("dataset layout class");
                        n.d.addr = ule(body, 8, 8);
                        n.d.nbytes = kUndef;
                    } else {
                        unsupported("layout message version " + std::to_string(ver));
                    }
                    have_layout = true;
                    break;
                }
                case 0x0C: n.attrs.push_back(decode_attribute(body)); break;
                default: break;  // NIL, fill value, modification time, ...
            }
            ++seen;
            p += 8 + len;
        }
    }
    if (!n.is_group && !(have_space && have_type && have_layout)) unsupported("object at " + std::to_string(addr) + " is neither a group nor a simple dataset");
    if (!n.is_group && n.d.nbytes == kUndef) n.d.nbytes = n.d.count() * 4;
    return n;
}

void read_group(const Reader &r, uint64_t btree, uint64_t heap, Group &g, int depth);

void collect(const Reader &r, uint64_t node, uint64_t heap_data, std::vector<std::pair<std::string, uint64_t>> &out, int guard) {
    if (guard > 64) fail("B-tree too deep");
    if (r.bytes(node, 4) != "TREE") fail("bad B-tree node");
    int level = int(r.u(node + 5, 1));
    uint64_t used = r.u(node + 6, 2);
    for (uint64_t i = 0; i < used; ++i) {
        uint64_t child = r.u(node + 24 + 16 * i + 8, 8);
        if (level > 0) {
            collect(r, child, heap_data, out, guard + 1);
            continue;
        }
        if (r.bytes(child, 4) != "SNOD") fail("bad symbol-table node");
        uint64_t nsym = r.u(child + 6, 2);
        for (uint64_t k = 0; k < nsym; ++k) {
            uint64_t e = child + 8 + 40 * k;
            uint64_t name_off = r.u(e, 8), header = r.u(e + 8, 8);
            std::string name;
            for (uint64_t p = heap_data + name_off;; ++p) {
                char c = char(r.u(p, 1));
                if (!c) break;
                name.push_back(c);
                if (name.size() > 4096) fail("unterminated name in local heap");
            }
            out.push_back({name, header});
        }
    }
}

void read_group(const Reader &r, uint64_t btree, uint64_t heap, Group &g, int depth) {
    if (depth > 32) fail("groups nested too deeply");
    if (r.bytes(heap, 4) != "HEAP") fail("bad local heap");
    uint64_t heap_data = r.u(heap + 24, 8);
    std::vector<std::pair<std::string, uint64_t>> members;
    collect(r, btree, heap_data, members, 0);
    for (auto &m : members) {
        Node n = read_node(r, m.second);
        if (n.is_group) {
            Group c;
            c.name = m.first;
            c.header = m.second;
            c.btree = n.btree;
            c.heap = n.heap;
            c.attrs = std::move(n.attrs);
            read_group(r, n.btree, n.heap, c, depth + 1);
            g.groups.push_back(std::move(c));
        } else {
            n.d.name = m.first;
            n.d.attrs = std::move(n.attrs);
            g.datasets.push_back(std::move(n.d));
        }
    }
}

}  // namespace

// ---------------------------------------------------------------- public API
uint64_t Dataset::count() const {
    uint64_t c = 1;
    for (uint64_t d : dims) c *= d;
    return c * (array3 ? 3 : 1);
}

Group *Group::group(const std::string &n) {
    for (Group &g : groups)
        if (g.name == n) return &g;
    return nullptr;
}
const Group *Group::group(const std::string &n) const { return const_cast<Group *>(this)->group(n); }
Dataset *Group::dataset(const std::string &n) {
    for (Dataset &d : datasets)
        if (d.name == n) return &d;
    return nullptr;
}
const Dataset *Group::dataset(const std::string &n) const { return const_cast<Group *>(this)->dataset(n); }
const Attribute *Group::attr(const std::string &n) const {
    for (const Attribute &a : attrs)
        if (a.name == n) return &a;
    return nullptr;
}
Group &Group::add_group(const std::string &n) {
    if (group(n) || dataset(n)) throw Error(ErrorType::Argument, "HDF5: member '" + n + "' exists");
    header = btree = heap = kUndef;  // this group changes: it is written anew
    groups.emplace_back();
    groups.back().name = n;
    return groups.back();
}
std::vector<std::string> Group::member_names() const {
    std::vector<std::string> v;
    for (const Group &g : groups) v.push_back(g.name);
    for (const Dataset &d : datasets) v.push_back(d.name);
    std::sort(v.begin(), v.end());
    return v;
}

bool File::is_hdf5(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char sig[8] = {0};
    size_t n = std::fread(sig, 1, 8, f);
    std::fclose(f);
    return n == 8 && std::memcmp(sig, kSignature, 8) == 0;
}

File File::open(const std::string &path) {
    Reader r(path);
    if (r.size() < kSuperblockBytes || r.bytes(0, 8) != std::string(kSignature, 8)) fail("'" + path + "' is not an HDF5 file");
    if (r.u(8, 1) != 0) unsupported("superblock version " + std::to_string(r.u(8, 1)) + " in '" + path + "'");
    if (r.u(13, 1) != 8 || r.u(14, 1) != 8) unsupported("only 8-byte offsets and lengths are supported");
    if (r.u(24, 8) != 0) unsupported("non-zero base address");
    File f;
    f.path = path;
    f.eof = r.u(40, 8);
    uint64_t header = r.u(64, 8);
    Node n = read_node(r, header);
    if (!n.is_group) fail("root object is not a group");
    f.root.attrs = std::move(n.attrs);
    read_group(r, n.btree, n.heap, f.root, 0);
    return f;
}

void File::load(Dataset &d) const {
    if (d.compact) return;
    uint64_t count = d.count();
    if (d.addr == kUndef) {
        d.data.assign(count, 0.0f);
        return;
    }
    if (d.nbytes != count * 4) fail("dataset '" + d.name + "' storage size does not match its shape");
    Reader r(path);
    std::string s = r.bytes(d.addr, d.nbytes);
    d.data.resize(count);
    std::memcpy(d.data.data(), s.data(), d.nbytes);
}

void File::load_all(Group &g) const {
    for (Dataset &d : g.datasets) load(d);
    for (Group &c : g.groups) load_all(c);
}

std::string serialize(const Group &root) {
    Image img(0);
    img.alloc(kSuperblockBytes);
    Written w = write_group(img, root, false);
    write_superblock(img.at(0), img.end(), w);
    return img.b;
}

void write_file(const std::string &path, const Group &root) {
    std::string bytes = serialize(root);
    std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) throw Error(ErrorType::IO, "Could not open file [" + path + "] for writing");
    bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        throw Error(ErrorType::IO, "Could not write file [" + path + "]");
    }
}

void append_file(const File &file, const Group &root) {
    FILE *f = std::fopen(file.path.c_str(), "r+b");
    if (!f) throw Error(ErrorType::IO, "Could not open file [" + file.path + "] for writing");
    std::fseek(f, 0, SEEK_END);
    uint64_t size = uint64_t(ftello(f));
    Image img(pad8(std::max(size, file.eof)));
    Written w = write_group(img, root, true);
    std::string sb(kSuperblockBytes, '\0');
    write_superblock(&sb[0], img.end(), w);
    bool ok = fseeko(f, off_t(img.base), SEEK_SET) == 0 && std::fwrite(img.b.data(), 1, img.b.size(), f) == img.b.size();
    // the new tree is complete on disk before the superblock points at it
    ok = ok && std::fflush(f) == 0;
    ok = ok && fseeko(f, 0, SEEK_SET) == 0 && std::fwrite(sb.data(), 1, sb.size(), f) == sb.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw Error(ErrorType::IO, "Could not append to file [" + file.path + "]");
}

}  // namespace h5
}  // namespace spn
