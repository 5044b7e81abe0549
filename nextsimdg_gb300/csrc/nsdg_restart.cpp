// NetCDF-4 (HDF5 subset) reader: see nsdg_restart.hpp for what it covers.
// Every address and length read from the file is checked against the file
// size before use; loops over file structures are bounded (continuation
// chunks by a visited set, B-tree and heap walks by depth), so a damaged
// file raises FormatError instead of reading out of bounds.
#include "nsdg_restart.hpp"

#include <algorithm>
#include <cstring>
#include <fcntl.h>
#include <functional>
#include <set>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

namespace nsdg_nc {

namespace {

constexpr uint64_t kUndef = UINT64_MAX;

inline uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

uint64_t le(const uint8_t* p, size_t n)
{
    uint64_t v = 0;
    for (size_t i = 0; i < n; ++i)
        v |= static_cast<uint64_t>(p[i]) << (8 * i);
    return v;
}

// bounds-checked little-endian reader over one message or block
struct Cur {
    const uint8_t* p;
    const uint8_t* end;
    void need(size_t n) const
    {
        if (p > end || static_cast<size_t>(end - p) < n)
            throw FormatError("truncated HDF5 structure");
    }
    uint64_t u(size_t n)
    {
        need(n);
        const uint64_t v = le(p, n);
        p += n;
        return v;
    }
    uint8_t u8() { return static_cast<uint8_t>(u(1)); }
    uint16_t u16() { return static_cast<uint16_t>(u(2)); }
    uint32_t u32() { return static_cast<uint32_t>(u(4)); }
    uint64_t u64() { return u(8); }
    void skip(size_t n)
    {
        need(n);
        p += n;
    }
    size_t left() const { return p > end ? 0 : static_cast<size_t>(end - p); }
};

int log2u(uint64_t v)
{
    int r = -1;
    while (v) {
        v >>= 1;
        ++r;
    }
    return r;
}

// Datatype message (type 0x0003)
Datatype parseType(Cur& c)
{
    Datatype t;
    const uint8_t cv = c.u8();
    const int cls = cv & 0x0f;
    const uint32_t bits = static_cast<uint32_t>(c.u(3));
    t.size = c.u32();
    switch (cls) {
    case 0: // fixed-point: bit offset, precision
        t.cls = TypeClass::Fixed;
        t.bigEndian = bits & 1u;
        t.isSigned = bits & 8u;
        c.skip(4);
        if (t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8)
            throw Unsupported("integer type of unusual size");
        break;
    case 1: { // floating-point: offset, precision, exponent and mantissa layout, bias
        t.cls = TypeClass::Float;
        t.bigEndian = bits & 1u;
        c.skip(12);
        if (t.size != 4 && t.size != 8)
            throw Unsupported("floating-point type of unusual size");
        break;
    }
    case 3:
        t.cls = TypeClass::String;
        break;
    case 7:
        t.cls = TypeClass::Reference;
        break;
    case 9:
        t.cls = TypeClass::VarLen;
        t.vlenString = (bits & 0x0fu) == 1u;
        t.base = std::make_shared<Datatype>(parseType(c));
        break;
    case 6: // compound (REFERENCE_LIST): kept as opaque bytes
        t.cls = TypeClass::Compound;
        c.p = c.end;
        break;
    default:
        t.cls = TypeClass::Other;
        c.p = c.end;
        break;
    }
    return t;
}

// Dataspace message (type 0x0001), versions 1 and 2
void parseSpace(Cur& c, std::vector<uint64_t>& dims, std::vector<uint64_t>* maxDims)
{
    const int ver = c.u8();
    const int rank = c.u8();
    const int flags = c.u8();
    if (ver == 1)
        c.skip(5);
    else if (ver == 2)
        c.skip(1); // 0 scalar, 1 simple, 2 null
    else
        throw Unsupported("dataspace message version " + std::to_string(ver));
    dims.resize(rank);
    for (int i = 0; i < rank; ++i)
        dims[i] = c.u64();
    if (maxDims) {
        maxDims->assign(dims.begin(), dims.end());
        if (flags & 1)
            for (int i = 0; i < rank; ++i)
                (*maxDims)[i] = c.u64();
    }
}

// n elements of es bytes: a damaged dataspace or type must not wrap the size
uint64_t bytesOf(uint64_t n, uint64_t es)
{
    if (es != 0 && n > UINT64_MAX / es)
        throw FormatError("data size overflows");
    return n * es;
}

uint64_t product(const std::vector<uint64_t>& d)
{
    uint64_t n = 1;
    for (uint64_t x : d) {
        if (x != 0 && n > UINT64_MAX / x)
            throw FormatError("dataspace size overflows");
        n *= x;
    }
    return n;
}

// one element of a numeric type, as double
double toDouble(const Datatype& t, const uint8_t* p)
{
    uint8_t b[8];
    std::memcpy(b, p, t.size);
    if (t.bigEndian)
        std::reverse(b, b + t.size);
    const uint64_t v = le(b, t.size);
    if (t.cls == TypeClass::Float) {
        if (t.size == 8) {
            double d;
            std::memcpy(&d, &v, 8);
            return d;
        }
        const uint32_t w = static_cast<uint32_t>(v);
        float f;
        std::memcpy(&f, &w, 4);
        return f;
    }
    if (t.cls == TypeClass::Fixed) {
        if (!t.isSigned)
            return static_cast<double>(v);
        const int sh = 64 - 8 * static_cast<int>(t.size);
        return static_cast<double>(static_cast<int64_t>(v << sh) >> sh);
    }
    throw Unsupported("not a numeric type");
}

} // namespace

uint32_t lookup3(const uint8_t* k, size_t length, uint32_t initval)
{
    uint32_t a, b, c;
    a = b = c = 0xdeadbeefu + static_cast<uint32_t>(length) + initval;
    auto mix = [&]() {
        a -= c; a ^= rotl(c, 4);  c += b;
        b -= a; b ^= rotl(a, 6);  a += c;
        c -= b; c ^= rotl(b, 8);  b += a;
        a -= c; a ^= rotl(c, 16); c += b;
        b -= a; b ^= rotl(a, 19); a += c;
        c -= b; c ^= rotl(b, 4);  b += a;
    };
    while (length > 12) {
        a += static_cast<uint32_t>(le(k, 4));
        b += static_cast<uint32_t>(le(k + 4, 4));
        c += static_cast<uint32_t>(le(k + 8, 4));
        mix();
        length -= 12;
        k += 12;
    }
    if (length == 0)
        return c;
    // the last 1..12 bytes, little-endian into a, b, c (missing bytes 0)
    uint8_t tail[12] = {};
    std::memcpy(tail, k, length);
    a += static_cast<uint32_t>(le(tail, 4));
    b += static_cast<uint32_t>(le(tail + 4, 4));
    c += static_cast<uint32_t>(le(tail + 8, 4));
    c ^= b; c -= rotl(b, 14);
    a ^= c; a -= rotl(c, 11);
    b ^= a; b -= rotl(a, 25);
    c ^= b; c -= rotl(b, 16);
    a ^= c; a -= rotl(c, 4);
    b ^= a; b -= rotl(a, 14);
    c ^= b; c -= rotl(b, 24);
    return c;
}

// ---------------------------------------------------------------- file
File::File(const std::string& path)
{
    fd_ = ::open(path.c_str(), O_RDONLY);
    if (fd_ < 0)
        throw std::runtime_error("cannot open " + path);
    struct stat st {};
    if (::fstat(fd_, &st) != 0 || st.st_size < 48) {
        ::close(fd_);
        fd_ = -1;
        throw FormatError(path + " is not an HDF5 file (too short)");
    }
    size_ = static_cast<uint64_t>(st.st_size);
    void* m = ::mmap(nullptr, size_, PROT_READ, MAP_PRIVATE, fd_, 0);
    if (m == MAP_FAILED) {
        ::close(fd_);
        fd_ = -1;
        throw std::runtime_error("cannot map " + path);
    }
    base_ = static_cast<const uint8_t*>(m);
    static const uint8_t sig[8] = { 0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n' };
    // the superblock sits at 0, 512, 1024, 2048, ... (after a user block)
    uint64_t at = 0;
    while (at + 48 <= size_ && std::memcmp(base_ + at, sig, 8) != 0)
        at = at ? 2 * at : 512;
    try {
        if (at + 48 > size_)
            throw FormatError(path + " is not an HDF5 file (no superblock signature)");
        const uint8_t* s = base_ + at;
        const int ver = s[8];
        if (ver == 0 || ver == 1)
            throw Unsupported("HDF5 superblock version " + std::to_string(ver)
                + " (files written without link creation order; netCDF-4 files use version 2 or 3)");
        if (ver != 2 && ver != 3)
            throw Unsupported("HDF5 superblock version " + std::to_string(ver));
        if (s[9] != 8 || s[10] != 8)
            throw Unsupported("HDF5 offsets or lengths not 8 bytes wide");
        if (lookup3(s, 44) != static_cast<uint32_t>(le(s + 44, 4)))
            throw FormatError("HDF5 superblock checksum mismatch");
        if (le(s + 12, 8) != at)
            throw Unsupported("HDF5 base address other than the superblock's position");
        rootAddr_ = le(s + 36, 8);
    } catch (...) {
        ::munmap(const_cast<uint8_t*>(base_), size_);
        ::close(fd_);
        throw;
    }
}

File::~File()
{
    if (base_)
        ::munmap(const_cast<uint8_t*>(base_), size_);
    if (fd_ >= 0)
        ::close(fd_);
}

const uint8_t* File::span(uint64_t addr, uint64_t len) const
{
    if (addr == kUndef || addr > size_ || len > size_ - addr)
        throw FormatError("HDF5 address out of the file");
    return base_ + addr;
}

const Object& File::object(uint64_t addr)
{
    auto it = objects_.find(addr);
    if (it != objects_.end())
        return *it->second;
    if (objects_.size() > 100000)
        throw FormatError("too many HDF5 objects");
    auto o = std::make_unique<Object>();
    o->addr = addr;
    parseHeader(*o);
    const Object& r = *o;
    objects_.emplace(addr, std::move(o));
    return r;
}

// version 2 object header: "OHDR", version, flags, [times], [attribute
// phase change], chunk-0 size, messages, checksum; continuation chunks
// "OCHK", messages, checksum
void File::parseHeader(Object& o)
{
    const uint8_t* h = span(o.addr, 6);
    if (h[0] == 1)
        throw Unsupported("version 1 HDF5 object header");
    if (std::memcmp(h, "OHDR", 4) != 0 || h[4] != 2)
        throw FormatError("bad HDF5 object header signature");
    const int flags = h[5];
    Cur c { h + 6, base_ + size_ };
    if (flags & 0x20)
        c.skip(16);
    if (flags & 0x10)
        c.skip(4);
    const uint64_t size0 = c.u(size_t(1) << (flags & 3));
    const uint64_t start0 = static_cast<uint64_t>(c.p - base_);
    const bool crtOrder = flags & 0x04;
    std::vector<uint64_t> dense;
    std::vector<std::pair<uint64_t, uint64_t>> conts;
    auto messages = [&](uint64_t from, uint64_t to) {
        Cur m { span(from, to - from), base_ + to };
        const size_t hdr = crtOrder ? 6 : 4;
        while (m.left() >= hdr) {
            const int type = m.u8();
            const size_t len = m.u16();
            const int mflags = m.u8();
            if (crtOrder)
                m.skip(2);
            m.need(len);
            if ((mflags & 0x02) && type != 0)
                throw Unsupported("shared HDF5 object header message");
            parseMessage(o, type, m.p, len, dense, conts);
            m.skip(len);
        }
    };
    const uint64_t end0 = start0 + size0;
    const uint8_t* ck = span(o.addr, end0 - o.addr + 4);
    if (lookup3(ck, end0 - o.addr) != static_cast<uint32_t>(le(ck + (end0 - o.addr), 4)))
        throw FormatError("HDF5 object header checksum mismatch");
    messages(start0, end0);
    std::set<uint64_t> seen;
    for (size_t i = 0; i < conts.size(); ++i) {
        const uint64_t a = conts[i].first, len = conts[i].second;
        if (!seen.insert(a).second || seen.size() > 10000)
            throw FormatError("HDF5 continuation chunks form a loop");
        const uint8_t* q = span(a, len);
        if (len < 8 || std::memcmp(q, "OCHK", 4) != 0)
            throw FormatError("bad HDF5 continuation chunk at " + std::to_string(a));
        if (lookup3(q, len - 4) != static_cast<uint32_t>(le(q + len - 4, 4)))
            throw FormatError("HDF5 continuation chunk checksum mismatch");
        messages(a + 4, a + len - 4);
    }
    if (dense.size() == 2)
        readDenseLinks(o, dense[0], dense[1]);
    if (o.isDataset && o.layoutClass < 0)
        throw FormatError("HDF5 dataset without a layout message");
}

void File::parseMessage(Object& o, int type, const uint8_t* p, size_t len, std::vector<uint64_t>& dense,
    std::vector<std::pair<uint64_t, uint64_t>>& conts)
{
    Cur c { p, p + len };
    switch (type) {
    case 0x01: // dataspace
        parseSpace(c, o.dims, &o.maxDims);
        break;
    case 0x02: { // link info
        c.u8();
        const int f = c.u8();
        if (f & 1)
            c.skip(8);
        const uint64_t heap = c.u64();
        const uint64_t names = c.u64();
        if (heap != kUndef)
            dense = { heap, names };
        break;
    }
    case 0x03: // datatype
        o.type = parseType(c);
        o.isDataset = true;
        break;
    case 0x05: { // fill value, versions 2 and 3
        const int ver = c.u8();
        bool defined = false;
        if (ver == 1 || ver == 2) {
            c.skip(2);
            defined = c.u8() != 0;
            if (ver == 1)
                defined = true;
        } else if (ver == 3) {
            const int f = c.u8();
            defined = f & 0x20;
        }
        if (defined && c.left() >= 4) {
            const uint32_t n = c.u32();
            c.need(n);
            o.fill.assign(c.p, c.p + n);
        }
        break;
    }
    case 0x06: { // link
        if (c.u8() != 1)
            throw Unsupported("link message version");
        const int f = c.u8();
        int ltype = 0;
        if (f & 0x08)
            ltype = c.u8();
        if (f & 0x04)
            c.skip(8);
        if (f & 0x10)
            c.skip(1);
        const uint64_t n = c.u(size_t(1) << (f & 3));
        c.need(n);
        std::string name(reinterpret_cast<const char*>(c.p), n);
        c.skip(n);
        if (ltype == 0)
            o.links.emplace_back(name, c.u64());
        break;
    }
    case 0x08: { // data layout
        const int ver = c.u8();
        if (ver != 3 && ver != 4)
            throw Unsupported("data layout message version " + std::to_string(ver));
        o.layoutClass = c.u8();
        if (o.layoutClass == 0) {
            const size_t n = c.u16();
            c.need(n);
            o.compact.assign(c.p, c.p + n);
        } else if (o.layoutClass == 1) {
            o.dataAddr = c.u64();
            o.dataSize = c.u64();
        } else if (o.layoutClass == 2) {
            if (ver == 4)
                throw Unsupported("chunked layout with a version 4 index (files written for HDF5 1.10 only)");
            const int nd = c.u8();
            o.dataAddr = c.u64();
            o.chunk.resize(nd);
            for (int i = 0; i < nd; ++i)
                o.chunk[i] = c.u32();
        } else {
            throw Unsupported("virtual dataset layout");
        }
        break;
    }
    case 0x0B: // filter pipeline
        o.hasFilters = true;
        break;
    case 0x0C: { // attribute
        const int ver = c.u8();
        const int f = c.u8();
        if (f & 0x03)
            throw Unsupported("shared attribute datatype or dataspace");
        const size_t ns = c.u16(), ts = c.u16(), ss = c.u16();
        if (ver == 3)
            c.skip(1);
        auto pad = [&](size_t n) { return ver == 1 ? (n + 7) & ~size_t(7) : n; };
        Attribute a;
        c.need(ns);
        a.name.assign(reinterpret_cast<const char*>(c.p), strnlen(reinterpret_cast<const char*>(c.p), ns));
        c.skip(pad(ns));
        c.need(ts);
        Cur tc { c.p, c.p + ts };
        a.type = parseType(tc);
        c.skip(pad(ts));
        c.need(ss);
        Cur sc { c.p, c.p + ss };
        parseSpace(sc, a.dims, nullptr);
        c.skip(pad(ss));
        const uint64_t n = bytesOf(product(a.dims), a.type.size);
        c.need(n);
        a.raw.assign(c.p, c.p + n);
        o.attrs.push_back(std::move(a));
        break;
    }
    case 0x10: { // continuation: address, then length
        const uint64_t a = c.u64();
        const uint64_t n = c.u64();
        conts.emplace_back(a, n);
        break;
    }
    case 0x11:
        throw Unsupported("old-style (symbol table) HDF5 group");
    default:
        break;
    }
}

// Links of a group in dense storage: the name index (version 2 B-tree of
// type 5 records: name hash, heap ID) into the fractal heap that holds the
// link messages.  Heap blocks are followed from the root (a direct block,
// or an indirect block's direct rows).
void File::readDenseLinks(Object& o, uint64_t heapAddr, uint64_t btreeAddr)
{
    Cur h { span(heapAddr, 4), base_ + size_ };
    if (std::memcmp(h.p, "FRHP", 4) != 0)
        throw FormatError("bad fractal heap signature");
    h.skip(4);
    h.u8();
    const unsigned idLen = h.u16();
    const unsigned filterLen = h.u16();
    const int hflags = h.u8();
    const uint32_t maxManaged = h.u32();
    h.skip(8 * 12);
    const unsigned width = h.u16();
    const uint64_t startBlock = h.u64();
    const uint64_t maxDirect = h.u64();
    const unsigned maxHeapBits = h.u16();
    h.u16(); // starting rows
    const uint64_t rootAddr = h.u64();
    const unsigned curRows = h.u16();
    if (filterLen)
        throw Unsupported("filtered fractal heap");
    if (width == 0 || startBlock == 0 || maxDirect < startBlock || maxHeapBits == 0 || maxHeapBits > 64)
        throw FormatError("bad fractal heap header");
    const size_t offBytes = (maxHeapBits + 7) / 8;
    const size_t lenBytes = std::min<size_t>((log2u(maxDirect) + 7) / 8, log2u(maxManaged) / 8 + 1);
    const int maxDirectRows = log2u(maxDirect) - log2u(startBlock) + 2;

    // the heap object at heap offset off (length len)
    auto heapBytes = [&](uint64_t off, uint64_t len) -> const uint8_t* {
        uint64_t blockAddr = kUndef, blockOff = 0, blockSize = startBlock;
        if (curRows == 0) {
            blockAddr = rootAddr;
        } else {
            Cur ib { span(rootAddr, 5 + 8 + offBytes), base_ + size_ };
            if (std::memcmp(ib.p, "FHIB", 4) != 0)
                throw FormatError("bad fractal heap indirect block");
            ib.skip(5 + 8 + offBytes);
            uint64_t bo = 0;
            for (unsigned r = 0; r < curRows && blockAddr == kUndef; ++r) {
                const uint64_t rs = r == 0 ? startBlock : startBlock << (r - 1);
                for (unsigned col = 0; col < width; ++col) {
                    if (static_cast<int>(r) >= maxDirectRows)
                        throw Unsupported("fractal heap deeper than one indirect block");
                    const uint64_t a = ib.u64();
                    if (off >= bo && off < bo + rs) {
                        blockAddr = a;
                        blockOff = bo;
                        blockSize = rs;
                        break;
                    }
                    bo += rs;
                }
            }
        }
        if (blockAddr == kUndef || off - blockOff + len > blockSize || blockSize < 5 + 8 + offBytes + 4)
            throw FormatError("fractal heap object outside its block");
        const uint8_t* b = span(blockAddr, blockSize);
        if (std::memcmp(b, "FHDB", 4) != 0 || le(b + 5 + 8, offBytes) != blockOff)
            throw FormatError("bad fractal heap direct block");
        (void)hflags;
        return b + (off - blockOff);
    };

    // node sizes of the version 2 B-tree, as its header defines them
    Cur bt { span(btreeAddr, 4), base_ + size_ };
    if (std::memcmp(bt.p, "BTHD", 4) != 0)
        throw FormatError("bad version 2 B-tree header");
    bt.skip(4);
    bt.u8();
    if (bt.u8() != 5)
        throw Unsupported("link name index of unexpected B-tree type");
    const uint32_t nodeSize = bt.u32();
    const unsigned recSize = bt.u16();
    const unsigned depth = bt.u16();
    bt.skip(2);
    const uint64_t root = bt.u64();
    const unsigned rootRecs = bt.u16();
    if (recSize != 4 + idLen || nodeSize < 10 + recSize || depth > 16)
        throw FormatError("bad version 2 B-tree header");
    struct Level {
        uint64_t maxNrec, cumMax;
        int cumSize;
    };
    std::vector<Level> lv(depth + 1);
    lv[0] = { (nodeSize - 10) / recSize, (nodeSize - 10) / recSize, 0 };
    const int maxNrecSize = log2u(lv[0].maxNrec) / 8 + 1;
    for (unsigned u = 1; u <= depth; ++u) {
        const uint64_t ptr = 8 + maxNrecSize + (u > 1 ? lv[u - 1].cumSize : 0);
        if (nodeSize < 10 + 2 * ptr + recSize)
            throw FormatError("version 2 B-tree nodes too small for their depth");
        lv[u].maxNrec = (nodeSize - (10 + ptr)) / (recSize + ptr);
        lv[u].cumMax = (lv[u].maxNrec + 1) * lv[u - 1].cumMax + lv[u].maxNrec;
        lv[u].cumSize = log2u(lv[u].cumMax) / 8 + 1;
    }
    std::vector<std::pair<uint64_t, std::pair<std::string, uint64_t>>> found; // creation order, link
    auto record = [&](const uint8_t* r) {
        const uint8_t* id = r + 4;
        if ((id[0] >> 4) & 3)
            throw Unsupported("huge or tiny link objects in a fractal heap");
        const uint64_t off = le(id + 1, offBytes), len = le(id + 1 + offBytes, lenBytes);
        Object tmp;
        std::vector<uint64_t> d;
        std::vector<std::pair<uint64_t, uint64_t>> cs;
        const uint8_t* m = heapBytes(off, len);
        parseMessage(tmp, 0x06, m, len, d, cs);
        // creation order, when the link message carries one
        uint64_t order = found.size();
        if (m[1] & 0x04)
            order = le(m + 2 + ((m[1] & 0x08) ? 1 : 0), 8);
        for (auto& l : tmp.links)
            found.push_back({ order, l });
    };
    std::set<uint64_t> seen;
    std::function<void(uint64_t, unsigned, unsigned)> walk = [&](uint64_t a, unsigned nrec, unsigned d) {
        if (!seen.insert(a).second)
            throw FormatError("version 2 B-tree node visited twice");
        const uint8_t* n = span(a, nodeSize);
        if (std::memcmp(n, d == 0 ? "BTLF" : "BTIN", 4) != 0)
            throw FormatError("bad version 2 B-tree node");
        if (nrec > lv[d].maxNrec)
            throw FormatError("version 2 B-tree node overfull");
        const uint8_t* r = n + 6;
        for (unsigned i = 0; i < nrec; ++i)
            record(r + size_t(i) * recSize);
        if (d == 0)
            return;
        Cur c { r + size_t(nrec) * recSize, n + nodeSize };
        for (unsigned i = 0; i <= nrec; ++i) {
            const uint64_t ca = c.u64();
            const unsigned cn = static_cast<unsigned>(c.u(maxNrecSize));
            if (d > 1)
                c.skip(lv[d - 1].cumSize);
            walk(ca, cn, d - 1);
        }
    };
    if (root != kUndef && rootRecs)
        walk(root, rootRecs, depth);
    std::stable_sort(found.begin(), found.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    for (auto& f : found)
        o.links.push_back(f.second);
}

// object `index` of the global heap collection at `collection`
std::vector<uint8_t> File::heapObject(uint64_t collection, uint32_t index)
{
    const uint8_t* g = span(collection, 16);
    if (std::memcmp(g, "GCOL", 4) != 0)
        throw FormatError("bad global heap collection");
    const uint64_t csize = le(g + 8, 8);
    if (csize < 16)
        throw FormatError("bad global heap collection size");
    Cur c { span(collection, csize) + 16, span(collection, csize) + csize };
    while (c.left() >= 16) {
        const unsigned idx = c.u16();
        c.skip(6);
        const uint64_t sz = c.u64();
        if (idx == 0)
            break;
        c.need(sz);
        if (idx == index)
            return std::vector<uint8_t>(c.p, c.p + sz);
        c.skip(std::min<uint64_t>(c.left(), (sz + 7) & ~uint64_t(7)));
    }
    throw FormatError("global heap object not found");
}

// elements [first, first + count) of the dataset's row-major order, as
// stored bytes (unwritten parts hold the fill value); a chunked dataset
// copies only the chunk rows that overlap the window
void File::readRaw(const Object& o, uint8_t* out, uint64_t first, uint64_t count)
{
    if (!o.isDataset)
        throw std::invalid_argument("not a dataset");
    if (o.hasFilters)
        throw Unsupported("filtered (compressed) variables");
    const uint64_t es = o.type.size;
    const uint64_t n = product(o.dims);
    if (first > n || count > n - first)
        throw std::out_of_range("read beyond the variable");
    if (count > (size_ + (uint64_t(1) << 30)) / std::max<uint64_t>(es, 1))
        throw FormatError("dataset larger than its file allows");
    const uint64_t total = count * es;
    std::memset(out, 0, total);
    if (o.fill.size() == es && es > 0 && o.layoutClass == 2)
        for (uint64_t i = 0; i < total; i += es)
            std::memcpy(out + i, o.fill.data(), es);
    if (o.layoutClass == 0) {
        if (o.compact.size() < bytesOf(first + count, es))
            throw FormatError("compact dataset shorter than its dataspace");
        std::memcpy(out, o.compact.data() + first * es, total);
    } else if (o.layoutClass == 1) {
        if (o.dataAddr != kUndef)
            std::memcpy(out, span(o.dataAddr, bytesOf(n, es)) + first * es, total);
        else if (o.fill.size() == es && es > 0)
            for (uint64_t i = 0; i < total; i += es)
                std::memcpy(out + i, o.fill.data(), es);
    } else {
        if (o.chunk.size() != o.dims.size() + 1 || o.chunk.back() != es)
            throw FormatError("chunk dimensions do not match the dataspace");
        for (size_t i = 0; i + 1 < o.chunk.size(); ++i)
            if (o.chunk[i] == 0)
                throw FormatError("zero chunk dimension");
        if (o.dataAddr != kUndef) {
            std::set<uint64_t> seen;
            chunkWalk(o, o.dataAddr, 0, out, first, count, seen);
        }
    }
}

// version 1 B-tree of raw-data chunks: "TREE", type 1, level, entries,
// siblings, then keys (chunk size, filter mask, offsets) and child addresses
void File::chunkWalk(const Object& o, uint64_t node, int depth, uint8_t* out, uint64_t first,
    uint64_t count, std::set<uint64_t>& seen)
{
    if (depth > 32)
        throw FormatError("chunk B-tree too deep");
    if (!seen.insert(node).second)
        throw FormatError("chunk B-tree node visited twice");
    const size_t rank = o.dims.size();
    const size_t keySize = 8 + 8 * (rank + 1);
    Cur c { span(node, 24), base_ + size_ };
    if (std::memcmp(c.p, "TREE", 4) != 0 || c.p[4] != 1)
        throw FormatError("bad chunk B-tree node");
    c.skip(5);
    const int level = c.u8();
    const unsigned entries = c.u16();
    c.skip(16);
    c.need(entries * (keySize + 8) + keySize);
    const uint64_t es = o.type.size;
    std::vector<uint64_t> chunkDims(o.chunk.begin(), o.chunk.end() - 1);
    const uint64_t chunkBytes = bytesOf(product(chunkDims), es);
    for (unsigned e = 0; e < entries; ++e) {
        const uint32_t csize = c.u32();
        c.skip(4);
        std::vector<uint64_t> off(rank);
        for (size_t d = 0; d < rank; ++d)
            off[d] = c.u64();
        c.skip(8);
        const uint64_t child = c.u64();
        if (level > 0) {
            chunkWalk(o, child, depth + 1, out, first, count, seen);
            continue;
        }
        if (csize != chunkBytes)
            throw FormatError("chunk of unexpected size");
        bool inside = rank > 0;
        for (size_t d = 0; d < rank; ++d)
            inside = inside && off[d] < o.dims[d];
        if (!inside)
            continue;
        // the chunk's flat index range; skip chunks outside the window
        uint64_t lo0 = 0, hi0 = 0;
        for (size_t d = 0; d < rank; ++d) {
            lo0 = lo0 * o.dims[d] + off[d];
            hi0 = hi0 * o.dims[d] + std::min<uint64_t>(off[d] + chunkDims[d], o.dims[d]) - 1;
        }
        if (hi0 + 1 <= first || lo0 >= first + count)
            continue;
        const uint8_t* src = span(child, chunkBytes);
        // a chunk spanning every dimension but the first (one record of a
        // forcing or diagnostic file) is one contiguous run
        bool whole = true;
        for (size_t d = 1; d < rank; ++d)
            whole = whole && off[d] == 0 && chunkDims[d] == o.dims[d];
        if (whole) {
            const uint64_t lo = std::max(lo0, first), hi = std::min(hi0 + 1, first + count);
            std::memcpy(out + (lo - first) * es, src + (lo - lo0) * es, (hi - lo) * es);
            continue;
        }
        // otherwise copy the chunk's rows (fastest dimension) in the window
        const uint64_t rowLen = std::min<uint64_t>(chunkDims[rank - 1], o.dims[rank - 1] - off[rank - 1]);
        std::vector<uint64_t> k(rank, 0);
        for (bool more = true; more;) {
            bool ok = true;
            uint64_t dst = 0, srcIdx = 0;
            for (size_t d = 0; d < rank; ++d) {
                ok = ok && off[d] + k[d] < o.dims[d];
                dst = dst * o.dims[d] + off[d] + k[d];
                srcIdx = srcIdx * chunkDims[d] + k[d];
            }
            if (ok) {
                const uint64_t lo = std::max(dst, first), hi = std::min(dst + rowLen, first + count);
                if (lo < hi)
                    std::memcpy(out + (lo - first) * es, src + (srcIdx + lo - dst) * es, (hi - lo) * es);
            }
            // next row: increment the chunk index over all but the last dimension
            more = false;
            for (size_t d = rank - 1; d-- > 0;) {
                if (++k[d] < chunkDims[d]) {
                    more = true;
                    break;
                }
                k[d] = 0;
            }
        }
    }
}

void File::readDoubles(const Object& o, uint64_t first, uint64_t count, double* out)
{
    const uint64_t n = product(o.dims);
    if (first > n || count > n - first)
        throw std::out_of_range("read beyond the variable");
    if (o.type.cls != TypeClass::Float && o.type.cls != TypeClass::Fixed)
        throw Unsupported("variable is not numeric");
    const uint64_t es = o.type.size;
    // little-endian FP64 is stored as the caller wants it: no conversion
    if (o.type.cls == TypeClass::Float && es == 8 && !o.type.bigEndian) {
        readRaw(o, reinterpret_cast<uint8_t*>(out), first, count);
        return;
    }
    if (count > (size_ + (uint64_t(1) << 30)) / std::max<uint64_t>(es, 1))
        throw FormatError("dataset larger than its file allows");
    std::vector<uint8_t> raw(count * es);
    readRaw(o, raw.data(), first, count);
    for (uint64_t i = 0; i < count; ++i)
        out[i] = toDouble(o.type, raw.data() + i * es);
}

std::vector<double> File::readDoubles(const Object& o)
{
    std::vector<double> v(product(o.dims));
    readDoubles(o, 0, v.size(), v.data());
    return v;
}

namespace {
std::string fixedText(const uint8_t* p, size_t n)
{
    size_t k = 0;
    while (k < n && p[k])
        ++k;
    return std::string(reinterpret_cast<const char*>(p), k);
}
} // namespace

std::string File::attrText(const Attribute& a)
{
    if (a.type.cls == TypeClass::String)
        return fixedText(a.raw.data(), a.raw.size());
    if (a.type.cls == TypeClass::VarLen && a.type.vlenString && a.raw.size() >= 16) {
        const uint32_t len = static_cast<uint32_t>(le(a.raw.data(), 4));
        if (len == 0)
            return std::string();
        const auto b = heapObject(le(a.raw.data() + 4, 8), static_cast<uint32_t>(le(a.raw.data() + 12, 4)));
        return fixedText(b.data(), std::min<size_t>(len, b.size()));
    }
    throw Unsupported("attribute " + a.name + " is not text");
}

double File::attrDouble(const Attribute& a, size_t i)
{
    if ((a.type.cls != TypeClass::Float && a.type.cls != TypeClass::Fixed) || (i + 1) * a.type.size > a.raw.size())
        throw Unsupported("attribute " + a.name + " is not numeric");
    return toDouble(a.type, a.raw.data() + i * a.type.size);
}

std::string File::readText(const Object& o)
{
    std::vector<uint8_t> raw;
    if (o.type.cls != TypeClass::String && !(o.type.cls == TypeClass::VarLen && o.type.vlenString))
        throw Unsupported("variable is not text");
    const uint64_t n = product(o.dims);
    if (n > (size_ + (uint64_t(1) << 30)) / std::max<uint64_t>(o.type.size, 1))
        throw FormatError("dataset larger than its file allows");
    raw.resize(n * o.type.size);
    readRaw(o, raw.data(), 0, n);
    Attribute a;
    a.type = o.type;
    a.raw = raw;
    return attrText(a);
}

// ------------------------------------------------------------ navigation
namespace {
std::vector<std::string> splitPath(const std::string& path)
{
    std::vector<std::string> parts;
    size_t i = 0;
    while (i <= path.size()) {
        const size_t j = path.find('/', i);
        const std::string s = path.substr(i, j == std::string::npos ? std::string::npos : j - i);
        if (!s.empty())
            parts.push_back(s);
        if (j == std::string::npos)
            break;
        i = j + 1;
    }
    return parts;
}

const char* const kDimOnly = "This is a netCDF dimension but not a netCDF variable";
} // namespace

const Object& File::at(const std::string& path)
{
    const Object* o = &object(rootAddr_);
    for (const auto& part : splitPath(path)) {
        const Object* next = nullptr;
        for (const auto& l : o->links)
            if (l.first == part) {
                next = &object(l.second);
                break;
            }
        if (!next)
            throw std::out_of_range("no " + path + " in the file");
        o = next;
    }
    return *o;
}

bool File::exists(const std::string& path)
{
    try {
        at(path);
        return true;
    } catch (const std::out_of_range&) {
        return false;
    }
}

std::vector<std::string> File::groups(const std::string& group)
{
    std::vector<std::string> g;
    for (const auto& l : at(group).links)
        if (!object(l.second).isDataset)
            g.push_back(l.first);
    return g;
}

// netCDF dimension names of a dataset: the dimension scales DIMENSION_LIST
// refers to (looked up in the group and its ancestors), or the dataset
// itself for a coordinate variable
std::vector<std::string> File::dimNames(const Object& o, const std::string& group)
{
    std::vector<std::string> names(o.dims.size());
    const Attribute* dl = o.attr("DIMENSION_LIST");
    std::vector<std::string> chain { "" };
    std::string acc;
    for (const auto& part : splitPath(group)) {
        acc += (acc.empty() ? "" : "/") + part;
        chain.push_back(acc);
    }
    auto nameOf = [&](uint64_t addr) -> std::string {
        for (auto it = chain.rbegin(); it != chain.rend(); ++it)
            for (const auto& l : at(*it).links)
                if (l.second == addr)
                    return l.first;
        return std::string();
    };
    if (dl && dl->type.cls == TypeClass::VarLen && dl->raw.size() >= 16 * names.size()) {
        for (size_t i = 0; i < names.size(); ++i) {
            const uint8_t* e = dl->raw.data() + 16 * i;
            if (le(e, 4) == 0)
                continue;
            const auto refs = heapObject(le(e + 4, 8), static_cast<uint32_t>(le(e + 12, 4)));
            if (refs.size() >= 8)
                names[i] = nameOf(le(refs.data(), 8));
        }
    } else if (names.size() == 1) {
        const Attribute* cls = o.attr("CLASS");
        if (cls && attrText(*cls) == "DIMENSION_SCALE")
            names[0] = nameOf(o.addr);
    }
    for (size_t i = 0; i < names.size(); ++i)
        if (names[i].empty())
            names[i] = "phony_dim_" + std::to_string(i);
    return names;
}

std::vector<Variable> File::variables(const std::string& group)
{
    std::vector<Variable> vars;
    std::string g;
    for (const auto& part : splitPath(group))
        g += (g.empty() ? "" : "/") + part;
    for (const auto& l : at(g).links) {
        const Object& o = object(l.second);
        if (!o.isDataset)
            continue;
        const Attribute* nm = o.attr("NAME");
        if (nm && nm->type.cls == TypeClass::String && attrText(*nm).rfind(kDimOnly, 0) == 0)
            continue;
        Variable v;
        v.name = l.first;
        v.path = g.empty() ? l.first : g + "/" + l.first;
        v.dims = o.dims;
        v.dimNames = dimNames(o, g);
        v.obj = &o;
        vars.push_back(std::move(v));
    }
    return vars;
}

Variable File::variable(const std::string& path)
{
    auto parts = splitPath(path);
    if (parts.empty())
        throw std::out_of_range("empty variable path");
    const std::string name = parts.back();
    parts.pop_back();
    std::string g;
    for (const auto& p : parts)
        g += (g.empty() ? "" : "/") + p;
    for (auto& v : variables(g))
        if (v.name == name)
            return v;
    throw std::out_of_range("no variable " + path + " in the file");
}

} // namespace nsdg_nc
