// Writer of restart files in ParaGridIO's NetCDF-4 layout
// (ParaGridIO::dumpModelState, core/src/ParaGridIO.cpp:272-348, with the
// groups of CommonRestartMetadata, core/src/CommonRestartMetadata.cpp:18-72).
//
// The file is the HDF5 subset nsdg_restart.cpp reads, written the simple way:
// version 2 superblock, version 2 object headers holding everything in one
// chunk, groups with compact link storage (link info, group info and link
// messages), contiguous datasets, version 3 attribute messages, and netCDF-4
// dimensions as dimension scales (CLASS, NAME, _Netcdf4Dimid on the scale;
// DIMENSION_LIST on each variable, through one global heap collection).
// Dimension scales carry no REFERENCE_LIST back-references, and link and
// attribute creation order is not tracked: netCDF-C then lists them by
// name.  The file is built in memory and written in one pass.
#include "nsdg_restart.hpp"

#include <cstdio>
#include <cstring>
#include <fstream>

namespace nsdg_nc {

namespace {

constexpr uint64_t kUndef = UINT64_MAX;

void put(std::vector<uint8_t>& b, uint64_t v, int n)
{
    for (int i = 0; i < n; ++i)
        b.push_back(static_cast<uint8_t>(v >> (8 * i)));
}

// datatype messages (class and version byte, three bit-field bytes, size, properties)
std::vector<uint8_t> typeF64()
{
    std::vector<uint8_t> t { 0x11, 0x20, 63, 0 };
    put(t, 8, 4);
    put(t, 0, 2);
    put(t, 64, 2);
    t.insert(t.end(), { 52, 11, 0, 52 });
    put(t, 1023, 4);
    return t;
}
std::vector<uint8_t> typeF32BE()
{
    std::vector<uint8_t> t { 0x11, 0x21, 31, 0 };
    put(t, 4, 4);
    put(t, 0, 2);
    put(t, 32, 2);
    t.insert(t.end(), { 23, 8, 0, 23 });
    put(t, 127, 4);
    return t;
}
std::vector<uint8_t> typeInt(int bytes)
{
    std::vector<uint8_t> t { 0x10, 0x08, 0, 0 };
    put(t, bytes, 4);
    put(t, 0, 2);
    put(t, 8 * bytes, 2);
    return t;
}
std::vector<uint8_t> typeText(size_t n)
{
    std::vector<uint8_t> t { 0x13, 0x00, 0, 0 }; // NUL-terminated ASCII
    put(t, n, 4);
    return t;
}
std::vector<uint8_t> typeRefList()
{
    std::vector<uint8_t> t { 0x19, 0x00, 0, 0 }; // variable-length sequence
    put(t, 16, 4);
    std::vector<uint8_t> r { 0x17, 0x00, 0, 0 }; // object reference
    put(r, 8, 4);
    t.insert(t.end(), r.begin(), r.end());
    return t;
}
std::vector<uint8_t> space(const std::vector<uint64_t>& dims)
{
    std::vector<uint8_t> s { 2, static_cast<uint8_t>(dims.size()), 0, static_cast<uint8_t>(dims.empty() ? 0 : 1) };
    for (uint64_t d : dims)
        put(s, d, 8);
    return s;
}

} // namespace

// ------------------------------------------------------------------ model
struct Writer::Attr {
    std::string name;
    std::vector<uint8_t> type, space, data;
};

struct Writer::Node {
    std::string name;
    bool group = true;
    std::vector<int> children;
    std::vector<Attr> attrs;
    std::vector<uint8_t> type;
    std::vector<uint64_t> dims;
    std::vector<uint8_t> data;   // empty: never written (dimension-only scale)
    uint64_t storageSize = 0;
    std::vector<int> dimRefs;    // dimension scales of a variable
    std::vector<uint8_t> fill;
    uint64_t addr = 0, dataAddr = kUndef;
    uint32_t heapFirst = 0;      // first global heap index of its DIMENSION_LIST
};

Writer::Writer() { nodes_.emplace_back(); }
Writer::~Writer() = default;

int Writer::addGroup(int parent, const std::string& name)
{
    Node n;
    n.name = name;
    nodes_.push_back(std::move(n));
    nodes_.at(parent).children.push_back(static_cast<int>(nodes_.size() - 1));
    return static_cast<int>(nodes_.size() - 1);
}

void Writer::attrText(int node, const std::string& name, const std::string& value)
{
    Attr a { name, typeText(value.size() + 1), space({}), {} };
    a.data.assign(value.begin(), value.end());
    a.data.push_back(0);
    nodes_.at(node).attrs.push_back(std::move(a));
}

void Writer::attrDouble(int node, const std::string& name, double v)
{
    Attr a { name, typeF64(), space({}), {} };
    uint64_t u;
    std::memcpy(&u, &v, 8);
    put(a.data, u, 8);
    nodes_.at(node).attrs.push_back(std::move(a));
}

void Writer::attrInt(int node, const std::string& name, int32_t v)
{
    Attr a { name, typeInt(4), space({}), {} };
    put(a.data, static_cast<uint32_t>(v), 4);
    nodes_.at(node).attrs.push_back(std::move(a));
}

int Writer::addDimension(int group, const std::string& name, uint64_t length, int dimid)
{
    const int id = addGroup(group, name);
    Node& n = nodes_[id];
    n.group = false;
    n.type = typeF32BE();
    n.dims = { length };
    n.storageSize = 4 * length;
    attrText(id, "CLASS", "DIMENSION_SCALE");
    char nm[128];
    std::snprintf(nm, sizeof nm, "This is a netCDF dimension but not a netCDF variable.%10llu",
        static_cast<unsigned long long>(length));
    attrText(id, "NAME", nm);
    attrInt(id, "_Netcdf4Dimid", dimid);
    return id;
}

int Writer::addDouble(int group, const std::string& name, const std::vector<int>& dims, const double* data)
{
    const int id = addGroup(group, name);
    Node& n = nodes_[id];
    n.group = false;
    n.type = typeF64();
    uint64_t count = 1;
    for (int d : dims) {
        n.dims.push_back(nodes_.at(d).dims.at(0));
        count *= n.dims.back();
    }
    n.dimRefs = dims;
    n.data.resize(8 * count);
    if (count)
        std::memcpy(n.data.data(), data, n.data.size());
    n.storageSize = n.data.size();
    const double fill = 9.9692099683868690e+36; // netCDF's default fill for doubles
    uint64_t u;
    std::memcpy(&u, &fill, 8);
    put(n.fill, u, 8);
    return id;
}

int Writer::addInt64(int group, const std::string& name, int64_t value)
{
    const int id = addGroup(group, name);
    Node& n = nodes_[id];
    n.group = false;
    n.type = typeInt(8);
    put(n.data, static_cast<uint64_t>(value), 8);
    n.storageSize = 8;
    return id;
}

// ------------------------------------------------------------ encoding
std::vector<uint8_t> Writer::header(const Node& n, uint64_t heapAddr) const
{
    std::vector<uint8_t> m;
    auto msg = [&](int type, const std::vector<uint8_t>& d, int flags) {
        if (d.size() > 0xffff)
            throw Unsupported("object header message over 64 KiB");
        m.push_back(static_cast<uint8_t>(type));
        put(m, d.size(), 2);
        m.push_back(static_cast<uint8_t>(flags));
        m.insert(m.end(), d.begin(), d.end());
    };
    if (n.group) {
        std::vector<uint8_t> li { 0, 0 }; // link info: no dense storage
        put(li, kUndef, 8);
        put(li, kUndef, 8);
        msg(0x02, li, 0);
        msg(0x0A, { 0, 0 }, 0); // group info: defaults
        for (int c : n.children) {
            const Node& ch = nodes_[c];
            const bool wide = ch.name.size() > 255;
            std::vector<uint8_t> l { 1, static_cast<uint8_t>(wide ? 1 : 0) };
            put(l, ch.name.size(), wide ? 2 : 1);
            l.insert(l.end(), ch.name.begin(), ch.name.end());
            put(l, ch.addr, 8);
            msg(0x06, l, 0);
        }
    } else {
        msg(0x01, space(n.dims), 0);
        msg(0x03, n.type, 0x01);
        // fill value: allocation early (written data) or late (scales),
        // written if set, the value when defined
        std::vector<uint8_t> fv { 3, static_cast<uint8_t>(n.fill.empty() ? 0x0A : 0x29) };
        if (!n.fill.empty()) {
            put(fv, n.fill.size(), 4);
            fv.insert(fv.end(), n.fill.begin(), n.fill.end());
        }
        msg(0x05, fv, 0);
        std::vector<uint8_t> lay { 3, 1 }; // contiguous
        put(lay, n.dataAddr, 8);
        put(lay, n.storageSize, 8);
        msg(0x08, lay, 0);
    }
    auto attrMsg = [&](const Attr& a) {
        std::vector<uint8_t> d { 3, 0 };
        put(d, a.name.size() + 1, 2);
        put(d, a.type.size(), 2);
        put(d, a.space.size(), 2);
        d.push_back(0); // ASCII name
        d.insert(d.end(), a.name.begin(), a.name.end());
        d.push_back(0);
        d.insert(d.end(), a.type.begin(), a.type.end());
        d.insert(d.end(), a.space.begin(), a.space.end());
        d.insert(d.end(), a.data.begin(), a.data.end());
        msg(0x0C, d, 0);
    };
    for (const auto& a : n.attrs)
        attrMsg(a);
    if (!n.dimRefs.empty()) {
        Attr dl { "DIMENSION_LIST", typeRefList(), space({ n.dimRefs.size() }), {} };
        for (size_t i = 0; i < n.dimRefs.size(); ++i) {
            put(dl.data, 1, 4);
            put(dl.data, heapAddr, 8);
            put(dl.data, n.heapFirst + i, 4);
        }
        attrMsg(dl);
    }
    std::vector<uint8_t> h { 'O', 'H', 'D', 'R', 2, 0x02 };
    put(h, m.size(), 4);
    h.insert(h.end(), m.begin(), m.end());
    put(h, lookup3(h.data(), h.size()), 4);
    return h;
}

std::vector<uint8_t> Writer::serialize()
{
    // global heap objects: one object reference per variable dimension
    uint32_t nHeap = 0;
    for (auto& n : nodes_)
        if (!n.dimRefs.empty()) {
            n.heapFirst = nHeap + 1;
            nHeap += static_cast<uint32_t>(n.dimRefs.size());
        }
    if (nHeap > 60000)
        throw Unsupported("too many variable dimensions for one global heap collection");
    const uint64_t used = 16 + 24 * uint64_t(nHeap);
    const uint64_t coll = nHeap ? std::max<uint64_t>(4096, used + 16) : 0;
    // object header sizes do not depend on addresses: size, place, encode
    std::vector<uint64_t> sizes;
    for (const auto& n : nodes_)
        sizes.push_back(header(n, 0).size());
    uint64_t pos = 48;
    const uint64_t heapAddr = nHeap ? pos : kUndef;
    pos += coll;
    for (size_t i = 0; i < nodes_.size(); ++i) {
        nodes_[i].addr = pos;
        pos += sizes[i];
    }
    for (auto& n : nodes_) {
        if (n.group || n.data.empty())
            continue;
        pos = (pos + 7) & ~uint64_t(7);
        n.dataAddr = pos;
        pos += n.data.size();
    }
    std::vector<uint8_t> f;
    f.reserve(pos);
    const uint8_t sig[8] = { 0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n' };
    f.insert(f.end(), sig, sig + 8);
    f.insert(f.end(), { 2, 8, 8, 0 });
    put(f, 0, 8);
    put(f, kUndef, 8);
    put(f, pos, 8);
    put(f, nodes_[0].addr, 8);
    put(f, lookup3(f.data(), f.size()), 4);
    if (nHeap) {
        f.insert(f.end(), { 'G', 'C', 'O', 'L', 1, 0, 0, 0 });
        put(f, coll, 8);
        for (const auto& n : nodes_)
            for (size_t i = 0; i < n.dimRefs.size(); ++i) {
                put(f, n.heapFirst + i, 2);
                put(f, 1, 2); // reference count
                put(f, 0, 4);
                put(f, 8, 8);
                put(f, nodes_[n.dimRefs[i]].addr, 8);
            }
        put(f, 0, 2); // free space to the end of the collection
        put(f, 0, 2);
        put(f, 0, 4);
        put(f, coll - used, 8);
        f.resize(heapAddr + coll, 0);
    }
    for (size_t i = 0; i < nodes_.size(); ++i) {
        const auto h = header(nodes_[i], heapAddr);
        if (h.size() != sizes[i] || f.size() != nodes_[i].addr)
            throw std::logic_error("object header size changed between passes");
        f.insert(f.end(), h.begin(), h.end());
    }
    for (const auto& n : nodes_) {
        if (n.group || n.data.empty())
            continue;
        f.resize(n.dataAddr, 0);
        f.insert(f.end(), n.data.begin(), n.data.end());
    }
    return f;
}

void Writer::save(const std::string& path)
{
    const auto bytes = serialize();
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out)
        throw std::runtime_error("cannot create " + path);
    out.write(reinterpret_cast<const char*>(bytes.data()), static_cast<std::streamsize>(bytes.size()));
    if (!out)
        throw std::runtime_error("cannot write " + path);
}

} // namespace nsdg_nc
