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
// Record variables (the diagnostic files of writeDiagnosticTime) are chunked
// along the unlimited time axis, one chunk per record, with a version 1
// B-tree chunk index.  Dimension scales carry no REFERENCE_LIST
// back-references, and link and attribute creation order is not tracked:
// netCDF-C then lists them by name.  The file is built in memory (records
// included) and written in one pass when it is saved.
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
    // record variables: chunked along an unlimited first dimension, one
    // chunk per record, indexed by a version 1 B-tree
    bool chunked = false;
    std::vector<std::vector<uint8_t>> records;
    std::vector<uint64_t> recordAddrs;
    uint64_t btreeAddr = kUndef;
};

namespace {
constexpr uint64_t kUnlimited = UINT64_MAX;
constexpr unsigned kBtreeK = 32; // HDF5's default for chunk B-trees: at most 2K entries a node
} // namespace

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

int Writer::addTimeAxis(int group, const std::string& name, int dimid)
{
    const int id = addGroup(group, name);
    Node& n = nodes_[id];
    n.group = false;
    n.chunked = true;
    n.type = typeF64();
    n.dims = { 0 };
    attrText(id, "CLASS", "DIMENSION_SCALE");
    attrText(id, "NAME", name);
    attrInt(id, "_Netcdf4Dimid", dimid);
    return id;
}

int Writer::addRecordDouble(int group, const std::string& name, const std::vector<int>& dims)
{
    if (dims.empty() || !nodes_.at(dims[0]).chunked)
        throw std::invalid_argument("a record variable's first dimension is the time axis");
    const int id = addGroup(group, name);
    Node& n = nodes_[id];
    n.group = false;
    n.chunked = true;
    n.type = typeF64();
    n.dims.push_back(0);
    for (size_t i = 1; i < dims.size(); ++i)
        n.dims.push_back(nodes_.at(dims[i]).dims.at(0));
    n.dimRefs = dims;
    const double fill = 9.9692099683868690e+36;
    uint64_t u;
    std::memcpy(&u, &fill, 8);
    put(n.fill, u, 8);
    return id;
}

void Writer::appendRecord(int var, const double* data)
{
    Node& n = nodes_.at(var);
    if (!n.chunked)
        throw std::invalid_argument("not a record variable");
    uint64_t count = 1;
    for (size_t i = 1; i < n.dims.size(); ++i)
        count *= n.dims[i];
    std::vector<uint8_t> r(8 * count);
    if (count)
        std::memcpy(r.data(), data, r.size());
    n.records.push_back(std::move(r));
    n.dims[0] = n.records.size();
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
        if (n.chunked) {
            std::vector<uint8_t> sp { 2, static_cast<uint8_t>(n.dims.size()), 1, 1 };
            for (uint64_t d : n.dims)
                put(sp, d, 8);
            for (size_t i = 0; i < n.dims.size(); ++i)
                put(sp, i == 0 ? kUnlimited : n.dims[i], 8);
            msg(0x01, sp, 0);
        } else {
            msg(0x01, space(n.dims), 0);
        }
        msg(0x03, n.type, 0x01);
        // fill value: allocation early (written data) or late (scales),
        // written if set, the value when defined
        std::vector<uint8_t> fv { 3, static_cast<uint8_t>(n.fill.empty() ? 0x0A : 0x29) };
        if (!n.fill.empty()) {
            put(fv, n.fill.size(), 4);
            fv.insert(fv.end(), n.fill.begin(), n.fill.end());
        }
        msg(0x05, fv, 0);
        if (n.chunked) { // chunk = one record; the last chunk dimension is the element size
            std::vector<uint8_t> lay { 3, 2, static_cast<uint8_t>(n.dims.size() + 1) };
            put(lay, n.btreeAddr, 8);
            for (size_t i = 0; i < n.dims.size(); ++i)
                put(lay, i == 0 ? 1 : n.dims[i], 4);
            put(lay, 8, 4);
            msg(0x08, lay, 0);
        } else {
            std::vector<uint8_t> lay { 3, 1 }; // contiguous
            put(lay, n.dataAddr, 8);
            put(lay, n.storageSize, 8);
            msg(0x08, lay, 0);
        }
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
    return encode(true);
}

// The metadata (superblock, global heap, object headers, chunk B-trees)
// followed, when withData, by the contiguous data and the records at the
// addresses the headers give them (all data lies after the metadata).
std::vector<uint8_t> Writer::encode(bool withData)
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
    // chunk B-trees of the record variables: leaves of at most 2K chunks,
    // then parent levels of at most 2K children, root last
    std::vector<std::vector<std::vector<uint64_t>>> levels(nodes_.size()); // [node][level][i] address
    auto nodeSize = [](size_t rank) { return 24 + 2 * kBtreeK * 8 + (2 * kBtreeK + 1) * (8 + 8 * (rank + 1)); };
    for (size_t i = 0; i < nodes_.size(); ++i) {
        Node& n = nodes_[i];
        if (!n.chunked || n.records.empty())
            continue;
        size_t count = n.records.size();
        do {
            count = (count + 2 * kBtreeK - 1) / (2 * kBtreeK);
            levels[i].emplace_back();
            for (size_t k = 0; k < count; ++k) {
                levels[i].back().push_back(pos);
                pos += nodeSize(n.dims.size());
            }
        } while (count > 1);
        n.btreeAddr = levels[i].back().at(0);
    }
    for (auto& n : nodes_) {
        if (n.group || n.data.empty())
            continue;
        pos = (pos + 7) & ~uint64_t(7);
        n.dataAddr = pos;
        pos += n.data.size();
    }
    for (auto& n : nodes_) {
        n.recordAddrs.clear();
        for (const auto& r : n.records) {
            pos = (pos + 7) & ~uint64_t(7);
            n.recordAddrs.push_back(pos);
            pos += r.size();
        }
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
    // B-tree nodes: a key is (chunk bytes, filter mask, chunk offset in
    // every dimension and 0 for the element); a node's last key bounds its
    // last chunk (offset plus the chunk extent)
    for (size_t i = 0; i < nodes_.size(); ++i) {
        const Node& n = nodes_[i];
        const size_t rank = n.dims.size();
        const uint64_t csize = n.records.empty() ? 0 : n.records[0].size();
        auto key = [&](std::vector<uint8_t>& b, uint64_t rec, bool upper) {
            put(b, upper ? 0 : csize, 4);
            put(b, 0, 4);
            put(b, upper ? rec + 1 : rec, 8);
            for (size_t d = 1; d < rank; ++d)
                put(b, upper ? n.dims[d] : 0, 8);
            put(b, 0, 8);
        };
        uint64_t span = 1; // records under one entry at this level
        for (size_t lv = 0; lv < levels[i].size(); ++lv) {
            const auto& addrs = levels[i][lv];
            const uint64_t per = span * 2 * kBtreeK;
            for (size_t k = 0; k < addrs.size(); ++k) {
                const uint64_t first = k * per;
                const uint64_t last = std::min<uint64_t>(first + per, n.records.size());
                const uint64_t entries = (last - first + span - 1) / span;
                std::vector<uint8_t> b { 'T', 'R', 'E', 'E', 1, static_cast<uint8_t>(lv) };
                put(b, entries, 2);
                put(b, k ? addrs[k - 1] : kUndef, 8);
                put(b, k + 1 < addrs.size() ? addrs[k + 1] : kUndef, 8);
                for (uint64_t e = 0; e < entries; ++e) {
                    const uint64_t rec = first + e * span;
                    key(b, rec, false);
                    put(b, lv == 0 ? n.recordAddrs[rec] : levels[i][lv - 1][rec / span], 8);
                }
                key(b, last - 1, true);
                b.resize(nodeSize(rank), 0);
                if (f.size() != addrs[k])
                    throw std::logic_error("B-tree node placed out of order");
                f.insert(f.end(), b.begin(), b.end());
            }
            span = per;
        }
    }
    if (!withData)
        return f;
    for (const auto& n : nodes_) {
        if (n.group || n.data.empty())
            continue;
        f.resize(n.dataAddr, 0);
        f.insert(f.end(), n.data.begin(), n.data.end());
    }
    for (const auto& n : nodes_)
        for (size_t r = 0; r < n.records.size(); ++r) {
            f.resize(n.recordAddrs[r], 0);
            f.insert(f.end(), n.records[r].begin(), n.records[r].end());
        }
    return f;
}

// Writes to path + ".tmp" and renames it over path once every byte has been
// written and the stream closed without error, so that a failed dump (disk
// full, quota) leaves the previous file at path intact.
void Writer::save(const std::string& path)
{
    const auto meta = encode(false);
    const std::string tmp = path + ".tmp";
    std::ofstream out(tmp, std::ios::binary | std::ios::trunc);
    if (!out)
        throw std::runtime_error("cannot create " + tmp);
    uint64_t pos = 0;
    auto block = [&](uint64_t addr, const std::vector<uint8_t>& b) {
        static const char zeros[8] = {};
        if (addr < pos || addr - pos > 8)
            throw std::logic_error("data block out of order");
        out.write(zeros, static_cast<std::streamsize>(addr - pos));
        out.write(reinterpret_cast<const char*>(b.data()), static_cast<std::streamsize>(b.size()));
        pos = addr + b.size();
    };
    out.write(reinterpret_cast<const char*>(meta.data()), static_cast<std::streamsize>(meta.size()));
    pos = meta.size();
    for (const auto& n : nodes_)
        if (!n.group && !n.data.empty())
            block(n.dataAddr, n.data);
    for (const auto& n : nodes_)
        for (size_t r = 0; r < n.records.size(); ++r)
            block(n.recordAddrs[r], n.records[r]);
    out.close(); // the final flush can fail too
    if (!out) {
        std::remove(tmp.c_str());
        throw std::runtime_error("cannot write " + path);
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        throw std::runtime_error("cannot rename " + tmp + " to " + path);
    }
}

} // namespace nsdg_nc
