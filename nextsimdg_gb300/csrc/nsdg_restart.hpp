// Reader of the NetCDF-4 files neXtSIM_DG's ParaGridIO reads and writes
// (core/src/ParaGridIO.cpp:87-208 getModelState, :210-270
// readForcingTimeStatic, :272-348 dumpModelState, which writes restarts).
//
// NetCDF-4 files are HDF5 files.  This is a self-contained reader of the
// part of the HDF5 file format (the published "HDF5 File Format
// Specification", version 3) that netCDF-C and netCDF4-python produce:
//   * superblock versions 2 and 3, 8-byte offsets and lengths;
//   * version 2 object headers ("OHDR") and their continuation chunks
//     ("OCHK"), Jenkins lookup3 checksums verified;
//   * groups with link messages in the header (compact storage) or in a
//     fractal heap indexed by a version 2 B-tree (dense storage: a root
//     direct block or the direct rows of a root indirect block, enough for
//     groups of several hundred variables);
//   * datasets with contiguous, compact or chunked layout (version 3 layout
//     message, version 1 B-tree chunk index), without filters;
//   * fixed-point, floating-point, fixed-length string, variable-length
//     string and object-reference types, attributes in the header;
//   * the dimension scales netCDF-4 builds dimensions from (CLASS,
//     NAME, DIMENSION_LIST through the global heap).
// It is host code only: file bytes are mapped read-only and values are
// converted to double on the host; the dynamics handle then takes them
// through setData.  Anything outside this subset (filters, old-style
// symbol-table groups, version 1 object headers, offsets or lengths other
// than 8 bytes) is reported as unsupported, never read wrongly.
#pragma once

#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace nsdg_nc {

struct FormatError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct Unsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Bob Jenkins' lookup3 hashlittle (2006, public domain), the checksum of
// HDF5's version 2 metadata, with initial value 0 as HDF5 uses it.
uint32_t lookup3(const uint8_t* data, size_t length, uint32_t initval = 0);

enum class TypeClass { Fixed = 0, Float = 1, String = 3, Compound = 6, Reference = 7, VarLen = 9, Other = -1 };

struct Datatype {
    TypeClass cls = TypeClass::Other;
    uint32_t size = 0;
    bool bigEndian = false;
    bool isSigned = false;
    bool vlenString = false;          // VarLen of kind string
    std::shared_ptr<Datatype> base;   // VarLen base type
};

struct Attribute {
    std::string name;
    Datatype type;
    std::vector<uint64_t> dims;       // empty: scalar
    std::vector<uint8_t> raw;         // the stored bytes
};

struct Object {
    uint64_t addr = 0;
    bool isDataset = false;
    // group
    std::vector<std::pair<std::string, uint64_t>> links; // in creation order when tracked
    // dataset
    Datatype type;
    std::vector<uint64_t> dims;       // slowest first, as netCDF lists them
    std::vector<uint64_t> maxDims;
    int layoutClass = -1;             // 0 compact, 1 contiguous, 2 chunked
    uint64_t dataAddr = UINT64_MAX;   // contiguous data or chunk B-tree
    uint64_t dataSize = 0;
    std::vector<uint8_t> compact;
    std::vector<uint32_t> chunk;      // chunk extent per dimension
    bool hasFilters = false;
    std::vector<uint8_t> fill;        // fill value bytes (empty: zeros)
    std::vector<Attribute> attrs;

    const Attribute* attr(const std::string& n) const
    {
        for (const auto& a : attrs)
            if (a.name == n)
                return &a;
        return nullptr;
    }
};

// A netCDF variable: a dataset that is not a dimension-only scale.
struct Variable {
    std::string name;
    std::string path;                 // "data/hice"
    std::vector<std::string> dimNames;
    std::vector<uint64_t> dims;
    const Object* obj = nullptr;
};

class File {
public:
    explicit File(const std::string& path);
    ~File();
    File(const File&) = delete;
    File& operator=(const File&) = delete;

    // the object at a '/'-separated path ("" or "/" is the root group)
    const Object& at(const std::string& path);
    bool exists(const std::string& path);
    // netCDF variables of a group, in link order
    std::vector<Variable> variables(const std::string& group);
    Variable variable(const std::string& path);
    // names of the child groups of a group, in link order
    std::vector<std::string> groups(const std::string& group);
    // every element of a numeric dataset, converted to double
    std::vector<double> readDoubles(const Object& o);
    // the elements [first, first + count) in row-major order, as double
    void readDoubles(const Object& o, uint64_t first, uint64_t count, double* out);
    // a string dataset or attribute (fixed-length or variable-length)
    std::string readText(const Object& o);
    std::string attrText(const Attribute& a);
    double attrDouble(const Attribute& a, size_t i = 0);
    uint64_t fileSize() const { return size_; }

private:
    const uint8_t* base_ = nullptr;
    uint64_t size_ = 0;
    int fd_ = -1;
    uint64_t rootAddr_ = 0;
    std::map<uint64_t, std::unique_ptr<Object>> objects_;

    const uint8_t* span(uint64_t addr, uint64_t len) const;
    const Object& object(uint64_t addr);
    void parseHeader(Object& o);
    void parseMessage(Object& o, int type, const uint8_t* p, size_t len, std::vector<uint64_t>& denseLinks,
        std::vector<std::pair<uint64_t, uint64_t>>& conts);
    void readDenseLinks(Object& o, uint64_t heapAddr, uint64_t btreeAddr);
    std::vector<uint8_t> heapObject(uint64_t collection, uint32_t index);
    void readRaw(const Object& o, uint8_t* out, uint64_t first, uint64_t count);
    void chunkWalk(const Object& o, uint64_t node, int depth, uint8_t* out, uint64_t first,
        uint64_t count, std::set<uint64_t>& seen);
    std::vector<std::string> dimNames(const Object& o, const std::string& group);
};

// Builder of a file in the same subset (nsdg_restart_write.cpp).  Node 0 is
// the root group; nodes are groups, dimension scales or variables.
class Writer {
public:
    Writer();
    ~Writer();
    int addGroup(int parent, const std::string& name);
    void attrText(int node, const std::string& name, const std::string& value);
    void attrDouble(int node, const std::string& name, double value);
    void attrInt(int node, const std::string& name, int32_t value);
    // a netCDF dimension without a coordinate variable
    int addDimension(int group, const std::string& name, uint64_t length, int dimid);
    // a double variable over dimension nodes (slowest first), data row-major
    int addDouble(int group, const std::string& name, const std::vector<int>& dims, const double* data);
    // a scalar int64 variable
    int addInt64(int group, const std::string& name, int64_t value);
    // the unlimited "time" axis: a coordinate variable that is its own dimension
    int addTimeAxis(int group, const std::string& name, int dimid);
    // a double variable over (time axis, dimension nodes...); records appended in order
    int addRecordDouble(int group, const std::string& name, const std::vector<int>& dims);
    void appendRecord(int var, const double* data);
    std::vector<uint8_t> serialize();
    void save(const std::string& path);

private:
    struct Attr;
    struct Node;
    std::vector<Node> nodes_;
    std::vector<uint8_t> header(const Node& n, uint64_t heapAddr) const;
    std::vector<uint8_t> encode(bool withData);
};

} // namespace nsdg_nc
