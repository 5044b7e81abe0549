// nsdg_restart_capi.cpp — the C ABI of the restart and forcing file reader
// (nsdg_restart_* in include/nsdg.h): ParaGridIO::getModelState and
// ParaGridIO::readForcingTimeStatic (core/src/ParaGridIO.cpp:87-270) over
// the host reader in nsdg_restart.cpp.
#include "nsdg.h"
#include "nsdg_restart.hpp"

#include <cstring>
#include <map>
#include <string>

struct nsdg_restart {
    std::unique_ptr<nsdg_nc::File> file;
    std::string error;
};

namespace {

thread_local std::string gOpenError;

// ParaGridIO's dimension keys (core/src/ParaGridIO.cpp:34-47): the netCDF
// dimension names of a variable, concatenated in file order
int modelType(const std::string& key)
{
    static const std::map<std::string, int> keys = {
        { "yx", NSDG_MA_H },
        { "ydimxdim", NSDG_MA_H },
        { "zyx", NSDG_MA_Z },
        { "zdimydimxdim", NSDG_MA_Z },
        { "yxdg_comp", NSDG_MA_DG },
        { "ydimxdimdg_comp", NSDG_MA_DG },
        { "yxdgstress_comp", NSDG_MA_DGSTRESS },
        { "ydimxdimdgstress_comp", NSDG_MA_DGSTRESS },
        { "ycgxcg", NSDG_MA_CG },
        { "yvertexxvertexncoords", NSDG_MA_VERTEX },
    };
    const auto it = keys.find(key);
    return it == keys.end() ? NSDG_MA_NONE : it->second;
}

// the leading record dimension of forcing files
bool isRecordDim(const nsdg_nc::Variable& v)
{
    return !v.dims.empty() && v.dimNames[0] == "time" && v.dims.size() > 1;
}

template <class F>
int guarded(nsdg_restart* r, F&& f)
{
    if (!r)
        return NSDG_ERR_BAD_ARG;
    try {
        r->error.clear();
        return f();
    } catch (const nsdg_nc::Unsupported& e) {
        r->error = e.what();
        return NSDG_ERR_UNSUPPORTED;
    } catch (const nsdg_nc::FormatError& e) {
        r->error = e.what();
        return NSDG_ERR_LOGIC;
    } catch (const std::out_of_range& e) {
        r->error = e.what();
        return NSDG_ERR_UNKNOWN_FIELD;
    } catch (const std::exception& e) {
        r->error = e.what();
        return NSDG_ERR_BAD_ARG;
    }
}

int copyText(const std::string& s, char* out, size_t cap)
{
    if (!out || cap == 0)
        return NSDG_ERR_BAD_ARG;
    if (s.size() + 1 > cap)
        return NSDG_ERR_SIZE_MISMATCH;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return NSDG_OK;
}

} // namespace

extern "C" {

int nsdg_restart_open(const char* path, nsdg_restart** out)
{
    if (!path || !out)
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    try {
        auto r = std::make_unique<nsdg_restart>();
        r->file = std::make_unique<nsdg_nc::File>(path);
        r->file->at(""); // parses the root group
        *out = r.release();
        gOpenError.clear();
        return NSDG_OK;
    } catch (const nsdg_nc::Unsupported& e) {
        gOpenError = e.what();
        return NSDG_ERR_UNSUPPORTED;
    } catch (const nsdg_nc::FormatError& e) {
        gOpenError = e.what();
        return NSDG_ERR_LOGIC;
    } catch (const std::exception& e) {
        gOpenError = e.what();
        return NSDG_ERR_BAD_ARG;
    }
}

int nsdg_restart_close(nsdg_restart* r)
{
    delete r;
    return NSDG_OK;
}

const char* nsdg_restart_last_error(const nsdg_restart* r)
{
    return r ? r->error.c_str() : gOpenError.c_str();
}

int nsdg_restart_num_vars(nsdg_restart* r, const char* group, size_t* n)
{
    return guarded(r, [&] {
        if (!n)
            return NSDG_ERR_BAD_ARG;
        *n = r->file->variables(group ? group : "").size();
        return NSDG_OK;
    });
}

int nsdg_restart_var_info(nsdg_restart* r, const char* group, size_t index, char* name, size_t name_cap,
    int* model_type, size_t* n_components, size_t* n_records, size_t* n_values)
{
    return guarded(r, [&] {
        const auto vars = r->file->variables(group ? group : "");
        if (index >= vars.size())
            return NSDG_ERR_BAD_ARG;
        const auto& v = vars[index];
        const size_t skip = isRecordDim(v) ? 1 : 0;
        std::string key;
        for (size_t i = skip; i < v.dimNames.size(); ++i)
            key += v.dimNames[i];
        const int type = modelType(key);
        size_t values = 1;
        for (size_t i = skip; i < v.dims.size(); ++i)
            values *= v.dims[i];
        if (name) {
            const int st = copyText(v.name, name, name_cap);
            if (st != NSDG_OK)
                return st;
        }
        if (model_type)
            *model_type = type;
        if (n_components)
            *n_components = (type == NSDG_MA_DG || type == NSDG_MA_DGSTRESS || type == NSDG_MA_VERTEX)
                ? v.dims.back() : 1;
        if (n_records)
            *n_records = skip ? v.dims[0] : 1;
        if (n_values)
            *n_values = values;
        return NSDG_OK;
    });
}

int nsdg_restart_dim_names(nsdg_restart* r, const char* path, char* out, size_t cap)
{
    return guarded(r, [&] {
        if (!path)
            return NSDG_ERR_BAD_ARG;
        const auto v = r->file->variable(path);
        std::string s;
        for (size_t i = 0; i < v.dimNames.size(); ++i)
            s += (i ? "," : "") + v.dimNames[i];
        return copyText(s, out, cap);
    });
}

int nsdg_restart_read(nsdg_restart* r, const char* path, size_t record, double* out, size_t n)
{
    return guarded(r, [&] {
        if (!path || (!out && n))
            return NSDG_ERR_BAD_ARG;
        const auto v = r->file->variable(path);
        const bool rec = isRecordDim(v);
        const uint64_t records = rec ? v.dims[0] : 1;
        uint64_t per = 1;
        for (size_t i = rec ? 1 : 0; i < v.dims.size(); ++i)
            per *= v.dims[i];
        if (record >= records)
            return NSDG_ERR_BAD_ARG;
        if (n != per)
            return NSDG_ERR_SIZE_MISMATCH;
        r->file->readDoubles(*v.obj, record * per, per, out);
        return NSDG_OK;
    });
}

int nsdg_restart_text(nsdg_restart* r, const char* path, const char* attribute, char* out, size_t cap)
{
    return guarded(r, [&] {
        if (!path)
            return NSDG_ERR_BAD_ARG;
        const auto& o = r->file->at(path);
        if (!attribute)
            return copyText(r->file->readText(o), out, cap);
        const auto* a = o.attr(attribute);
        if (!a)
            throw std::out_of_range(std::string("no attribute ") + attribute + " on " + path);
        return copyText(r->file->attrText(*a), out, cap);
    });
}

} // extern "C"

// ---------------------------------------------------------------- writer
struct nsdg_restart_writer {
    nsdg_nc::Writer w;
    std::string error;
    size_t nx = 0, ny = 0, nz = 1;
    int dg = 0, dgs = 0, cg = 2;
    int data = 0;
    int dim[10] = {}; // xdim ydim zdim xvertex yvertex x_cg y_cg dg_comp dgstress_comp ncoords
    // diagnostic files: the time axis and the record variables by name
    int time = -1;
    size_t records = 0;
    std::map<std::string, std::pair<int, int>> vars; // name -> (node, model type)
};

namespace {

bool validShape(size_t nx, size_t ny, size_t nz, int dg, int dgs, int cg)
{
    return nx && ny && nz && dg > 0 && dgs > 0 && (cg == 1 || cg == 2);
}

// CommonRestartMetadata's groups and the data group's dimensions, in the
// order dumpModelState (diagnostic = false) or writeDiagnosticTime
// (diagnostic = true: metadata and data first, the time axis before the
// other dimensions) creates them
void layOut(nsdg_restart_writer& r, const char* structure, long long t, const char* formatted, bool diagnostic)
{
    auto& w = r.w;
    int meta = 0;
    if (!diagnostic)
        w.attrText(w.addGroup(0, "structure"), "type", structure);
    meta = w.addGroup(0, "metadata");
    if (diagnostic)
        r.data = w.addGroup(0, "data");
    if (diagnostic)
        w.attrText(w.addGroup(0, "structure"), "type", structure);
    w.attrText(meta, "type", structure);
    const int timeGroup = w.addGroup(meta, "time");
    const int tv = w.addInt64(timeGroup, "time", t);
    w.attrText(tv, "units", "seconds since 1970-01-01T00:00:00Z");
    w.attrText(tv, "format", "%Y-%m-%dT%H:%M:%SZ");
    w.attrText(tv, "formatted", formatted);
    w.addGroup(meta, "configuration");
    if (!diagnostic)
        r.data = w.addGroup(0, "data");
    int dimid = 0;
    if (diagnostic)
        r.time = w.addTimeAxis(r.data, "time", dimid++);
    const char* names[10] = { "xdim", "ydim", "zdim", "xvertex", "yvertex", "x_cg", "y_cg", "dg_comp",
        "dgstress_comp", "ncoords" };
    const uint64_t sizes[10] = { r.nx, r.ny, r.nz, r.nx + 1, r.ny + 1, r.cg * r.nx + 1, r.cg * r.ny + 1,
        static_cast<uint64_t>(r.dg), static_cast<uint64_t>(r.dgs), 2 };
    for (int i = 0; i < 10; ++i)
        r.dim[i] = w.addDimension(r.data, names[i], sizes[i], dimid++);
}

// the netCDF dimensions of a ModelArray type (dumpModelState's dimMap) and
// the values they hold; empty for an unknown type
std::vector<int> typeDims(const nsdg_restart_writer& w, int model_type, size_t& values)
{
    const int* d = w.dim;
    std::vector<int> dims;
    switch (model_type) {
    case NSDG_MA_H:
    case NSDG_MA_U:
    case NSDG_MA_V:
        dims = { d[1], d[0] };
        break;
    case NSDG_MA_Z:
        dims = { d[2], d[1], d[0] };
        break;
    case NSDG_MA_DG:
        dims = { d[1], d[0], d[7] };
        break;
    case NSDG_MA_DGSTRESS:
        dims = { d[1], d[0], d[8] };
        break;
    case NSDG_MA_CG:
        dims = { d[6], d[5] };
        break;
    case NSDG_MA_VERTEX:
        dims = { d[4], d[3], d[9] };
        break;
    default:
        break;
    }
    const size_t sizes[10] = { w.nx, w.ny, w.nz, w.nx + 1, w.ny + 1, w.cg * w.nx + 1, w.cg * w.ny + 1,
        static_cast<size_t>(w.dg), static_cast<size_t>(w.dgs), 2 };
    values = 1;
    for (int id : dims)
        for (int k = 0; k < 10; ++k)
            if (d[k] == id)
                values *= sizes[k];
    return dims;
}

} // namespace

extern "C" {

int nsdg_restart_writer_create(size_t nx, size_t ny, size_t nz, int dg_comp, int dgstress_comp, int cg_degree,
    const char* structure_type, long long time_seconds, const char* time_formatted, nsdg_restart_writer** out)
{
    if (!out || !structure_type || !time_formatted || !validShape(nx, ny, nz, dg_comp, dgstress_comp, cg_degree))
        return NSDG_ERR_BAD_ARG;
    auto r = std::make_unique<nsdg_restart_writer>();
    r->nx = nx;
    r->ny = ny;
    r->nz = nz;
    r->dg = dg_comp;
    r->dgs = dgstress_comp;
    r->cg = cg_degree;
    layOut(*r, structure_type, time_seconds, time_formatted, false);
    *out = r.release();
    return NSDG_OK;
}

int nsdg_restart_writer_add(nsdg_restart_writer* w, const char* name, int model_type, const double* data, size_t n)
{
    if (!w || !name || !*name || (!data && n))
        return NSDG_ERR_BAD_ARG;
    if (w->time >= 0)
        return NSDG_ERR_LOGIC; // a diagnostic file takes records
    size_t expect = 0;
    const std::vector<int> dims = typeDims(*w, model_type, expect);
    if (dims.empty())
        return NSDG_ERR_BAD_ARG;
    if (n != expect)
        return NSDG_ERR_SIZE_MISMATCH;
    try {
        const int v = w->w.addDouble(w->data, name, dims, data);
        w->w.attrDouble(v, "missing_value", 1.7e38); // MissingData::defaultValue
        return NSDG_OK;
    } catch (const std::exception& e) {
        w->error = e.what();
        return NSDG_ERR_BAD_ARG;
    }
}

int nsdg_diagnostic_writer_create(size_t nx, size_t ny, size_t nz, int dg_comp, int dgstress_comp, int cg_degree,
    const char* structure_type, long long time_seconds, const char* time_formatted, nsdg_restart_writer** out)
{
    if (!out || !structure_type || !time_formatted || !validShape(nx, ny, nz, dg_comp, dgstress_comp, cg_degree))
        return NSDG_ERR_BAD_ARG;
    auto r = std::make_unique<nsdg_restart_writer>();
    r->nx = nx;
    r->ny = ny;
    r->nz = nz;
    r->dg = dg_comp;
    r->dgs = dgstress_comp;
    r->cg = cg_degree;
    layOut(*r, structure_type, time_seconds, time_formatted, true);
    *out = r.release();
    return NSDG_OK;
}

int nsdg_diagnostic_writer_record(nsdg_restart_writer* w, double time_seconds, size_t n_fields,
    const char* const* names, const int* model_types, const double* const* data, const size_t* n)
{
    if (!w || w->time < 0 || (n_fields && (!names || !model_types || !data || !n)))
        return NSDG_ERR_BAD_ARG;
    const bool first = w->records == 0;
    // check the whole record before anything is appended
    std::vector<std::vector<int>> dims(n_fields);
    for (size_t f = 0; f < n_fields; ++f) {
        if (!names[f] || !*names[f] || (!data[f] && n[f]))
            return NSDG_ERR_BAD_ARG;
        size_t expect = 0;
        dims[f] = typeDims(*w, model_types[f], expect);
        if (dims[f].empty())
            return NSDG_ERR_BAD_ARG;
        if (n[f] != expect)
            return NSDG_ERR_SIZE_MISMATCH;
        const std::string nm = names[f];
        const bool once = nm == "mask" || model_types[f] == NSDG_MA_VERTEX;
        if (!first && !once) {
            const auto it = w->vars.find(nm);
            if (it == w->vars.end() || it->second.second != model_types[f]) {
                w->error = "field " + nm + " is not a variable of this diagnostic file";
                return NSDG_ERR_UNKNOWN_FIELD;
            }
        }
    }
    try {
        w->w.appendRecord(w->time, &time_seconds);
        std::map<std::string, bool> given;
        for (size_t f = 0; f < n_fields; ++f) {
            const std::string nm = names[f];
            if (nm == "mask" || model_types[f] == NSDG_MA_VERTEX) {
                if (!first)
                    continue;
                // written once, without the time axis; the mask with the
                // dimensions (xdim, ydim) in the order writeDiagnosticTime
                // lists them (ParaGridIO.cpp:439-451)
                const std::vector<int> d = nm == "mask" ? std::vector<int> { w->dim[0], w->dim[1] } : dims[f];
                const int v = w->w.addDouble(w->data, nm, d, data[f]);
                if (nm != "mask")
                    w->w.attrDouble(v, "missing_value", 1.7e38);
                continue;
            }
            if (first) {
                std::vector<int> d { w->time };
                d.insert(d.end(), dims[f].begin(), dims[f].end());
                const int v = w->w.addRecordDouble(w->data, nm, d);
                w->w.attrDouble(v, "missing_value", 1.7e38);
                w->vars[nm] = { v, model_types[f] };
            }
            w->w.appendRecord(w->vars.at(nm).first, data[f]);
            given[nm] = true;
        }
        // variables this record leaves out keep netCDF's fill value there
        for (const auto& kv : w->vars)
            if (!given.count(kv.first)) {
                size_t values = 0;
                typeDims(*w, kv.second.second, values);
                const std::vector<double> fill(values, 9.9692099683868690e+36);
                w->w.appendRecord(kv.second.first, fill.data());
            }
        ++w->records;
        return NSDG_OK;
    } catch (const std::exception& e) {
        w->error = e.what();
        return NSDG_ERR_BAD_ARG;
    }
}

int nsdg_restart_writer_save(nsdg_restart_writer* w, const char* path)
{
    if (!w || !path)
        return NSDG_ERR_BAD_ARG;
    try {
        w->error.clear();
        w->w.save(path);
        return NSDG_OK;
    } catch (const std::exception& e) {
        w->error = e.what();
        return NSDG_ERR_BAD_ARG;
    }
}

int nsdg_restart_writer_destroy(nsdg_restart_writer* w)
{
    delete w;
    return NSDG_OK;
}

const char* nsdg_restart_writer_last_error(const nsdg_restart_writer* w)
{
    return w ? w->error.c_str() : "";
}

} // extern "C"
