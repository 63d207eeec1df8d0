// ingest.cu -- KVSML structured volumes and AVS fields read straight into
// resident device volumes.
//
// The reference reads a .kvsml file into a host kvs::StructuredVolumeObject
// (StructuredVolumeObject::read, Object/StructuredVolumeObject.cpp:171-229,
// through KVSMLStructuredVolumeObject::read, FileFormat/KVSML/
// KVSMLStructuredVolumeObject.cpp:159-260, and DataArrayTag / DataArray).
// Here the same file becomes a row-padded device volume, the values never
// held whole in host memory when they are external binary data: the file is
// read in chunks of whole rows into two pinned buffers, each copied by
// cudaMemcpy2DAsync into its device rows while the next chunk is read.  Data
// of the other endianness is byte-swapped on the GPU.  ASCII data (inline or
// external) is parsed on the host the reference's way: tokens split at
// " ,\t\n", each through atof and a cast to the element type
// (DataArray.h:26-31, 230-240).
//
// Header rules kept from the reference: resolution "nx ny nz" (atoi each),
// veclen (atoi), min_value / max_value (atof), object_coord / external_coord
// (6 floats, atof each); the volume's min/max are the file's when it gives
// both, else the scanned min/max with the given one substituted
// (StructuredVolumeObject.cpp:214-226); object coords are the file's or
// [0, res - 1], and then external coords default to them
// (StructuredVolumeObject.cpp:193-209, 348-423).
#include <fcntl.h>
#include <unistd.h>

#include <atomic>
#include <thread>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

namespace {

using kvsmc_host::fail;

// ------------------------------------------------------------ XML subset

struct Elem {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;          // the element's first text child (whitespace kept)
    std::vector<int> children;
    int parent = -1;
    const std::string* attr(const char* k) const
    {
        for (auto& a : attrs)
            if (a.first == k) return &a.second;
        return nullptr;
    }
};

std::string decode_entities(const std::string& s)
{
    std::string o;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == '&') {
            static const char* names[5] = {"&lt;", "&gt;", "&amp;", "&quot;", "&apos;"};
            static const char chars[5] = {'<', '>', '&', '"', '\''};
            bool done = false;
            for (int k = 0; k < 5 && !done; ++k)
                if (s.compare(i, std::strlen(names[k]), names[k]) == 0) {
                    o += chars[k];
                    i += std::strlen(names[k]) - 1;
                    done = true;
                }
            if (!done) o += s[i];
        } else {
            o += s[i];
        }
    }
    return o;
}

// Elements, attributes and text of a KVSML document (no DTDs, no CDATA).
bool parse_xml(const std::string& doc, std::vector<Elem>& out, std::string& err)
{
    out.clear();
    int cur = -1;
    size_t i = 0;
    const size_t n = doc.size();
    while (i < n) {
        if (doc[i] != '<') {
            const size_t j = doc.find('<', i);
            const size_t e = j == std::string::npos ? n : j;
            if (cur >= 0 && out[cur].text.empty() && out[cur].children.empty())
                out[cur].text = decode_entities(doc.substr(i, e - i));
            i = e;
            continue;
        }
        if (doc.compare(i, 4, "<!--") == 0) {
            const size_t j = doc.find("-->", i + 4);
            if (j == std::string::npos) { err = "unterminated comment"; return false; }
            i = j + 3;
            continue;
        }
        if (doc.compare(i, 2, "<?") == 0 || doc.compare(i, 2, "<!") == 0) {
            const size_t j = doc.find('>', i);
            if (j == std::string::npos) { err = "unterminated declaration"; return false; }
            i = j + 1;
            continue;
        }
        if (doc.compare(i, 2, "</") == 0) {
            const size_t j = doc.find('>', i);
            if (j == std::string::npos || cur < 0) { err = "bad end tag"; return false; }
            cur = out[cur].parent;
            i = j + 1;
            continue;
        }
        // start tag
        size_t j = i + 1;
        while (j < n && !std::isspace((unsigned char)doc[j]) && doc[j] != '>' && doc[j] != '/') ++j;
        Elem e;
        e.name = doc.substr(i + 1, j - i - 1);
        bool self_close = false;
        for (;;) {
            while (j < n && std::isspace((unsigned char)doc[j])) ++j;
            if (j >= n) { err = "unterminated tag <" + e.name + ">"; return false; }
            if (doc[j] == '>') { ++j; break; }
            if (doc[j] == '/') {
                if (j + 1 < n && doc[j + 1] == '>') { self_close = true; j += 2; break; }
                err = "bad tag <" + e.name + ">";
                return false;
            }
            size_t k = j;
            while (k < n && doc[k] != '=' && !std::isspace((unsigned char)doc[k]) && doc[k] != '>') ++k;
            const std::string key = doc.substr(j, k - j);
            while (k < n && std::isspace((unsigned char)doc[k])) ++k;
            if (k >= n || doc[k] != '=') { err = "attribute without value in <" + e.name + ">"; return false; }
            ++k;
            while (k < n && std::isspace((unsigned char)doc[k])) ++k;
            if (k >= n || (doc[k] != '"' && doc[k] != '\'')) { err = "unquoted attribute in <" + e.name + ">"; return false; }
            const char q = doc[k];
            const size_t v0 = k + 1;
            const size_t v1 = doc.find(q, v0);
            if (v1 == std::string::npos) { err = "unterminated attribute in <" + e.name + ">"; return false; }
            e.attrs.push_back({key, decode_entities(doc.substr(v0, v1 - v0))});
            j = v1 + 1;
        }
        e.parent = cur;
        out.push_back(e);
        const int id = (int)out.size() - 1;
        if (cur >= 0) out[cur].children.push_back(id);
        if (!self_close) cur = id;
        i = j;
    }
    return true;
}

int child(const std::vector<Elem>& x, int parent, const char* name)
{
    if (parent < 0) {
        for (size_t i = 0; i < x.size(); ++i)
            if (x[i].parent < 0 && x[i].name == name) return (int)i;
        return -1;
    }
    for (int c : x[parent].children)
        if (x[c].name == name) return c;
    return -1;
}

// kvs::Tokenizer over a set of delimiter characters: the non-empty tokens.
template <typename F> void tokens(const char* s, size_t len, const char* delim, F&& f)
{
    size_t i = 0;
    while (i < len) {
        while (i < len && std::strchr(delim, s[i]) && s[i]) ++i;
        size_t j = i;
        while (j < len && !(std::strchr(delim, s[j]) && s[j])) ++j;
        if (j > i && !f(s + i, j - i)) return;
        i = j;
    }
}

double atof_n(const char* s, size_t len)
{
    char buf[128];
    if (len < sizeof buf) {
        std::memcpy(buf, s, len);
        buf[len] = 0;
        return std::atof(buf);
    }
    return std::atof(std::string(s, len).c_str());
}

int atoi_n(const char* s, size_t len)
{
    return std::atoi(std::string(s, len).c_str());
}

int dtype_of(const std::string& t)
{
    if (t == "char") return KVSMC_I8;
    if (t == "unsigned char" || t == "uchar") return KVSMC_U8;
    if (t == "short") return KVSMC_I16;
    if (t == "unsigned short" || t == "ushort") return KVSMC_U16;
    if (t == "int") return KVSMC_I32;
    if (t == "unsigned int" || t == "uint") return KVSMC_U32;
    if (t == "float") return KVSMC_F32;
    if (t == "double") return KVSMC_F64;
    return -1;
}

size_t dsize(int dt)
{
    switch (dt) {
    case KVSMC_I8: case KVSMC_U8: return 1;
    case KVSMC_I16: case KVSMC_U16: return 2;
    case KVSMC_I32: case KVSMC_U32: case KVSMC_F32: return 4;
    default: return 8;
    }
}

template <typename T> void cast_store(void* out, size_t i, double v) { static_cast<T*>(out)[i] = static_cast<T>(v); }

void store_value(int dt, void* out, size_t i, double v)
{
    switch (dt) {
    case KVSMC_I8: cast_store<int8_t>(out, i, v); break;
    case KVSMC_U8: cast_store<uint8_t>(out, i, v); break;
    case KVSMC_I16: cast_store<int16_t>(out, i, v); break;
    case KVSMC_U16: cast_store<uint16_t>(out, i, v); break;
    case KVSMC_I32: cast_store<int32_t>(out, i, v); break;
    case KVSMC_U32: cast_store<uint32_t>(out, i, v); break;
    case KVSMC_F32: cast_store<float>(out, i, v); break;
    default: cast_store<double>(out, i, v); break;
    }
}

bool read_file(const std::string& path, std::string& out)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(size > 0 ? (size_t)size : 0);
    const bool ok = size <= 0 || std::fread(&out[0], 1, (size_t)size, f) == (size_t)size;
    std::fclose(f);
    return ok;
}

std::string dir_of(const std::string& path)
{
    const size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string(".") : path.substr(0, s);
}

// The parsed header plus where the values are.
struct Header {
    kvsmc_kvsml_info info;
    std::string text;          // inline ASCII values
    std::string data_file;     // external data, full path
};

bool parse_floats6(const std::string& s, float* v)
{
    int k = 0;
    bool ok = true;
    tokens(s.data(), s.size(), " \n", [&](const char* t, size_t len) {
        if (k < 6) v[k++] = (float)atof_n(t, len);
        return k < 6;
    });
    ok = k == 6;
    return ok;
}

kvsmc_status read_header(const char* path, Header& h, std::string& err)
{
    std::memset(&h.info, 0, sizeof h.info);
    std::string doc;
    if (!read_file(path, doc)) { err = std::string("cannot read ") + path; return KVSMC_ERR_INVALID_ARGUMENT; }
    std::vector<Elem> x;
    if (!parse_xml(doc, x, err)) return KVSMC_ERR_INVALID_ARGUMENT;
    const int kvsml = child(x, -1, "KVSML");
    const int object = child(x, kvsml, "Object");
    const int svo = object >= 0 ? child(x, object, "StructuredVolumeObject") : -1;
    if (kvsml < 0 || object < 0) { err = "no <KVSML><Object>"; return KVSMC_ERR_INVALID_ARGUMENT; }
    if (svo < 0) { err = "Cannot read <StructuredVolumeObject>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    kvsmc_kvsml_info& in = h.info;
    // <Object external_coord object_coord> (ObjectTag.cpp:173-240)
    if (const std::string* a = x[object].attr("external_coord"); a && !a->empty()) {
        float v[6];
        if (!parse_floats6(*a, v)) { err = "6 components are required for 'external_coord'"; return KVSMC_ERR_INVALID_ARGUMENT; }
        in.has_external_coord = 1;
        for (int k = 0; k < 3; ++k) { in.min_external_coord[k] = v[k]; in.max_external_coord[k] = v[3 + k]; }
    }
    bool file_object = false;
    if (const std::string* a = x[object].attr("object_coord"); a && !a->empty()) {
        float v[6];
        if (!parse_floats6(*a, v)) { err = "6 components are required for 'object_coord'"; return KVSMC_ERR_INVALID_ARGUMENT; }
        file_object = true;
        for (int k = 0; k < 3; ++k) { in.min_object_coord[k] = v[k]; in.max_object_coord[k] = v[3 + k]; }
    }
    // <StructuredVolumeObject resolution grid_type> (StructuredVolumeObjectTag.cpp:122-161)
    const std::string* res = x[svo].attr("resolution");
    if (!res || res->empty()) { err = "'resolution' is not specified in <StructuredVolumeObject>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    uint32_t r[3];
    int nr = 0;
    tokens(res->data(), res->size(), " \n", [&](const char* t, size_t len) {
        if (nr < 3) r[nr++] = (uint32_t)atoi_n(t, len);
        return nr < 3;
    });
    if (nr != 3) { err = "3 components are required for 'resolution'"; return KVSMC_ERR_INVALID_ARGUMENT; }
    in.nx = r[0]; in.ny = r[1]; in.nz = r[2];
    const std::string* grid = x[svo].attr("grid_type");
    if (!grid || grid->empty()) { err = "'grid_type' is not specified in <StructuredVolumeObject>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    in.grid_uniform = *grid == "uniform" ? 1 : 0;
    // <Node><Value veclen min_value max_value> (ValueTag.cpp:50-70)
    const int node = child(x, svo, "Node");
    const int value = node >= 0 ? child(x, node, "Value") : -1;
    if (value < 0) { err = "Cannot read <Node><Value>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    const std::string* veclen = x[value].attr("veclen");
    if (!veclen || veclen->empty()) { err = "'veclen' is not specified in <Value>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    in.veclen = (uint32_t)std::atoi(veclen->c_str());
    if (const std::string* a = x[value].attr("min_value"); a && !a->empty()) { in.has_min_value = 1; in.min_value = std::atof(a->c_str()); }
    if (const std::string* a = x[value].attr("max_value"); a && !a->empty()) { in.has_max_value = 1; in.max_value = std::atof(a->c_str()); }
    // <DataArray type file format endian> (DataArrayTag.cpp:173-330)
    const int da = child(x, value, "DataArray");
    if (da < 0) { err = "Cannot read <DataArray> for <Value>."; return KVSMC_ERR_INVALID_ARGUMENT; }
    const std::string* type = x[da].attr("type");
    in.dtype = type ? dtype_of(*type) : -1;
    if (in.dtype < 0) { err = "'type' is not specified or unknown data type in <DataArray>."; return KVSMC_ERR_UNSUPPORTED_DTYPE; }
    const std::string* file = x[da].attr("file");
    if (!file || file->empty()) {
        in.data_format = 0;
        h.text = x[da].text;
    } else {
        const std::string* format = x[da].attr("format");
        if (!format || format->empty()) { err = "'format' is not specified in <DataArray>."; return KVSMC_ERR_INVALID_ARGUMENT; }
        if (*format == "binary") in.data_format = 2;
        else if (*format == "ascii") in.data_format = 1;
        else { err = "Unknown format '" + *format + "'."; return KVSMC_ERR_INVALID_ARGUMENT; }
        h.data_file = dir_of(path) + "/" + *file;
        const std::string* endian = x[da].attr("endian");
        in.byte_swap = (in.data_format == 2 && endian && *endian == "big") ? 1 : 0;   // little-endian host
    }
    // coords (StructuredVolumeObject.cpp:193-209 with updateMinMaxCoords, :348-423)
    if (file_object) {
        in.has_object_coord = 1;
    } else {
        in.has_object_coord = 1;
        for (int k = 0; k < 3; ++k) in.min_object_coord[k] = 0.0f;
        in.max_object_coord[0] = (float)in.nx - 1.0f;
        in.max_object_coord[1] = (float)in.ny - 1.0f;
        in.max_object_coord[2] = (float)in.nz - 1.0f;
        if (!in.has_external_coord) {
            in.has_external_coord = 1;
            for (int k = 0; k < 3; ++k) {
                in.min_external_coord[k] = in.min_object_coord[k];
                in.max_external_coord[k] = in.max_object_coord[k];
            }
        }
    }
    return KVSMC_OK;
}

__global__ void k_byteswap(uint8_t* p, uint64_t n, int es)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint8_t* e = p + i * es;
        for (int a = 0, b = es - 1; a < b; ++a, --b) {
            const uint8_t t = e[a];
            e[a] = e[b];
            e[b] = t;
        }
    }
}

// External binary values (from byte `offset` of the file) streamed into the
// device rows.
// Read len bytes at file offset off into dst with pread, split over up to
// `threads` host threads (page-cache copies run in parallel); false on a
// short read or an error.
bool pread_parallel(int fd, uint8_t* dst, size_t len, uint64_t off, unsigned threads)
{
    const size_t min_piece = 4u << 20;
    unsigned t = (unsigned)std::min<size_t>(threads, std::max<size_t>(1, len / min_piece));
    std::atomic<bool> ok{true};
    auto part = [&](size_t a, size_t b) {
        while (a < b) {
            const ssize_t r = ::pread(fd, dst + a, b - a, (off_t)(off + a));
            if (r <= 0) { ok = false; return; }
            a += (size_t)r;
        }
    };
    if (t <= 1) {
        part(0, len);
        return ok;
    }
    std::vector<std::thread> pool;
    const size_t step = (len + t - 1) / t;
    for (unsigned i = 0; i < t; ++i) {
        const size_t a = std::min(len, i * step), b = std::min(len, a + step);
        if (a < b) pool.emplace_back(part, a, b);
    }
    for (auto& th : pool) th.join();
    return ok;
}

// External binary values: chunks of whole rows read into two pinned buffers
// (each chunk by several threads) and copied into the padded device rows
// while the next chunk is read.
kvsmc_status load_binary(kvsmc_context* ctx, const std::string& file, kvsmc_volume* v, long offset = 0)
{
    const size_t es = dsize(v->view.dtype);
    const size_t row = (size_t)v->view.nx * es;
    const uint64_t rows = (uint64_t)v->view.ny * v->view.nz;
    const size_t chunk_rows = std::max<size_t>(1, (64u << 20) / std::max<size_t>(row, 1));
    const int fd = ::open(file.c_str(), O_RDONLY);
    if (fd < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: Cannot open '%s'.", file.c_str());
    const unsigned threads = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    uint8_t* h[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    const size_t bytes = chunk_rows * row;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaMallocHost(&h[b], bytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
    }
    bool short_read = false;
    uint64_t r0 = 0;
    for (int k = 0; r0 < rows && e == cudaSuccess && !short_read; ++k) {
        const int b = k & 1;
        if (k >= 2) e = cudaEventSynchronize(ev[b]);   // its previous copy has left the buffer
        if (e != cudaSuccess) break;
        const uint64_t nr = std::min<uint64_t>(chunk_rows, rows - r0);
        if (!pread_parallel(fd, h[b], nr * row, (uint64_t)offset + r0 * row, threads)) {
            short_read = true;
            break;
        }
        e = cudaMemcpy2DAsync(static_cast<uint8_t*>(v->dev) + r0 * v->view.pitch * es, v->view.pitch * es, h[b], row,
                              row, nr, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], ctx->stream);
        r0 += nr;
    }
    cudaStreamSynchronize(ctx->stream);
    ::close(fd);
    for (int b = 0; b < 2; ++b) {
        if (h[b]) cudaFreeHost(h[b]);
        if (ev[b]) cudaEventDestroy(ev[b]);
    }
    if (e != cudaSuccess)
        return fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA, "kvsml: %s",
                    cudaGetErrorString(e));
    if (short_read) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: Cannot read '%s'.", file.c_str());
    return KVSMC_OK;
}

// ASCII values (inline text or an external file), parsed on the host.
kvsmc_status load_ascii(kvsmc_context* ctx, const Header& hd, kvsmc_volume* v)
{
    std::string ext;
    const std::string* text = &hd.text;
    if (hd.info.data_format == 1) {
        if (!read_file(hd.data_file, ext))
            return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: Cannot open '%s'.", hd.data_file.c_str());
        text = &ext;
    }
    const int dt = v->view.dtype;
    const uint64_t n = (uint64_t)v->view.nx * v->view.ny * v->view.nz;
    std::vector<uint8_t> host(n * dsize(dt));
    uint64_t got = 0;
    tokens(text->data(), text->size(), " ,\t\n", [&](const char* t, size_t len) {
        if (got < n) store_value(dt, host.data(), got++, atof_n(t, len));
        return got < n;
    });
    if (got < n)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: %llu values for %llu nodes",
                    (unsigned long long)got, (unsigned long long)n);
    const size_t es = dsize(dt);
    const size_t row = (size_t)v->view.nx * es;
    KVSMC_CUDA(ctx, cudaMemcpy2DAsync(v->dev, v->view.pitch * es, host.data(), row, row,
                                      (size_t)v->view.ny * v->view.nz, cudaMemcpyHostToDevice, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

// ------------------------------------------------------------ AVS field
//
// kvs::AVSField::read (FileFormat/AVSField/AVSField.cpp): the first line
// starts "# AVS"; then "key = value" lines (tokens split at " ,\t\n", lines
// starting '#' skipped) up to a line starting with a form feed; the values
// follow the first "\f\f" of the file, raw, in the host's byte order.
// StructuredVolumeImporter::import(const AVSField*) (:155-189) takes only
// uniform fields; object coords [0, dim - 1]; external coords min_ext /
// max_ext when either is given (defaults (0,0,0) / (1,1,1)), else the object
// coords; min/max by the scan.
struct AvsHeader {
    kvsmc_kvsml_info info;
    long data_offset = -1;
    bool uniform = false;
};

kvsmc_status read_avs_header(const char* path, AvsHeader& h, std::string& err)
{
    std::memset(&h.info, 0, sizeof h.info);
    std::string doc;
    if (!read_file(path, doc)) { err = std::string("Cannot open ") + path; return KVSMC_ERR_INVALID_ARGUMENT; }
    if (doc.compare(0, 5, "# AVS") != 0) { err = "not an AVS field file"; return KVSMC_ERR_INVALID_ARGUMENT; }
    kvsmc_kvsml_info& in = h.info;
    in.veclen = 1;
    in.nx = in.ny = in.nz = 1;
    float min_ext[3] = {0, 0, 0}, max_ext[3] = {1, 1, 1};
    bool has_ext = false;
    int data = -1;
    std::string field;
    size_t pos = doc.find('\n') == std::string::npos ? doc.size() : doc.find('\n') + 1;
    while (pos < doc.size()) {
        if (doc[pos] == '\f') break;   // the data separator
        const size_t eol = doc.find('\n', pos);
        const size_t end = eol == std::string::npos ? doc.size() : eol;
        const std::string line = doc.substr(pos, end - pos);
        pos = end + 1;
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> t;
        tokens(line.data(), line.size(), " ,\t\n", [&](const char* s, size_t n) { t.emplace_back(s, n); return true; });
        if (t.size() < 3 || t[1] != "=") continue;
        const std::string& key = t[0];
        const char* val = t[2].c_str();
        if (key == "veclen") in.veclen = (uint32_t)std::atoi(val);
        else if (key == "dim1") in.nx = (uint32_t)std::atoi(val);
        else if (key == "dim2") in.ny = (uint32_t)std::atoi(val);
        else if (key == "dim3") in.nz = (uint32_t)std::atoi(val);
        else if (key == "field") field = t[2];
        else if (key == "data") {
            data = t[2] == "byte" ? KVSMC_U8 : t[2] == "short" ? KVSMC_I16 : t[2] == "integer" ? KVSMC_I32
                 : t[2] == "float" ? KVSMC_F32 : t[2] == "double" ? KVSMC_F64 : -1;
        } else if ((key == "min_ext" || key == "max_ext") && t.size() >= 5) {
            float* e = key == "min_ext" ? min_ext : max_ext;
            for (int k = 0; k < 3; ++k) e[k] = (float)std::atof(t[2 + k].c_str());
            has_ext = true;
        }
    }
    const size_t ff = doc.find("\f\f");
    if (ff == std::string::npos) { err = "no data separator"; return KVSMC_ERR_INVALID_ARGUMENT; }
    h.data_offset = (long)(ff + 2);
    h.uniform = field == "uniform";
    in.grid_uniform = h.uniform ? 1 : 0;
    in.dtype = data;
    in.data_format = 2;
    if (data < 0) { err = "unknown 'data' type"; return KVSMC_ERR_UNSUPPORTED_DTYPE; }
    in.has_object_coord = 1;
    in.max_object_coord[0] = (float)in.nx - 1.0f;
    in.max_object_coord[1] = (float)in.ny - 1.0f;
    in.max_object_coord[2] = (float)in.nz - 1.0f;
    in.has_external_coord = 1;
    for (int k = 0; k < 3; ++k) {
        in.min_external_coord[k] = has_ext ? min_ext[k] : in.min_object_coord[k];
        in.max_external_coord[k] = has_ext ? max_ext[k] : in.max_object_coord[k];
    }
    return KVSMC_OK;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_avs_read_info(const char* path, kvsmc_kvsml_info* info)
{
    if (!path || !info) return KVSMC_ERR_INVALID_ARGUMENT;
    AvsHeader h;
    std::string err;
    const kvsmc_status st = read_avs_header(path, h, err);
    *info = h.info;
    return st;
}

kvsmc_status kvsmc_volume_load_avs(kvsmc_context* ctx, const char* path, kvsmc_volume** vol, kvsmc_kvsml_info* info)
{
    if (!ctx || !path || !vol) return KVSMC_ERR_INVALID_ARGUMENT;
    *vol = nullptr;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    AvsHeader h;
    std::string err;
    kvsmc_status st = read_avs_header(path, h, err);
    if (info) *info = h.info;
    if (st) return fail(ctx, st, "avs: %s: %s", path, err.c_str());
    if (!h.uniform) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "'Uniform' type in kvs::AVSField format is only supported.");
    if (h.info.veclen != 1)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "avs: veclen %u: the device volumes are scalar fields",
                    h.info.veclen);
    kvsmc_volume* v = nullptr;
    if ((st = kvsmc_host::volume_create(ctx, (kvsmc_dtype)h.info.dtype, h.info.nx, h.info.ny, h.info.nz, &v)))
        return st;
    st = load_binary(ctx, path, v, h.data_offset);
    if (!st) st = kvsmc_volume_minmax(ctx, v, &v->vmin, &v->vmax);
    if (!st) st = kvsmc_host::volume_bricks(ctx, v);
    if (st) {
        kvsmc_volume_free(ctx, v);
        return st;
    }
    if (info) {
        info->volume_min = v->vmin;
        info->volume_max = v->vmax;
    }
    *vol = v;
    return KVSMC_OK;
}

kvsmc_status kvsmc_kvsml_read_info(const char* path, kvsmc_kvsml_info* info)
{
    if (!path || !info) return KVSMC_ERR_INVALID_ARGUMENT;
    Header h;
    std::string err;
    const kvsmc_status st = read_header(path, h, err);
    *info = h.info;
    return st;
}

kvsmc_status kvsmc_volume_load_kvsml(kvsmc_context* ctx, const char* path, kvsmc_volume** vol,
                                     kvsmc_kvsml_info* info)
{
    if (!ctx || !path || !vol) return KVSMC_ERR_INVALID_ARGUMENT;
    *vol = nullptr;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    Header h;
    std::string err;
    kvsmc_status st = read_header(path, h, err);
    if (info) *info = h.info;
    if (st) return fail(ctx, st, "kvsml: %s: %s", path, err.c_str());
    if (h.info.veclen != 1)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: veclen %u: the device volumes are scalar fields",
                    h.info.veclen);
    if (!h.info.grid_uniform)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: only uniform grids are loaded onto the device");
    kvsmc_volume* v = nullptr;
    if ((st = kvsmc_host::volume_create(ctx, (kvsmc_dtype)h.info.dtype, h.info.nx, h.info.ny, h.info.nz, &v)))
        return st;
    st = h.info.data_format == 2 ? load_binary(ctx, h.data_file, v) : load_ascii(ctx, h, v);
    if (!st && h.info.byte_swap) {
        const uint64_t n = v->view.slice * v->view.nz;
        const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->num_sms * 8);
        k_byteswap<<<blocks, 256, 0, ctx->stream>>>(static_cast<uint8_t*>(v->dev), n, (int)dsize(h.info.dtype));
        ctx->launches += 1;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = fail(ctx, KVSMC_ERR_CUDA, "kvsml: byte swap: %s", cudaGetErrorString(e));
    }
    // the volume's min/max (StructuredVolumeObject.cpp:214-226)
    if (!st) {
        if (h.info.has_min_value && h.info.has_max_value) {
            v->vmin = h.info.min_value;
            v->vmax = h.info.max_value;
            v->has_minmax = true;
        } else {
            st = kvsmc_volume_minmax(ctx, v, &v->vmin, &v->vmax);
            if (!st) {
                if (h.info.has_min_value) v->vmin = h.info.min_value;
                if (h.info.has_max_value) v->vmax = h.info.max_value;
            }
        }
    }
    if (!st) st = kvsmc_host::volume_bricks(ctx, v);
    if (st) {
        kvsmc_volume_free(ctx, v);
        return st;
    }
    if (info) {
        info->volume_min = v->vmin;
        info->volume_max = v->vmax;
    }
    *vol = v;
    return KVSMC_OK;
}

}  // extern "C"
