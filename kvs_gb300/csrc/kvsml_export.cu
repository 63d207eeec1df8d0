// kvsml_export.cu -- the KVSML polygon file of a device mesh.
//
// What PolygonExporter<kvs::KVSMLPolygonObject>::exec
// (Source/Core/Visualization/Exporter/PolygonExporter.cpp:22-68) and
// KVSMLPolygonObject::write (Source/Core/FileFormat/KVSML/KVSMLPolygonObject.cpp:349-492)
// write for a triangle mesh, byte for byte: the XML declaration and comment,
// <KVSML>, <Object type="PolygonObject">, <PolygonObject polygon_type
// color_type normal_type>, <Vertex nvertices> with <Coord> (and <Normal> for
// vertex normals), <Polygon npolygons> with <Connection>, the single colour
// and opacity as <DataValue>s and <Normal> for polygon normals, indented by
// four blanks per level as the XML printer does.  Arrays, by writing data type
// (DataWriter.cpp, DataArrayTag.h:110-169, DataArray.h:365-440):
//   0 Ascii:          inside <DataArray type="...">, each value and a blank;
//   1 ExternalAscii:  <DataArray ... format="ascii" file="<base>_<kind>.dat" />,
//                     each value and ", " in that file;
//   2 ExternalBinary: format="binary" ... endian="little", the raw array.
// Floats print as an ostream prints them (six significant digits, "%g"),
// the connections' uint32 and the colour bytes as integers.  Binary arrays go
// from device memory to the file through pinned staging buffers in chunks;
// ASCII arrays are copied back and formatted on all host threads.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "context.h"

namespace {

using kvsmc_host::fail;

// base name (no directory, no extension) and directory of a path, as
// kvs::File::baseName / pathName give them
void split_path(const std::string& path, std::string& dir, std::string& base)
{
    const size_t slash = path.find_last_of('/');
    dir = slash == std::string::npos ? "." : path.substr(0, slash);
    const std::string file = slash == std::string::npos ? path : path.substr(slash + 1);
    const size_t dot = file.find_last_of('.');
    base = dot == std::string::npos ? file : file.substr(0, dot);
}

// Text of n values of a host array, each followed by `sep`, formatted on all
// host threads in order.
template <typename T>
std::string format_values(const T* v, uint64_t n, const char* sep)
{
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint64_t per = (n + nt - 1) / nt;
    std::vector<std::string> parts(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t a = t * per, b = std::min(n, a + per);
        if (a >= b) break;
        th.emplace_back([&, t, a, b]() {
            std::string& s = parts[t];
            s.reserve((b - a) * 12);
            char buf[64];
            for (uint64_t i = a; i < b; ++i) {
                int k;
                if constexpr (std::is_same<T, float>::value)
                    k = std::snprintf(buf, sizeof buf, "%.6g%s", (double)v[i], sep);
                else
                    k = std::snprintf(buf, sizeof buf, "%llu%s", (unsigned long long)v[i], sep);
                s.append(buf, (size_t)k);
            }
        });
    }
    for (auto& x : th) x.join();
    std::string out;
    size_t total = 0;
    for (auto& p : parts) total += p.size();
    out.reserve(total);
    for (auto& p : parts) out += p;
    return out;
}

// One device array written by the chosen writing data type.
struct ArrayOut {
    const void* d;
    uint64_t n;        // elements
    int is_float;      // float32, else uint32
    const char* kind;  // file suffix: coord, normal, connect
};

}  // namespace

extern "C" {

kvsmc_status kvsmc_write_kvsml_polygon(kvsmc_context* ctx, const char* path, int32_t writing_type, int32_t mode,
                                       const float* d_coords, uint64_t ncoords, const float* d_normals,
                                       uint64_t nnormals, const uint32_t* d_connections, uint64_t nconnections,
                                       const uint8_t* color, const uint8_t* opacity)
{
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    if (writing_type < 0 || writing_type > 2)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: bad writing data type %d", (int)writing_type);
    if (mode != KVSMC_DUP_POLYGON_NORMAL && mode != KVSMC_SHARED_POLYGON_NORMAL && mode != KVSMC_SHARED_VERTEX_NORMAL)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: bad mode %d", (int)mode);
    if ((ncoords && !d_coords) || (nnormals && !d_normals) || (nconnections && !d_connections))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: null mesh array");
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool vertex_normals = mode == KVSMC_SHARED_VERTEX_NORMAL;
    std::string dir, base;
    split_path(path, dir, base);
    const uint64_t nvertices = ncoords / 3;
    const uint64_t npolygons = nconnections > 0 ? nconnections / 3 : nvertices / 3;

    std::string x;
    x += "<?xml version=\"1.0\" ?>\n";
    x += "<!-- Generated by kvs::KVSMLPolygonObject::write() -->\n";
    x += "<KVSML>\n";
    x += "    <Object type=\"PolygonObject\">\n";
    x += std::string("        <PolygonObject polygon_type=\"triangle\" color_type=\"polygon\" normal_type=\"") +
         (vertex_normals ? "vertex" : "polygon") + "\">\n";

    std::vector<std::pair<std::string, ArrayOut>> externals;   // file name, array
    auto data_array = [&](const std::string& indent, const ArrayOut& a) -> kvsmc_status {
        const char* type = a.is_float ? "float" : "uint";
        if (writing_type == 0) {
            std::vector<uint32_t> h(a.n);
            if (a.n) {
                KVSMC_CUDA(ctx, cudaMemcpyAsync(h.data(), a.d, a.n * 4, cudaMemcpyDeviceToHost, ctx->stream));
                KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            }
            x += indent + "<DataArray type=\"" + type + "\">";
            x += a.is_float ? format_values(reinterpret_cast<const float*>(h.data()), a.n, " ")
                            : format_values(h.data(), a.n, " ");
            x += "\n" + indent + "</DataArray>\n";
        } else {
            const std::string file = base + "_" + a.kind + ".dat";
            x += indent + "<DataArray type=\"" + type + "\" format=\"" + (writing_type == 1 ? "ascii" : "binary") +
                 "\" file=\"" + file + "\"" + (writing_type == 2 ? " endian=\"little\"" : "") + " />\n";
            externals.push_back({dir + "/" + file, a});
        }
        return KVSMC_OK;
    };
    auto element = [&](const std::string& indent, const char* tag, const ArrayOut& a) -> kvsmc_status {
        if (a.n == 0) return KVSMC_OK;   // Write*Data write nothing for an empty array
        x += indent + "<" + tag + ">\n";
        kvsmc_status st = data_array(indent + "    ", a);
        if (st) return st;
        x += indent + "</" + tag + ">\n";
        return KVSMC_OK;
    };
    auto data_value = [&](const std::string& indent, const char* tag, const uint8_t* v, int n) {
        if (!v) return;
        x += indent + "<" + tag + ">\n" + indent + "    <DataValue>";
        for (int i = 0; i < n; ++i) x += std::to_string((int)v[i]) + " ";
        x += "\n" + indent + "    </DataValue>\n" + indent + "</" + tag + ">\n";
    };

    kvsmc_status st = KVSMC_OK;
    // an element without children prints as one empty-element tag
    auto close_parent = [&](size_t start, const std::string& open, const char* tag) {
        if (x.size() == start) x += "            <" + open + " />\n";
        else {
            x.insert(start, "            <" + open + ">\n");
            x += std::string("            </") + tag + ">\n";
        }
    };
    // <Vertex>: coordinates, and the normals when they are per vertex
    size_t start = x.size();
    if ((st = element("                ", "Coord", ArrayOut{d_coords, ncoords, 1, "coord"}))) return st;
    if (vertex_normals && (st = element("                ", "Normal", ArrayOut{d_normals, nnormals, 1, "normal"})))
        return st;
    close_parent(start, "Vertex nvertices=\"" + std::to_string(nvertices) + "\"", "Vertex");
    // <Polygon>: written since the colour type is polygon (KVSMLPolygonObject.cpp:436-437)
    start = x.size();
    if ((st = element("                ", "Connection", ArrayOut{d_connections, nconnections, 0, "connect"})))
        return st;
    data_value("                ", "Color", color, 3);
    data_value("                ", "Opacity", opacity, 1);
    if (!vertex_normals && (st = element("                ", "Normal", ArrayOut{d_normals, nnormals, 1, "normal"})))
        return st;
    close_parent(start, "Polygon npolygons=\"" + std::to_string(npolygons) + "\"", "Polygon");
    x += "        </PolygonObject>\n";
    x += "    </Object>\n";
    x += "</KVSML>\n";

    // external data files, in the order the writer makes them
    for (auto& ex : externals) {
        const ArrayOut& a = ex.second;
        FILE* f = std::fopen(ex.first.c_str(), "wb");
        if (!f) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: cannot open %s", ex.first.c_str());
        bool ok = true;
        if (writing_type == 1) {
            std::vector<uint32_t> h(a.n);
            cudaError_t e = cudaSuccess;
            if (a.n) e = cudaMemcpy(h.data(), a.d, a.n * 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                std::fclose(f);
                return fail(ctx, KVSMC_ERR_CUDA, "kvsml: %s", cudaGetErrorString(e));
            }
            const std::string s = a.is_float ? format_values(reinterpret_cast<const float*>(h.data()), a.n, ", ")
                                             : format_values(h.data(), a.n, ", ");
            ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
        } else {
            // raw little-endian words, through the context's two pinned staging
            // buffers: chunk i is copied while chunk i - 1 is written
            const size_t chunk = (size_t)64 << 20;
            const uint64_t bytes = a.n * 4;
            if (bytes && chunk > ctx->txt_bytes) {
                for (int b = 0; b < 2; ++b) {
                    if (ctx->txt_dbuf[b]) cudaFree(ctx->txt_dbuf[b]);
                    if (ctx->txt_hbuf[b]) cudaFreeHost(ctx->txt_hbuf[b]);
                    ctx->txt_dbuf[b] = nullptr;
                    ctx->txt_hbuf[b] = nullptr;
                }
                ctx->txt_bytes = 0;
                for (int b = 0; b < 2; ++b) {
                    if (cudaMalloc(&ctx->txt_dbuf[b], chunk) != cudaSuccess ||
                        cudaMallocHost(&ctx->txt_hbuf[b], chunk) != cudaSuccess ||
                        (!ctx->stl_ev[b] && cudaEventCreateWithFlags(&ctx->stl_ev[b], cudaEventDisableTiming) !=
                                                cudaSuccess)) {
                        std::fclose(f);
                        return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "kvsml: staging buffers");
                    }
                }
                ctx->txt_bytes = chunk;
            }
            const uint64_t nch = (bytes + chunk - 1) / chunk;
            cudaError_t e = cudaSuccess;
            for (uint64_t i = 0; i <= nch && ok && e == cudaSuccess; ++i) {
                if (i < nch) {
                    const int b = (int)(i & 1);
                    const uint64_t off = i * chunk, nb = std::min<uint64_t>(chunk, bytes - off);
                    e = cudaMemcpyAsync(ctx->txt_hbuf[b], static_cast<const char*>(a.d) + off, nb,
                                        cudaMemcpyDeviceToHost, ctx->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(ctx->stl_ev[b], ctx->stream);
                }
                if (i > 0 && e == cudaSuccess) {
                    const int b = (int)((i - 1) & 1);
                    const uint64_t off = (i - 1) * chunk, nb = std::min<uint64_t>(chunk, bytes - off);
                    e = cudaEventSynchronize(ctx->stl_ev[b]);
                    if (e == cudaSuccess) ok = std::fwrite(ctx->txt_hbuf[b], 1, nb, f) == nb;
                }
            }
            if (e != cudaSuccess) {
                std::fclose(f);
                cudaStreamSynchronize(ctx->stream);
                return fail(ctx, KVSMC_ERR_CUDA, "kvsml: %s", cudaGetErrorString(e));
            }
        }
        if (std::fclose(f) != 0 || !ok) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: writing %s failed",
                                                    ex.first.c_str());
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: cannot open %s", path);
    const bool ok = std::fwrite(x.data(), 1, x.size(), f) == x.size();
    if (std::fclose(f) != 0 || !ok) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "kvsml: writing %s failed", path);
    return KVSMC_OK;
}

}  // extern "C"
