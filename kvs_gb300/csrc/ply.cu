// ply.cu -- binary PLY files of triangle meshes, serialised on the GPU.
//
// What kvs::PolygonExporter<kvs::Ply>::exec (PolygonExporter.cpp:178-361)
// and kvs::Ply::write (Ply.cpp:389-488) with the Binary file type write for a
// mesh without connections: the header of ply_header_complete
// (PlyFile.cpp:399-460) -- "ply", the format line, "element vertex N" with
// the float x/y/z, uchar red/green/blue and float nx/ny/nz properties that
// are present, "element face 0" (the writer opens two elements and counts
// faces only from connections), "end_header" -- then one record per vertex:
// x, y, z, the colour when the mesh has one (its single colour repeated, or
// the vertex's own), the normal when the mesh has normals (zero for
// PolygonNormal meshes: the exporter averages polygon normals over the
// connections, of which there are none; the vertex's own for VertexNormal),
// little-endian, packed (27 bytes with both).
//
// One CTA per 256 vertices (grid-stride): the records are composed in shared
// memory and leave in 16-byte stores (256 records of 12, 15, 24 or 27 bytes
// are a multiple of 16 bytes).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "context.h"

namespace kvsmc {

namespace {

constexpr int kPlyThreads = 256;

__device__ __forceinline__ void put_f32(uint8_t* p, float v)
{
    const uint32_t u = __float_as_uint(v);
    p[0] = (uint8_t)u;
    p[1] = (uint8_t)(u >> 8);
    p[2] = (uint8_t)(u >> 16);
    p[3] = (uint8_t)(u >> 24);
}

__global__ void __launch_bounds__(kPlyThreads) k_ply_vertices(const float* coords, const uint8_t* colors,
                                                              int color_mode, const float* normals,
                                                              int normal_mode, uint64_t nverts, int rec,
                                                              uint8_t* out)
{
    extern __shared__ uint4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    for (uint64_t b = blockIdx.x; b * kPlyThreads < nverts; b += gridDim.x) {
        const uint64_t v0 = b * kPlyThreads;
        const uint32_t nb = (uint32_t)(nverts - v0 < (uint64_t)kPlyThreads ? nverts - v0 : kPlyThreads);
        if (threadIdx.x < nb) {
            const uint64_t v = v0 + threadIdx.x;
            uint8_t* r = sm + threadIdx.x * rec;
            put_f32(r, coords[3 * v]);
            put_f32(r + 4, coords[3 * v + 1]);
            put_f32(r + 8, coords[3 * v + 2]);
            int o = 12;
            if (color_mode) {
                const uint8_t* c = color_mode == 1 ? colors : colors + 3 * v;
                r[o] = c[0];
                r[o + 1] = c[1];
                r[o + 2] = c[2];
                o += 3;
            }
            if (normal_mode) {
                const float nx = normal_mode == 2 ? normals[3 * v] : 0.0f;
                const float ny = normal_mode == 2 ? normals[3 * v + 1] : 0.0f;
                const float nz = normal_mode == 2 ? normals[3 * v + 2] : 0.0f;
                put_f32(r + o, nx);
                put_f32(r + o + 4, ny);
                put_f32(r + o + 8, nz);
            }
        }
        __syncthreads();
        const uint32_t bytes = nb * (uint32_t)rec;
        uint8_t* dst = out + v0 * (uint64_t)rec;   // 16-byte aligned: 256 records are a multiple of 16 bytes
        const uint32_t words = bytes / 16;
        for (uint32_t w = threadIdx.x; w < words; w += kPlyThreads)
            reinterpret_cast<uint4*>(dst)[w] = smem4[w];
        for (uint32_t t = words * 16 + threadIdx.x; t < bytes; t += kPlyThreads) dst[t] = sm[t];
        __syncthreads();
    }
}

}  // namespace

int ply_record_bytes(int color_mode, int normal_mode)
{
    return 12 + (color_mode ? 3 : 0) + (normal_mode ? 12 : 0);
}

cudaError_t launch_ply_vertices(const float* coords, const uint8_t* colors, int color_mode, const float* normals,
                                int normal_mode, uint64_t nverts, uint8_t* out, const Launch& L)
{
    if (nverts == 0) return cudaSuccess;
    const int rec = ply_record_bytes(color_mode, normal_mode);
    const uint64_t blocks = (nverts + kPlyThreads - 1) / kPlyThreads;
    const uint64_t cap = (uint64_t)L.num_sms * 8;
    prof_begin(L, "ply_vertices");
    k_ply_vertices<<<(unsigned)(blocks < cap ? blocks : cap), kPlyThreads, kPlyThreads * rec, L.stream>>>(
        coords, colors, color_mode, normals, normal_mode, nverts, rec, out);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

kvsmc_status check_ply(kvsmc_context* ctx, const float* coords, uint64_t nvertices, const uint8_t* colors,
                       int32_t color_mode, const float* normals, int32_t normal_mode)
{
    if (color_mode < 0 || color_mode > 2 || normal_mode < 0 || normal_mode > 2)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "ply: bad colour / normal mode %d / %d", (int)color_mode,
                    (int)normal_mode);
    if (nvertices && (!coords || (color_mode && !colors) || (normal_mode == 2 && !normals)))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "ply: null mesh arrays");
    if (nvertices > 0x7fffffffull)
        return fail(ctx, KVSMC_ERR_TOO_LARGE, "ply: %llu vertices beyond the header's int count",
                    (unsigned long long)nvertices);
    return KVSMC_OK;
}

}  // namespace

extern "C" {

uint32_t kvsmc_ply_record_bytes(int32_t color_mode, int32_t normal_mode)
{
    return (uint32_t)kvsmc::ply_record_bytes(color_mode != 0, normal_mode != 0);
}

int64_t kvsmc_ply_header(uint64_t nvertices, int32_t color_mode, int32_t normal_mode, char* buf, uint64_t size)
{
    char h[512];
    int n = std::snprintf(h, sizeof h,
                          "ply\nformat binary_little_endian 1.0\nelement vertex %d\n"
                          "property float x\nproperty float y\nproperty float z\n%s%selement face 0\nend_header\n",
                          (int)nvertices,
                          color_mode ? "property uchar red\nproperty uchar green\nproperty uchar blue\n" : "",
                          normal_mode ? "property float nx\nproperty float ny\nproperty float nz\n" : "");
    if (n < 0) return -1;
    if (buf && size > (uint64_t)n) std::memcpy(buf, h, (size_t)n + 1);
    return n;
}

kvsmc_status kvsmc_ply_records(kvsmc_context* ctx, const float* d_coords, uint64_t nvertices, const uint8_t* d_colors,
                               int32_t color_mode, const float* d_normals, int32_t normal_mode, uint8_t* d_out)
{
    if (!ctx || (nvertices && !d_out)) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = check_ply(ctx, d_coords, nvertices, d_colors, color_mode, d_normals, normal_mode);
    if (st) return st;
    if (reinterpret_cast<uintptr_t>(d_out) & 15u)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "ply: the output must be 16-byte aligned");
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    KVSMC_CUDA(ctx, kvsmc::launch_ply_vertices(d_coords, d_colors, color_mode, d_normals, normal_mode, nvertices, d_out,
                                               kvsmc_host::launch_of(ctx)));
    return KVSMC_OK;
}

kvsmc_status kvsmc_write_ply(kvsmc_context* ctx, const char* path, const float* d_coords, uint64_t nvertices,
                             const uint8_t* d_colors, int32_t color_mode, const float* d_normals, int32_t normal_mode)
{
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = check_ply(ctx, d_coords, nvertices, d_colors, color_mode, d_normals, normal_mode);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const int rec = kvsmc::ply_record_bytes(color_mode, normal_mode);
    // chunks of 2^21 vertices, double-buffered through the context's export
    // staging buffers (the same pair the STL writer uses)
    const uint64_t chunk = 1ull << 21;
    const uint64_t nchunks = (nvertices + chunk - 1) / chunk;
    if (nchunks) {
        const size_t bytes = (size_t)(nvertices < chunk ? nvertices : chunk) * rec;
        if (bytes > ctx->stl_buf_bytes) {
            KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int b = 0; b < 2; ++b) {
                if (ctx->stl_dbuf[b]) cudaFree(ctx->stl_dbuf[b]);
                if (ctx->stl_hbuf[b]) cudaFreeHost(ctx->stl_hbuf[b]);
                ctx->stl_dbuf[b] = nullptr;
                ctx->stl_hbuf[b] = nullptr;
            }
            ctx->stl_buf_bytes = 0;
            for (int b = 0; b < 2; ++b) {
                KVSMC_CUDA(ctx, cudaMalloc(&ctx->stl_dbuf[b], bytes));
                KVSMC_CUDA(ctx, cudaMallocHost(&ctx->stl_hbuf[b], bytes));
                if (!ctx->stl_ev[b]) KVSMC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->stl_ev[b], cudaEventDisableTiming));
            }
            ctx->stl_buf_bytes = bytes;
        }
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "ply: cannot open %s", path);
    char header[512];
    const int64_t hn = kvsmc_ply_header(nvertices, color_mode, normal_mode, header, sizeof header);
    bool ok = hn > 0 && std::fwrite(header, 1, (size_t)hn, f) == (size_t)hn;
    const kvsmc::Launch L = kvsmc_host::launch_of(ctx);
    auto chunk_verts = [&](uint64_t i) { return (i + 1) * chunk <= nvertices ? chunk : nvertices - i * chunk; };
    cudaError_t e = cudaSuccess;
    for (uint64_t i = 0; i <= nchunks && e == cudaSuccess && ok; ++i) {
        if (i < nchunks) {
            const int b = (int)(i & 1);
            const uint64_t v0 = i * chunk, nv = chunk_verts(i);
            e = kvsmc::launch_ply_vertices(d_coords + 3 * v0, color_mode == 2 ? d_colors + 3 * v0 : d_colors,
                                           color_mode, normal_mode == 2 ? d_normals + 3 * v0 : d_normals, normal_mode,
                                           nv, static_cast<uint8_t*>(ctx->stl_dbuf[b]), L);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ctx->stl_hbuf[b], ctx->stl_dbuf[b], nv * rec, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ctx->stl_ev[b], ctx->stream);
        }
        if (i > 0 && e == cudaSuccess) {
            const int b = (int)((i - 1) & 1);
            e = cudaEventSynchronize(ctx->stl_ev[b]);
            if (e == cudaSuccess) {
                const size_t nb = chunk_verts(i - 1) * rec;
                ok = std::fwrite(ctx->stl_hbuf[b], 1, nb, f) == nb;
            }
        }
    }
    const bool closed = std::fclose(f) == 0;
    if (e != cudaSuccess) return fail(ctx, KVSMC_ERR_CUDA, "ply: %s", cudaGetErrorString(e));
    if (!ok || !closed) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "ply: writing %s failed", path);
    return KVSMC_OK;
}

kvsmc_status kvsmc_write_ply_host(kvsmc_context* ctx, const char* path, const float* coords, uint64_t nvertices,
                                  const uint8_t* colors, int32_t color_mode, const float* normals, int32_t normal_mode)
{
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = check_ply(ctx, coords, nvertices, colors, color_mode, normals, normal_mode);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bc = nvertices * 12, bk = color_mode == 2 ? nvertices * 3 : (color_mode ? 3 : 0),
                 bn = normal_mode == 2 ? nvertices * 12 : 0;
    char* d = nullptr;
    cudaError_t e = cudaSuccess;
    if (nvertices) {
        const size_t oc = kvsmc_host::align_up(bc, 256), ok_ = kvsmc_host::align_up(bk, 256);
        e = cudaMalloc(&d, oc + ok_ + bn + 16);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d, coords, bc, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && bk) e = cudaMemcpyAsync(d + oc, colors, bk, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && bn) e = cudaMemcpyAsync(d + oc + ok_, normals, bn, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            st = kvsmc_write_ply(ctx, path, reinterpret_cast<float*>(d), nvertices, reinterpret_cast<uint8_t*>(d + oc),
                                 color_mode, reinterpret_cast<float*>(d + oc + ok_), normal_mode);
    } else {
        st = kvsmc_write_ply(ctx, path, nullptr, 0, nullptr, color_mode, nullptr, normal_mode);
    }
    if (e != cudaSuccess)
        st = fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA, "ply: %s",
                  cudaGetErrorString(e));
    cudaStreamSynchronize(ctx->stream);
    if (d) cudaFree(d);
    return st;
}

}  // extern "C"
