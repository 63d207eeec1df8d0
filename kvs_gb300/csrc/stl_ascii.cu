// stl_ascii.cu -- ASCII STL text of a device triangle mesh, formatted on the GPU.
//
// kvs::Stl's default file type is ASCII (Source/Core/FileFormat/STL/Stl.cpp:86);
// Stl::write_ascii (Stl.cpp:447-480) prints, after "solid Generated by KVS\n",
// per triangle
//     facet normal %f %f %f\n outer loop\n (vertex %f %f %f\n) x 3 endloop\n endfacet\n
// (each line without leading blanks) and "endsolid\n" at the end, the
// triangles being what PolygonExporter<kvs::Stl>::exec hands it
// (PolygonExporter.cpp:78-176: connections expanded, vertex normals averaged
// as (n0 + n1 + n2) / 3 in float).
//
// "%f" of a float (promoted to double) is its exact binary value rounded to a
// multiple of 10^-6, ties to even (the C library's correctly rounded
// conversion in the default rounding mode), a '-' for a set sign bit (also
// for -0 and for negative values that round to zero), "inf" / "nan" with the
// sign for non-finite values.  A float is m * 2^e with m < 2^24:
//   * e >= 0: an integer, printed exactly (multi-word decimal conversion when
//     it passes 2^64), fraction 000000;
//   * -44 <= e < 0: integer part m >> -e; the fraction r = m mod 2^-e scaled
//     by 10^6 fits 64 bits, rounded to nearest with ties to even;
//   * e < -44: |value| < 2^-21 < 0.5 * 10^-6, so it prints as (-)0.000000.
// Records have different lengths, so each chunk of triangles takes two passes:
// lengths, an exclusive scan (record offsets), then every thread writes its
// triangle's text at its offset.  The text goes to pinned host memory and the
// file in chunks, the next chunk formatted while the previous one is written.
#include <cstdio>
#include <cstring>

#include "context.h"

namespace kvsmc {

namespace {

constexpr int kAsciiThreads = 256;

// The decimal form of one float under "%f".
struct Fixed6 {
    uint32_t neg;     // sign character
    uint32_t kind;    // 0 finite, 1 inf, 2 nan
    uint64_t ip;      // integer part when it fits 64 bits
    uint32_t big;     // 1: integer part m << e passes 2^64 (printed from m, e)
    uint32_t m;
    int32_t e;
    uint32_t frac;    // six decimals
};

__device__ __forceinline__ Fixed6 fixed6(float f)
{
    Fixed6 d;
    const uint32_t b = __float_as_uint(f);
    d.neg = b >> 31;
    const uint32_t ex = (b >> 23) & 0xffu, mant = b & 0x7fffffu;
    d.kind = ex == 0xffu ? (mant ? 2u : 1u) : 0u;
    d.ip = 0;
    d.big = 0;
    d.frac = 0;
    d.m = ex ? (mant | 0x800000u) : mant;
    d.e = ex ? (int32_t)ex - 150 : -149;
    if (d.kind) return d;
    if (d.e >= 0) {
        if (d.e < 40) d.ip = (uint64_t)d.m << d.e;
        else d.big = 1;
        return d;
    }
    const int s = -d.e;
    if (s > 44) return d;   // below 2^-21: rounds to zero
    const uint64_t m = d.m;
    d.ip = s >= 24 ? 0 : (m >> s);
    const uint64_t r = s >= 24 ? m : (m & ((1ull << s) - 1));
    const uint64_t t = r * 1000000ull;            // < 2^64
    uint64_t q = t >> s;
    const uint64_t rem = t & ((1ull << s) - 1);
    const uint64_t half = 1ull << (s - 1);
    if (rem > half || (rem == half && (q & 1ull))) ++q;
    if (q == 1000000ull) {
        q = 0;
        ++d.ip;
    }
    d.frac = (uint32_t)q;
    return d;
}

__device__ __forceinline__ uint32_t digits64(uint64_t v)
{
    uint32_t n = 1;
    while (v >= 10) {
        v /= 10;
        ++n;
    }
    return n;
}

// Decimal digits of m * 2^e (e >= 40, m < 2^24: below 2^128) into buf,
// most significant first; returns the count.
__device__ uint32_t big_digits(uint32_t m, int32_t e, char* buf)
{
    // little-endian 32-bit words of m << e
    uint32_t w[5] = {0, 0, 0, 0, 0};
    const int word = e / 32, bit = e % 32;
    const uint64_t v = (uint64_t)m << bit;
    w[word] = (uint32_t)v;
    if (word + 1 < 5) w[word + 1] = (uint32_t)(v >> 32);
    char tmp[48];
    uint32_t n = 0;
    for (;;) {
        // divide by 10^9, collect the remainder's nine digits
        uint64_t rem = 0;
        bool zero = true;
        for (int i = 4; i >= 0; --i) {
            const uint64_t cur = (rem << 32) | w[i];
            w[i] = (uint32_t)(cur / 1000000000ull);
            rem = cur % 1000000000ull;
            zero = zero && w[i] == 0;
        }
        for (int k = 0; k < 9; ++k) {
            tmp[n++] = (char)('0' + rem % 10);
            rem /= 10;
        }
        if (zero) break;
    }
    while (n > 1 && tmp[n - 1] == '0') --n;   // leading zeros of the top group
    for (uint32_t i = 0; i < n; ++i) buf[i] = tmp[n - 1 - i];
    return n;
}

__device__ __forceinline__ uint32_t fixed6_len(const Fixed6& d)
{
    if (d.kind) return d.neg + 3;
    if (d.big) {
        char tmp[48];
        return d.neg + big_digits(d.m, d.e, tmp) + 7;
    }
    return d.neg + digits64(d.ip) + 7;
}

__device__ __forceinline__ char* put_str(char* p, const char* s)
{
    while (*s) *p++ = *s++;
    return p;
}

__device__ char* fixed6_put(char* p, const Fixed6& d)
{
    if (d.neg) *p++ = '-';
    if (d.kind == 1) return put_str(p, "inf");
    if (d.kind == 2) return put_str(p, "nan");
    if (d.big) {
        char tmp[48];
        const uint32_t n = big_digits(d.m, d.e, tmp);
        for (uint32_t i = 0; i < n; ++i) *p++ = tmp[i];
    } else {
        const uint32_t n = digits64(d.ip);
        uint64_t v = d.ip;
        for (int i = (int)n - 1; i >= 0; --i) {
            p[i] = (char)('0' + v % 10);
            v /= 10;
        }
        p += n;
    }
    *p++ = '.';
    uint32_t fr = d.frac;
    for (int i = 5; i >= 0; --i) {
        p[i] = (char)('0' + fr % 10);
        fr /= 10;
    }
    return p + 6;
}

// The 12 floats of triangle t as the exporter hands them to the writer:
// normal (3), then the three vertices.  bad_index: set when a connection is
// out of range (that vertex reads as vertex 0).
__device__ __forceinline__ void stl_triangle(const float* __restrict__ coords, const float* __restrict__ normals,
                                             const uint32_t* __restrict__ conn, uint64_t nverts, uint64_t t,
                                             int mode, int* __restrict__ bad_index, float v[12])
{
    if (mode == KVSMC_DUP_POLYGON_NORMAL) {
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] = normals[3 * t + k];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[3 + k] = coords[9 * t + k];
        return;
    }
    uint64_t id[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        id[c] = conn[3 * t + c];
        if (id[c] >= nverts) {
            atomicExch(bad_index, 1);
            id[c] = 0;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) v[3 + 3 * c + k] = coords[3 * id[c] + k];
    }
    if (mode == KVSMC_SHARED_POLYGON_NORMAL) {
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] = normals[3 * t + k];
    } else {
        // ( normal0 + normal1 + normal2 ) / 3.0f (PolygonExporter.cpp:141-147)
#pragma unroll
        for (int k = 0; k < 3; ++k)
            v[k] = __fdiv_rn(__fadd_rn(__fadd_rn(normals[3 * id[0] + k], normals[3 * id[1] + k]), normals[3 * id[2] + k]),
                             3.0f);
    }
}

// "facet normal " + 3 numbers + 2 blanks + "\n", "outer loop\n",
// 3 x ("vertex " + 2 blanks + "\n") around 9 numbers, "endloop\n", "endfacet\n"
constexpr uint32_t kFixedText = 13 + 3 + 11 + 3 * (7 + 3) + 8 + 9;

__global__ void __launch_bounds__(kAsciiThreads)
    k_stl_ascii_len(const float* __restrict__ coords, const float* __restrict__ normals,
                    const uint32_t* __restrict__ conn, uint64_t nverts, uint64_t t0, uint64_t n, int mode,
                    uint32_t* __restrict__ lens, int* __restrict__ bad_index)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float v[12];
        stl_triangle(coords, normals, conn, nverts, t0 + i, mode, bad_index, v);
        uint32_t len = kFixedText;
#pragma unroll
        for (int k = 0; k < 12; ++k) len += fixed6_len(fixed6(v[k]));
        lens[i] = len;
    }
}

__global__ void __launch_bounds__(kAsciiThreads)
    k_stl_ascii_write(const float* __restrict__ coords, const float* __restrict__ normals,
                      const uint32_t* __restrict__ conn, uint64_t nverts, uint64_t t0, uint64_t n, int mode,
                      const uint64_t* __restrict__ offsets, char* __restrict__ out, int* __restrict__ bad_index)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float v[12];
        stl_triangle(coords, normals, conn, nverts, t0 + i, mode, bad_index, v);
        char* p = out + offsets[i];
        p = put_str(p, "facet normal ");
        for (int k = 0; k < 3; ++k) {
            p = fixed6_put(p, fixed6(v[k]));
            *p++ = k < 2 ? ' ' : '\n';
        }
        p = put_str(p, "outer loop\n");
        for (int c = 0; c < 3; ++c) {
            p = put_str(p, "vertex ");
            for (int k = 0; k < 3; ++k) {
                p = fixed6_put(p, fixed6(v[3 + 3 * c + k]));
                *p++ = k < 2 ? ' ' : '\n';
            }
        }
        put_str(p, "endloop\nendfacet\n");
    }
}

}  // namespace

cudaError_t launch_stl_ascii_len(const float* coords, const float* normals, const uint32_t* conn, uint64_t nverts,
                                 uint64_t t0, uint64_t n, int mode, uint32_t* lens, int* bad_index, const Launch& L)
{
    if (n == 0) return cudaSuccess;
    const uint64_t want = (n + kAsciiThreads - 1) / kAsciiThreads;
    const unsigned blocks = (unsigned)(want < (uint64_t)L.num_sms * 16 ? want : (uint64_t)L.num_sms * 16);
    prof_begin(L, "stl_ascii_len");
    k_stl_ascii_len<<<blocks, kAsciiThreads, 0, L.stream>>>(coords, normals, conn, nverts, t0, n, mode, lens,
                                                             bad_index);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_stl_ascii_write(const float* coords, const float* normals, const uint32_t* conn,
                                   uint64_t nverts, uint64_t t0, uint64_t n, int mode, const uint64_t* offsets,
                                   char* out, int* bad_index, const Launch& L)
{
    if (n == 0) return cudaSuccess;
    const uint64_t want = (n + kAsciiThreads - 1) / kAsciiThreads;
    const unsigned blocks = (unsigned)(want < (uint64_t)L.num_sms * 16 ? want : (uint64_t)L.num_sms * 16);
    prof_begin(L, "stl_ascii_write");
    k_stl_ascii_write<<<blocks, kAsciiThreads, 0, L.stream>>>(coords, normals, conn, nverts, t0, n, mode, offsets,
                                                               out, bad_index);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

kvsmc_status ascii_check(kvsmc_context* ctx, int32_t mode, const float* d_coords, const float* d_normals,
                         const uint32_t* d_connections, uint64_t ntriangles)
{
    if (mode != KVSMC_DUP_POLYGON_NORMAL && mode != KVSMC_SHARED_POLYGON_NORMAL && mode != KVSMC_SHARED_VERTEX_NORMAL)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: bad mode %d", (int)mode);
    if (ntriangles && (!d_coords || !d_normals || (mode != KVSMC_DUP_POLYGON_NORMAL && !d_connections)))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: null mesh array");
    return KVSMC_OK;
}

// Grow-only text buffers of the ASCII writer: two device, two pinned.
kvsmc_status ascii_buffers(kvsmc_context* ctx, size_t bytes)
{
    if (bytes <= ctx->txt_bytes) return KVSMC_OK;
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int b = 0; b < 2; ++b) {
        if (ctx->txt_dbuf[b]) cudaFree(ctx->txt_dbuf[b]);
        if (ctx->txt_hbuf[b]) cudaFreeHost(ctx->txt_hbuf[b]);
        ctx->txt_dbuf[b] = nullptr;
        ctx->txt_hbuf[b] = nullptr;
    }
    ctx->txt_bytes = 0;
    const size_t want = kvsmc_host::align_up(bytes + bytes / 4, 1 << 20);
    for (int b = 0; b < 2; ++b) {
        KVSMC_CUDA(ctx, cudaMalloc(&ctx->txt_dbuf[b], want));
        KVSMC_CUDA(ctx, cudaMallocHost(&ctx->txt_hbuf[b], want));
        if (!ctx->stl_ev[b]) KVSMC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->stl_ev[b], cudaEventDisableTiming));
    }
    ctx->txt_bytes = want;
    return KVSMC_OK;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_write_stl_ascii(kvsmc_context* ctx, const char* path, int32_t mode, const float* d_coords,
                                   const float* d_normals, const uint32_t* d_connections, uint64_t nvertices,
                                   uint64_t ntriangles)
{
    using namespace kvsmc_host;
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = ascii_check(ctx, mode, d_coords, d_normals, d_connections, ntriangles);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const uint64_t chunk = 1ull << 20;
    const uint64_t nchunks = (ntriangles + chunk - 1) / chunk;
    const uint64_t first = ntriangles < chunk ? ntriangles : chunk;
    // per chunk: u32 lengths, u64 offsets, the scan's scratch and total, the bad-index word
    const size_t lens_b = align_up(first * 4, 256), offs_b = align_up(first * 8, 256);
    const size_t scan_b = align_up(kvsmc::scan_scratch_bytes(first ? first : 1), 256);
    if (nchunks && (st = ensure_scratch(ctx, lens_b + offs_b + scan_b + 512))) return st;
    char* base = static_cast<char*>(ctx->scratch);
    uint32_t* d_lens = reinterpret_cast<uint32_t*>(base);
    uint64_t* d_offs = reinterpret_cast<uint64_t*>(base + lens_b);
    void* d_scan = base + lens_b + offs_b;
    uint64_t* d_total = reinterpret_cast<uint64_t*>(base + lens_b + offs_b + scan_b);
    int* d_bad = reinterpret_cast<int*>(base + lens_b + offs_b + scan_b + 256);
    if (nchunks) KVSMC_CUDA(ctx, cudaMemsetAsync(d_bad, 0, sizeof(int), ctx->stream));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: cannot open %s", path);
    bool ok = std::fputs("solid Generated by KVS\n", f) >= 0;
    const kvsmc::Launch L = launch_of(ctx);
    size_t pending = 0;   // bytes of the previous chunk in its pinned buffer
    cudaError_t e = cudaSuccess;
    for (uint64_t i = 0; i <= nchunks && ok && e == cudaSuccess && st == KVSMC_OK; ++i) {
        size_t bytes = 0;
        if (i < nchunks) {
            const uint64_t t0 = i * chunk, nt = (i + 1) * chunk <= ntriangles ? chunk : ntriangles - t0;
            e = kvsmc::launch_stl_ascii_len(d_coords, d_normals, d_connections, nvertices, t0, nt, mode, d_lens,
                                            d_bad, L);
            if (e == cudaSuccess) e = kvsmc::launch_scan(d_lens, d_offs, nt, d_scan, d_total, L);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ctx->h_small, d_total, 8, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) break;
            bytes = (size_t)ctx->h_small[0];
            if ((st = ascii_buffers(ctx, bytes))) break;
            const int b = (int)(i & 1);
            e = kvsmc::launch_stl_ascii_write(d_coords, d_normals, d_connections, nvertices, t0, nt, mode, d_offs,
                                              ctx->txt_dbuf[b], d_bad, L);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ctx->txt_hbuf[b], ctx->txt_dbuf[b], bytes, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ctx->stl_ev[b], ctx->stream);
        }
        // the previous chunk's text, formatted and copied by now or soon, leaves for the file
        if (i > 0 && e == cudaSuccess && st == KVSMC_OK) {
            const int b = (int)((i - 1) & 1);
            e = cudaEventSynchronize(ctx->stl_ev[b]);
            if (e == cudaSuccess) ok = std::fwrite(ctx->txt_hbuf[b], 1, pending, f) == pending;
        }
        pending = bytes;
    }
    if (ok) ok = std::fputs("endsolid\n", f) >= 0;
    int was_bad = 0;
    if (e == cudaSuccess && st == KVSMC_OK && nchunks) {
        e = cudaMemcpyAsync(ctx->h_small, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) std::memcpy(&was_bad, ctx->h_small, sizeof(int));
    }
    const bool closed = std::fclose(f) == 0;
    if (st) return st;
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        return fail(ctx, KVSMC_ERR_CUDA, "stl: %s", cudaGetErrorString(e));
    }
    if (!ok || !closed) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: writing %s failed", path);
    if (was_bad) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: a connection index is >= nvertices");
    return KVSMC_OK;
}

kvsmc_status kvsmc_write_stl_ascii_host(kvsmc_context* ctx, const char* path, int32_t mode, const float* coords,
                                        uint64_t ncoords, const float* normals, uint64_t nnormals,
                                        const uint32_t* connections, uint64_t nconnections)
{
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    if (mode != KVSMC_DUP_POLYGON_NORMAL && mode != KVSMC_SHARED_POLYGON_NORMAL && mode != KVSMC_SHARED_VERTEX_NORMAL)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: bad mode %d", (int)mode);
    const bool dup = mode == KVSMC_DUP_POLYGON_NORMAL;
    const uint64_t ntri = dup ? ncoords / 9 : nconnections / 3;
    const uint64_t nverts = ncoords / 3;
    const uint64_t need_normals = mode == KVSMC_SHARED_VERTEX_NORMAL ? 3 * nverts : 3 * ntri;
    if (nnormals < need_normals || (ntri && (!coords || !normals || (!dup && !connections))))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: mesh arrays of inconsistent sizes");
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    float* d_c = nullptr;
    float* d_n = nullptr;
    uint32_t* d_k = nullptr;
    cudaError_t e = cudaSuccess;
    if (ntri) {
        e = cudaMalloc(&d_c, ncoords * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&d_n, need_normals * sizeof(float));
        if (e == cudaSuccess && !dup) e = cudaMalloc(&d_k, 3 * ntri * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, coords, ncoords * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_n, normals, need_normals * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && !dup)
            e = cudaMemcpyAsync(d_k, connections, 3 * ntri * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
    }
    kvsmc_status st = KVSMC_OK;
    if (e != cudaSuccess)
        st = fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA, "stl: %s",
                  cudaGetErrorString(e));
    else
        st = kvsmc_write_stl_ascii(ctx, path, mode, d_c, d_n, d_k, nverts, ntri);
    cudaStreamSynchronize(ctx->stream);
    if (d_c) cudaFree(d_c);
    if (d_n) cudaFree(d_n);
    if (d_k) cudaFree(d_k);
    return st;
}

}  // extern "C"
