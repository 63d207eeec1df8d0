// export.cu -- binary STL serialisation of a device triangle mesh.
//
// The records are what kvs::PolygonExporter<kvs::Stl>::exec
// (Source/Core/Visualization/Exporter/PolygonExporter.cpp:78-176) and
// kvs::Stl::write_binary (Source/Core/FileFormat/STL/Stl.cpp:490-540) write:
// per triangle its normal (3 floats), its three vertices (9 floats) and two
// zero bytes, 50 bytes, little-endian, after an 84-byte header (80 bytes
// "Generated by KVS" zero-padded, the uint32 triangle count).  Shared-vertex
// meshes are expanded through their connections; with vertex normals the
// triangle's normal is (n0 + n1 + n2) / 3 in float, in that order
// (PolygonExporter.cpp:133-152, kvs::Vector3 operator+ and operator/).
//
// Duplicated meshes with 16-byte aligned arrays: a persistent CTA walks tiles
// of 256 triangles through a two-stage pipeline of bulk asynchronous copies
// (TMA): the next tile's 9,216 coordinate and 3,072 normal bytes load into
// shared memory (mbarrier completion) while the current tile's 12,800 record
// bytes are composed there and leave by one bulk shared-to-global copy.  The
// last partial tile, shared-vertex meshes (gathers through the connections)
// and unaligned arrays take the plain kernel: coalesced loads, the records
// composed in shared memory, 16-byte stores (a tile's records start at a
// multiple of 12,800 bytes, so every store is aligned).  HBM-bound: 48 bytes
// read and 50 written per triangle for a duplicated mesh.
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.h"
#include "tma.cuh"

namespace kvsmc {

namespace {

constexpr int kStlTile = 256;
constexpr int kStlRecord = 50;

__device__ __forceinline__ void put_float(uint16_t* r, int slot, float f)
{
    const uint32_t b = __float_as_uint(f);
    r[2 * slot] = (uint16_t)(b & 0xffffu);
    r[2 * slot + 1] = (uint16_t)(b >> 16);
}

// mode: KVSMC_DUP_POLYGON_NORMAL / KVSMC_SHARED_POLYGON_NORMAL / KVSMC_SHARED_VERTEX_NORMAL.
__global__ void __launch_bounds__(kStlTile)
    k_stl_records(const float* __restrict__ coords, const float* __restrict__ normals,
                  const uint32_t* __restrict__ conn, uint64_t nverts, uint64_t ntri, int mode,
                  uint8_t* __restrict__ out, int* __restrict__ bad_index)
{
    __shared__ float sc[kStlTile * 9];
    __shared__ float sn[kStlTile * 3];
    __shared__ __align__(16) uint16_t rec[kStlTile * kStlRecord / 2];
    const unsigned tid = threadIdx.x;
    for (uint64_t tile = blockIdx.x; tile * kStlTile < ntri; tile += gridDim.x) {
        const uint64_t t0 = tile * kStlTile;
        const uint32_t n = (uint32_t)(ntri - t0 < (uint64_t)kStlTile ? ntri - t0 : (uint64_t)kStlTile);
        if (mode == KVSMC_DUP_POLYGON_NORMAL) {
            const float* cs = coords + 9 * t0;
            for (uint32_t i = tid; i < 9 * n; i += kStlTile) sc[i] = cs[i];
            const float* ns = normals + 3 * t0;
            for (uint32_t i = tid; i < 3 * n; i += kStlTile) sn[i] = ns[i];
        } else {
            // one (triangle, corner) per thread pass: its vertex through the connections
            const uint32_t* cn = conn + 3 * t0;
            for (uint32_t i = tid; i < 3 * n; i += kStlTile) {
                uint64_t v = cn[i];
                if (v >= nverts) {
                    atomicExch(bad_index, 1);
                    v = 0;
                }
                sc[3 * i + 0] = coords[3 * v + 0];
                sc[3 * i + 1] = coords[3 * v + 1];
                sc[3 * i + 2] = coords[3 * v + 2];
            }
            if (mode == KVSMC_SHARED_POLYGON_NORMAL) {
                const float* ns = normals + 3 * t0;
                for (uint32_t i = tid; i < 3 * n; i += kStlTile) sn[i] = ns[i];
            } else if (tid < n) {
                // ( normal0 + normal1 + normal2 ) / 3.0f, component by component
                uint64_t v0 = cn[3 * tid], v1 = cn[3 * tid + 1], v2 = cn[3 * tid + 2];
                v0 = v0 < nverts ? v0 : 0;
                v1 = v1 < nverts ? v1 : 0;
                v2 = v2 < nverts ? v2 : 0;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float s = __fadd_rn(__fadd_rn(normals[3 * v0 + k], normals[3 * v1 + k]), normals[3 * v2 + k]);
                    sn[3 * tid + k] = __fdiv_rn(s, 3.0f);
                }
            }
        }
        __syncthreads();
        if (tid < n) {
            uint16_t* r = rec + tid * (kStlRecord / 2);
#pragma unroll
            for (int k = 0; k < 3; ++k) put_float(r, k, sn[3 * tid + k]);
#pragma unroll
            for (int k = 0; k < 9; ++k) put_float(r, 3 + k, sc[9 * tid + k]);
            r[24] = 0;   // the unused 2-byte attribute
        }
        __syncthreads();
        const uint32_t bytes = (uint32_t)kStlRecord * n;
        uint8_t* dst = out + (uint64_t)kStlRecord * t0;
        const uint4* src4 = reinterpret_cast<const uint4*>(rec);
        uint4* dst4 = reinterpret_cast<uint4*>(dst);
        for (uint32_t i = tid; i < bytes / 16; i += kStlTile) dst4[i] = src4[i];
        const uint8_t* src1 = reinterpret_cast<const uint8_t*>(rec);
        for (uint32_t i = bytes / 16 * 16 + tid; i < bytes; i += kStlTile) dst[i] = src1[i];
        __syncthreads();
    }
}

// Shared memory of the pipelined kernel: two stages of tile inputs and of
// composed records, and one mbarrier per input stage.
struct StlPipe {
    float c[2][kStlTile * 9];
    float n[2][kStlTile * 3];
    uint16_t rec[2][kStlTile * kStlRecord / 2];
    uint64_t bar[2];
};

constexpr uint32_t kStlPollLimit = 1u << 22;

// Full tiles [0, ntiles) of a duplicated mesh; coords, normals, out 16-byte
// aligned.  status: set to 2 when a load did not complete within the poll
// limit (the CTA then drains its own copies and stops).
__global__ void __launch_bounds__(kStlTile)
    k_stl_records_tma(const float* __restrict__ coords, const float* __restrict__ normals, uint64_t ntiles,
                      uint8_t* __restrict__ out, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    StlPipe& P = *reinterpret_cast<StlPipe*>(smem_raw);
    const unsigned tid = threadIdx.x;
    constexpr uint32_t kInBytes = kStlTile * 12 * sizeof(float);
    auto issue = [&](uint64_t tile, int b) {
        mbar_arrive_expect_tx(&P.bar[b], kInBytes);
        bulk_copy_g2s(P.c[b], coords + (uint64_t)kStlTile * 9 * tile, kStlTile * 9 * sizeof(float), &P.bar[b]);
        bulk_copy_g2s(P.n[b], normals + (uint64_t)kStlTile * 3 * tile, kStlTile * 3 * sizeof(float), &P.bar[b]);
    };
    if (tid == 0) {
        mbar_init(&P.bar[0], 1);
        mbar_init(&P.bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    uint64_t tile = blockIdx.x;
    if (tid == 0 && tile < ntiles) issue(tile, 0);
    uint32_t ph = 0;            // per input stage: parity of its next completion
    uint32_t pending = 0;       // per input stage: a load was issued and not yet waited for
    if (tile < ntiles) pending = 1u;
    for (uint32_t k = 0; tile < ntiles; tile += gridDim.x, ++k) {
        const int b = (int)(k & 1u);
        const uint64_t next = tile + gridDim.x;
        if (tid == 0 && next < ntiles) {
            fence_proxy_async();   // the stage was read by every thread in the previous step
            issue(next, b ^ 1);
        }
        if (next < ntiles) pending |= 1u << (b ^ 1);
        const bool ok = mbar_wait(&P.bar[b], (ph >> b) & 1u, kStlPollLimit);
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(status, 2);
            break;
        }
        ph ^= 1u << b;
        pending &= ~(1u << b);
        // this stage's records were handed to a bulk store two steps ago
        if (tid == 0) bulk_wait_read<1>();
        __syncthreads();
        uint16_t* r = P.rec[b] + tid * (kStlRecord / 2);
#pragma unroll
        for (int j = 0; j < 3; ++j) put_float(r, j, P.n[b][3 * tid + j]);
#pragma unroll
        for (int j = 0; j < 9; ++j) put_float(r, 3 + j, P.c[b][9 * tid + j]);
        r[24] = 0;
        fence_proxy_async();   // the records, written by this thread, are read by the async proxy
        __syncthreads();
        if (tid == 0) {
            bulk_copy_s2g(out + (uint64_t)kStlTile * kStlRecord * tile, P.rec[b], kStlTile * kStlRecord);
            bulk_commit();
        }
    }
    if (tid == 0) {
        // after a timeout: the loads still in flight land (bounded) before the CTA exits
        for (int b = 0; b < 2; ++b)
            if ((pending >> b) & 1u) mbar_wait(&P.bar[b], (ph >> b) & 1u, kStlPollLimit);
        bulk_wait<0>();
    }
}

}  // namespace

cudaError_t launch_stl_records(const float* coords, const float* normals, const uint32_t* conn, uint64_t nverts,
                               uint64_t ntri, int mode, uint8_t* out, int* bad_index, const Launch& L)
{
    if (ntri == 0) return cudaSuccess;
    prof_begin(L, "stl_records");
    uint64_t done = 0;
    cudaError_t e = cudaSuccess;
    const bool aligned = ((reinterpret_cast<uintptr_t>(coords) | reinterpret_cast<uintptr_t>(normals) |
                           reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
    if (mode == KVSMC_DUP_POLYGON_NORMAL && aligned && ntri >= (uint64_t)kStlTile) {
        const uint64_t full = ntri / kStlTile;
        const int smem = (int)sizeof(StlPipe);
        e = cudaFuncSetAttribute(k_stl_records_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stl_records_tma, kStlTile, smem);
        if (e == cudaSuccess) {
            const uint64_t cap = (uint64_t)(per_sm > 0 ? per_sm : 1) * L.num_sms;
            k_stl_records_tma<<<(unsigned)(full < cap ? full : cap), kStlTile, smem, L.stream>>>(coords, normals, full,
                                                                                              out, bad_index);
            e = cudaGetLastError();
            *L.counter += 1;
        }
        done = full * kStlTile;
    }
    if (e == cudaSuccess && done < ntri) {
        const uint64_t rest = ntri - done;
        const uint64_t tiles = (rest + kStlTile - 1) / kStlTile;
        // resident CTAs: 25 KB of shared memory and 256 threads each, a few per SM
        const uint64_t cap = (uint64_t)L.num_sms * 8;
        const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
        const bool dup = mode == KVSMC_DUP_POLYGON_NORMAL;
        k_stl_records<<<grid, kStlTile, 0, L.stream>>>(dup ? coords + 9 * done : coords,
                                                       (mode == KVSMC_SHARED_VERTEX_NORMAL) ? normals
                                                                                            : normals + 3 * done,
                                                       dup ? conn : conn + 3 * done, nverts, rest, mode,
                                                       out + kStlRecord * done, bad_index);
        e = cudaGetLastError();
        *L.counter += 1;
    }
    prof_end(L);
    return e;
}

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

kvsmc_status check_mesh(kvsmc_context* ctx, int32_t mode, const float* d_coords, const float* d_normals,
                        const uint32_t* d_connections, uint64_t ntriangles)
{
    if (mode != KVSMC_DUP_POLYGON_NORMAL && mode != KVSMC_SHARED_POLYGON_NORMAL && mode != KVSMC_SHARED_VERTEX_NORMAL)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: bad mode %d", (int)mode);
    if (ntriangles && (!d_coords || !d_normals || (mode != KVSMC_DUP_POLYGON_NORMAL && !d_connections)))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: null mesh array");
    return KVSMC_OK;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_stl_records(kvsmc_context* ctx, int32_t mode, const float* d_coords, const float* d_normals,
                               const uint32_t* d_connections, uint64_t nvertices, uint64_t ntriangles, void* d_out)
{
    if (!ctx) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = check_mesh(ctx, mode, d_coords, d_normals, d_connections, ntriangles);
    if (st) return st;
    if (ntriangles == 0) return KVSMC_OK;
    if (!d_out || (reinterpret_cast<uintptr_t>(d_out) & 15u))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: output must be 16-byte aligned device memory");
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->d_flag) KVSMC_CUDA(ctx, cudaMalloc(&ctx->d_flag, sizeof(int)));
    int* bad = ctx->d_flag;
    KVSMC_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
    KVSMC_CUDA(ctx, kvsmc::launch_stl_records(d_coords, d_normals, d_connections, nvertices, ntriangles, mode,
                                              static_cast<uint8_t*>(d_out), bad, kvsmc_host::launch_of(ctx)));
    int h_bad = 0;
    KVSMC_CUDA(ctx, cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_bad == 2) return fail(ctx, KVSMC_ERR_TIMEOUT, "stl: a shared-memory load did not complete");
    if (h_bad) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: a connection index is >= nvertices");
    return KVSMC_OK;
}

kvsmc_status kvsmc_write_stl(kvsmc_context* ctx, const char* path, int32_t mode, const float* d_coords,
                             const float* d_normals, const uint32_t* d_connections, uint64_t nvertices,
                             uint64_t ntriangles)
{
    if (!ctx || !path) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_status st = check_mesh(ctx, mode, d_coords, d_normals, d_connections, ntriangles);
    if (st) return st;
    if (ntriangles > 0xffffffffull)
        return fail(ctx, KVSMC_ERR_TOO_LARGE, "stl: %llu triangles do not fit the format's 32-bit count",
                    (unsigned long long)ntriangles);
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    // chunks of 2^20 triangles, double-buffered through the context's staging
    // buffers: chunk i is serialised and copied while chunk i - 1 is written
    const uint64_t chunk = 1ull << 20;
    const uint64_t nchunks = (ntriangles + chunk - 1) / chunk;
    if (nchunks) {
        const size_t bytes = (size_t)(ntriangles < chunk ? ntriangles : chunk) * kvsmc::kStlRecordBytes;
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
        if (!ctx->d_flag) KVSMC_CUDA(ctx, cudaMalloc(&ctx->d_flag, sizeof(int)));
        if (!ctx->h_flag) KVSMC_CUDA(ctx, cudaMallocHost(&ctx->h_flag, sizeof(int)));
        KVSMC_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: cannot open %s", path);
    char header[84];
    std::memset(header, 0, sizeof header);
    std::snprintf(header, 80, "Generated by KVS");
    const uint32_t count = (uint32_t)ntriangles;
    std::memcpy(header + 80, &count, 4);   // little-endian host (x86-64, aarch64)
    bool ok = std::fwrite(header, 1, 84, f) == 84;
    const kvsmc::Launch L = kvsmc_host::launch_of(ctx);
    auto chunk_tris = [&](uint64_t i) { return (i + 1) * chunk <= ntriangles ? chunk : ntriangles - i * chunk; };
    cudaError_t e = cudaSuccess;
    for (uint64_t i = 0; i <= nchunks && e == cudaSuccess && ok; ++i) {
        if (i < nchunks) {
            const int b = (int)(i & 1);
            const uint64_t t0 = i * chunk, nt = chunk_tris(i);
            const float* c = mode == KVSMC_DUP_POLYGON_NORMAL ? d_coords + 9 * t0 : d_coords;
            const float* nrm = mode == KVSMC_SHARED_VERTEX_NORMAL ? d_normals : d_normals + 3 * t0;
            const uint32_t* cn = mode == KVSMC_DUP_POLYGON_NORMAL ? nullptr : d_connections + 3 * t0;
            // the host buffer of this parity was written out before (chunk i - 2)
            e = kvsmc::launch_stl_records(c, nrm, cn, nvertices, nt, mode, ctx->stl_dbuf[b], ctx->d_flag, L);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ctx->stl_hbuf[b], ctx->stl_dbuf[b], nt * kvsmc::kStlRecordBytes,
                                    cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ctx->stl_ev[b], ctx->stream);
        }
        if (i > 0 && e == cudaSuccess) {
            const int b = (int)((i - 1) & 1);
            e = cudaEventSynchronize(ctx->stl_ev[b]);
            if (e == cudaSuccess) {
                const size_t nb = chunk_tris(i - 1) * kvsmc::kStlRecordBytes;
                ok = std::fwrite(ctx->stl_hbuf[b], 1, nb, f) == nb;
            }
        }
    }
    int was_bad = 0;
    if (e == cudaSuccess && nchunks) {
        e = cudaMemcpyAsync(ctx->h_flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) was_bad = *ctx->h_flag;
    }
    const bool closed = std::fclose(f) == 0;
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        return fail(ctx, KVSMC_ERR_CUDA, "stl: %s", cudaGetErrorString(e));
    }
    if (!ok || !closed) {
        cudaStreamSynchronize(ctx->stream);
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: writing %s failed", path);
    }
    if (was_bad == 2) return fail(ctx, KVSMC_ERR_TIMEOUT, "stl: a shared-memory load did not complete");
    if (was_bad) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "stl: a connection index is >= nvertices");
    return KVSMC_OK;
}

kvsmc_status kvsmc_write_stl_host(kvsmc_context* ctx, const char* path, int32_t mode, const float* coords,
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
        st = kvsmc_write_stl(ctx, path, mode, d_c, d_n, d_k, nverts, ntri);
    cudaStreamSynchronize(ctx->stream);
    if (d_c) cudaFree(d_c);
    if (d_n) cudaFree(d_n);
    if (d_k) cudaFree(d_k);
    return st;
}

}  // extern "C"
