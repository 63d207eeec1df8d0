// noalloc.cu -- kvsmc_extract_noalloc: one duplicated-vertex extraction that
// allocates no memory at all.
//
// Who needs it: code that runs inside a host application which owns the
// whole device-memory budget, or inside an interactive frame loop, where a
// cudaMalloc/cudaFree (which can synchronize the whole device) is not
// allowed or would stall the frame.  Such a caller brings its own volume and
// output buffers; everything else this call needs lives in a fixed static
// device array.
//
// The intermediates of the streaming kernels (work tables, one triangle
// count and one offset per tile, scan partials, status word) go into
// g_noalloc_scratch, a file-scope __device__ array of kNoAllocScratchBytes
// (4 MiB).  Every GPU that loads this library holds that array until the
// process exits.  A request whose intermediates do not fit is refused with
// KVSMC_ERR_TOO_LARGE (the limit covers volumes up to about 512^3: one u16
// count and one u32 offset per 256-cell row piece).
//
// In host code the name g_noalloc_scratch is only a host-side stand-in, not
// a device address, so the device address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the
// first call made on it.  That first call therefore must come before any
// stream capture is started on the calling thread.
//
// All calls share the array and it keeps the last call's contents: the
// status word is cleared each call, and everything else is fully rewritten
// before it is read.  Calls whose work overlaps on the GPU (different
// streams, or different host threads on one device) race on the array and
// must be serialized by the caller.
#include <cmath>
#include <cstring>
#include <mutex>

#include "batch.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 4u << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
char* g_scratch_addr[kMaxDevices];   // device address of the array, per device

// Device address of the scratch array on the current device (looked up once).
kvsmc_status scratch_address(char** out, int* device)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return KVSMC_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return KVSMC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return KVSMC_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<char*>(p);
    }
    *out = g_scratch_addr[dev];
    *device = dev;
    return KVSMC_OK;
}

bool equal_ref(double a, double b)
{
    const double d = a - b;
    return ((d < 0) ? -d : d) < 1.e-6;
}

}  // namespace

extern "C" kvsmc_status kvsmc_extract_noalloc(const void* d_values, kvsmc_dtype dtype, uint32_t nx, uint32_t ny,
                                              uint32_t nz, const kvsmc_params* p, float* d_coords,
                                              uint64_t coords_capacity, float* d_normals, uint64_t normals_capacity,
                                              void* stream, kvsmc_sizes* sizes)
{
    using namespace kvsmc;
    using kvsmc_host::align_up;
    if (!d_values || !p || !sizes) return KVSMC_ERR_INVALID_ARGUMENT;
    std::memset(sizes, 0, sizeof *sizes);
    if (p->mode != KVSMC_DUP_POLYGON_NORMAL) return KVSMC_ERR_INVALID_ARGUMENT;
    if (!(dtype == KVSMC_I8 || dtype == KVSMC_I16 || dtype == KVSMC_U8 || dtype == KVSMC_U16 || dtype == KVSMC_F32))
        return KVSMC_ERR_UNSUPPORTED_DTYPE;
    const size_t es = dtype_size(dtype);
    // rows are staged with bulk copies: they must start on 16-byte boundaries
    if (nx < 2 || ny < 2 || nz < 2 || nx - 1 > (uint32_t)kStreamMaxCells ||
        (reinterpret_cast<uintptr_t>(d_values) & 15u) || ((size_t)nx * es) % 16 != 0 || !std::isfinite(p->isolevel) ||
        std::fabs(p->isolevel) > 1.0e30)
        return KVSMC_ERR_INVALID_ARGUMENT;

    char* scratch = nullptr;
    int dev = 0;
    kvsmc_status st = scratch_address(&scratch, &dev);
    if (st) return st;
    int num_sms = 0;
    if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return KVSMC_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint64_t launches = 0;
    const Launch L{s, num_sms, &launches, nullptr};

    VolumeView v;
    v.data = d_values;
    v.nx = nx; v.ny = ny; v.nz = nz;
    v.dtype = dtype;
    v.pitch = nx;
    v.slice = (uint64_t)nx * ny;
    StreamGroup g;
    std::memset(&g, 0, sizeof g);
    g.vol = v;
    const int rows = kvsmc_host::stream_rows(nx - 1);
    g.rows = (uint32_t)rows;
    g.wpr = kvsmc_host::segments_per_row(v, rows);
    if (stream_shared_bytes(dtype, true, rows) > (size_t)227 * 1024 ||
        (double)(nx - 1) * (double)(ny - 1) * 5.0 >= 4294967295.0)
        return KVSMC_ERR_TOO_LARGE;
    const uint32_t cy = ny - 1, cz = nz - 1;
    const uint32_t cyr = (cy + rows - 1) / rows;
    g.zchunk = kvsmc_host::stream_zchunk((uint64_t)cz * cyr * g.wpr, num_sms);
    const uint64_t ntasks = kvsmc_host::stream_tasks(v, rows, g.wpr, g.zchunk);
    const uint64_t units = kvsmc_host::stream_units(v, g.wpr, 1);   // one isolevel: one counter per unit
    g.task_begin = 0;
    g.unit_base = 0;
    g.plane_begin = 0;
    g.seg_elems = (uint32_t)stream_row_elems(dtype, rows);
    g.seg_copy_bytes = g.seg_elems * (uint32_t)es;
    g.warp_smem_bytes = (uint32_t)stream_warp_smem_bytes(dtype, true, rows);
    g.warp_smem_offset = (uint32_t)stream_warp_smem_offset();

    // carve the static array
    size_t off = 0;
    auto take = [&](size_t bytes) { char* q = scratch + off; off = align_up(off + bytes, 256); return q; };
    StreamGroup* d_group = reinterpret_cast<StreamGroup*>(take(sizeof(StreamGroup)));
    StreamIso* d_iso = reinterpret_cast<StreamIso*>(take(sizeof(StreamIso)));
    uint16_t* d_unit_counts = reinterpret_cast<uint16_t*>(take(units * 2));
    uint32_t* d_unit_offsets = reinterpret_cast<uint32_t*>(take(units * 4));
    uint32_t* d_plane_totals = reinterpret_cast<uint32_t*>(take((size_t)cz * 4));
    uint64_t* d_plane_base = reinterpret_cast<uint64_t*>(take((size_t)cz * 8));
    void* d_scan = take(scan_scratch_bytes(cz));
    uint64_t* d_totals = reinterpret_cast<uint64_t*>(take(8));
    uint64_t* d_total = reinterpret_cast<uint64_t*>(take(8));
    int* d_status = reinterpret_cast<int*>(take(sizeof(int)));
    unsigned long long* d_next = reinterpret_cast<unsigned long long*>(take(2 * sizeof(unsigned long long)));
    double* d_mm = reinterpret_cast<double*>(take(2 * sizeof(double)));
    void* d_mm_part = take(minmax_scratch_bytes(num_sms));
    if (off > kNoAllocScratchBytes) return KVSMC_ERR_TOO_LARGE;

    // min/max: MapperBase::setRange (MapperBase.cpp:54-83)
    double vmin = p->min_value, vmax = p->max_value;
    if (!p->has_minmax) {
        double mm[2];
        if (launch_minmax(v, d_mm_part, d_mm, L) != cudaSuccess ||
            cudaMemcpyAsync(mm, d_mm, sizeof mm, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return KVSMC_ERR_CUDA;
        vmin = mm[0];
        vmax = mm[1];
    }
    sizes->min_value = vmin;
    sizes->max_value = vmax;
    if (equal_ref(vmin, vmax)) return KVSMC_OK;   // MarchingCubes.cpp:108-110
    sizes->extracted = 1;

    StreamIso iso;
    std::memset(&iso, 0, sizeof iso);
    iso.f = kvsmc_host::make_fast(p->isolevel, vmin, vmax, dtype);
    iso.ip.iso = p->isolevel;
    iso.ip.vmin = vmin;
    iso.ip.vmax = vmax;
    for (int k = 0; k < 3; ++k) { iso.ip.min_coord[k] = p->min_coord[k]; iso.ip.scale[k] = p->scale[k]; }
    iso.plane_index = 0;
    g.iso_begin = 0;
    g.niso = 1;
    kvsmc_host::bucket_params(iso.f.f_thr, iso.f.f_thr, g.bs, g.bo);

    // count -> unit scan -> plane scan -> total
    const int zero = 0;
    uint64_t total = 0;
    int status = 0;
    if (cudaMemcpyAsync(d_group, &g, sizeof g, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_iso, &iso, sizeof iso, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_status, &zero, sizeof zero, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(d_unit_counts, 0, units * sizeof(uint16_t), s) != cudaSuccess ||
        cudaMemsetAsync(d_next, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess ||
        launch_stream(false, dtype, rows, d_group, 1, ntasks, d_iso, d_unit_counts, nullptr, nullptr, d_status, d_next, L) !=
            cudaSuccess ||
        launch_unit_scan(d_group, 1, cz, d_iso, d_unit_counts, d_unit_offsets, d_plane_totals, L) != cudaSuccess ||
        launch_scan(d_plane_totals, d_plane_base, cz, d_scan, d_total, L) != cudaSuccess ||
        launch_iso_totals(d_iso, 1, d_plane_base, d_total, d_totals, L) != cudaSuccess ||
        cudaMemcpyAsync(&total, d_totals, sizeof total, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&status, d_status, sizeof status, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return KVSMC_ERR_CUDA;
    if (status) return KVSMC_ERR_TIMEOUT;
    sizes->ntriangles = total;
    sizes->nvertices = 3 * total;
    sizes->ncoords = 9 * total;
    sizes->nnormals = 3 * total;
    if (total == 0) return KVSMC_OK;
    if (sizes->ncoords > coords_capacity || sizes->nnormals > normals_capacity || !d_coords || !d_normals)
        return KVSMC_ERR_CAPACITY;

    // emit
    iso.coords = d_coords;
    iso.normals = d_normals;
    iso.cap_tris = total;
    if (cudaMemcpyAsync(d_iso, &iso, sizeof iso, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        launch_stream(true, dtype, rows, d_group, 1, ntasks, d_iso, d_unit_counts, d_unit_offsets, d_plane_base, d_status, d_next + 1, L) !=
            cudaSuccess ||
        cudaMemcpyAsync(&status, d_status, sizeof status, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return KVSMC_ERR_CUDA;
    return status ? KVSMC_ERR_TIMEOUT : KVSMC_OK;
}
