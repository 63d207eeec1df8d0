/* Test-only stand-in for libkvsmc's structured-volume entry points, answered
 * on the CPU by the oracle's restatement of the reference (oracle/mc_oracle.c),
 * so that the KVS drop-in classes' host logic (what they hand to the C ABI and
 * what they make of its answer) can be compared in one process with the
 * reference's own kvs::MarchingCubes and kvs::Isosurface where no GPU is
 * present.  Only tests link it; the entry points the comparison does not use
 * answer KVSMC_ERR_NO_DEVICE. */
#include "../../oracle/mc_oracle.c"

#include "kvsmc.h"

struct kvsmc_context { int unused; };
struct kvsmc_volume { int dtype; uint64_t n; void* values; };

static size_t elem_size(int dtype)
{
    static const size_t s[] = { 1, 2, 4, 8, 1, 2, 4, 8, 4, 8 };
    return (dtype >= 0 && dtype < 10) ? s[dtype] : 0;
}

kvsmc_status kvsmc_create(int device, kvsmc_context** ctx)
{
    (void)device;
    *ctx = (kvsmc_context*)calloc(1, sizeof(kvsmc_context));
    return *ctx ? KVSMC_OK : KVSMC_ERR_OUT_OF_MEMORY;
}

void kvsmc_destroy(kvsmc_context* ctx) { free(ctx); }

const char* kvsmc_status_string(kvsmc_status st) { return st == KVSMC_OK ? "ok" : "not in the test stand-in"; }

const char* kvsmc_last_error(const kvsmc_context* ctx)
{
    (void)ctx;
    return "";
}

kvsmc_status kvsmc_marching_cubes_host(kvsmc_context* ctx, const void* host_values, kvsmc_dtype dtype,
                                       uint32_t nx, uint32_t ny, uint32_t nz, const kvsmc_params* p,
                                       kvsmc_host_alloc_fn alloc, void* alloc_user, kvsmc_sizes* sizes)
{
    (void)ctx;
    const uint64_t n = (uint64_t)nx * ny * nz;
    if (!host_values || !p || !sizes || n == 0 || !elem_size((int)dtype)) return KVSMC_ERR_INVALID_ARGUMENT;
    double vmin = p->min_value, vmax = p->max_value;
    if (!p->has_minmax) mco_minmax((int)dtype, host_values, n, &vmin, &vmax);
    memset(sizes, 0, sizeof(*sizes));
    sizes->min_value = vmin;
    sizes->max_value = vmax;
    if (absd(vmin - vmax) < 1.e-6) return KVSMC_OK;   /* Math::Equal(min, max): nothing extracted */
    sizes->extracted = 1;
    mco_output o;
    memset(&o, 0, sizeof o);
    if (mco_extract((int)dtype, host_values, nx, ny, nz, p->isolevel, p->mode, vmin, vmax, p->min_coord, p->scale,
                    &o))
        return KVSMC_ERR_OUT_OF_MEMORY;
    sizes->ncoords = o.ncoords;
    sizes->nnormals = o.nnormals;
    sizes->nconnections = o.nconnections;
    sizes->ntriangles = p->mode == KVSMC_DUP_POLYGON_NORMAL ? o.ncoords / 9 : o.nconnections / 3;
    sizes->nvertices = o.ncoords / 3;
    kvsmc_status st = KVSMC_OK;
    const void* src[3] = { o.coords, o.normals, o.connections };
    const uint64_t count[3] = { o.ncoords, o.nnormals, o.nconnections };
    for (int which = 0; which < 3 && st == KVSMC_OK; ++which) {
        if (!count[which]) continue;
        void* dst = alloc(alloc_user, which, count[which]);
        if (!dst) st = KVSMC_ERR_OUT_OF_MEMORY;
        else memcpy(dst, src[which], 4 * count[which]);
    }
    mco_free(&o);
    return st;
}

kvsmc_status kvsmc_volume_upload(kvsmc_context* ctx, const void* host_values, kvsmc_dtype dtype, uint32_t nx,
                                 uint32_t ny, uint32_t nz, kvsmc_volume** vol)
{
    (void)ctx;
    const uint64_t n = (uint64_t)nx * ny * nz;
    const size_t es = elem_size((int)dtype);
    if (!host_values || !vol || n == 0 || !es) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_volume* v = (kvsmc_volume*)calloc(1, sizeof(kvsmc_volume));
    if (!v || !(v->values = malloc(n * es))) {
        free(v);
        return KVSMC_ERR_OUT_OF_MEMORY;
    }
    memcpy(v->values, host_values, n * es);
    v->dtype = (int)dtype;
    v->n = n;
    *vol = v;
    return KVSMC_OK;
}

kvsmc_status kvsmc_volume_minmax(kvsmc_context* ctx, kvsmc_volume* vol, double* min_value, double* max_value)
{
    (void)ctx;
    if (!vol) return KVSMC_ERR_INVALID_ARGUMENT;
    mco_minmax(vol->dtype, vol->values, vol->n, min_value, max_value);
    return KVSMC_OK;
}

void kvsmc_volume_free(kvsmc_context* ctx, kvsmc_volume* vol)
{
    (void)ctx;
    if (vol) free(vol->values);
    free(vol);
}

kvsmc_status kvsmc_marching_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                       kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                       const uint32_t* connections, uint64_t ncells, double isolevel,
                                       int32_t has_minmax, double min_value, double max_value,
                                       kvsmc_host_alloc_fn alloc, void* user, kvsmc_sizes* sizes)
{
    return KVSMC_ERR_NO_DEVICE;
}

kvsmc_status kvsmc_cells_bounds(kvsmc_context* ctx, kvsmc_cell_type cell_type, const float* coords, uint64_t nnodes,
                                const uint32_t* connections, uint64_t ncells, float* min_coord, float* max_coord)
{
    return KVSMC_ERR_NO_DEVICE;
}

kvsmc_status kvsmc_slice_plane(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles)
{
    return KVSMC_ERR_NO_DEVICE;
}

kvsmc_status kvsmc_slice_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                    kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                    const uint32_t* connections, uint64_t ncells, const kvsmc_slice_params* p,
                                    kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles)
{
    return KVSMC_ERR_NO_DEVICE;
}
