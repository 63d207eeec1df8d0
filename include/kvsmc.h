/*
 * kvsmc.h -- C ABI of the GB300 structured-grid marching-cubes library
 * (libkvsmc.so, CUDA for sm_103a).
 *
 * This is the boundary under kvs::cuda::MarchingCubes, the drop-in for the
 * reference mapper kvs::MarchingCubes
 * (Source/Core/Visualization/Mapper/MarchingCubes.h:23-62).  Plain pointers
 * and sizes only; every call returns a kvsmc_status and never aborts.
 *
 * Data model (the reference's, unchanged):
 *   volume values: nx*ny*nz scalars, x fastest, then y, then z
 *     (index = x + y*nx + z*nx*ny, MarchingCubes.cpp:162-164,187-194);
 *   output, duplicated mode: coords float[9*T] (three vertices per triangle),
 *     normals float[3*T] (one per triangle), no connections
 *     (MarchingCubes.cpp:156-243);
 *   output, shared-vertex modes: coords float[3*V], connections uint32[3*T],
 *     normals float[3*T] (polygon) or float[3*V] (vertex)
 *     (MarchingCubes.cpp:252-290).
 * Triangles come out in the reference's cell order (z, y, x with x fastest)
 * and in table order inside a cell, with the same vertex order and the same
 * float bits.
 */
#ifndef KVSMC_H
#define KVSMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KVSMC_VERSION_MAJOR 1
#define KVSMC_VERSION_MINOR 0

typedef enum kvsmc_status {
    KVSMC_OK = 0,
    KVSMC_ERR_INVALID_ARGUMENT = 1,  /* null pointer, zero-sized volume, bad enum   */
    KVSMC_ERR_UNSUPPORTED_DTYPE = 2, /* MarchingCubes.cpp:125-130                   */
    KVSMC_ERR_OUT_OF_MEMORY = 3,     /* device or pinned allocation failed          */
    KVSMC_ERR_CUDA = 4,              /* a CUDA runtime call failed (see last_error) */
    KVSMC_ERR_NO_DEVICE = 5,         /* no usable CUDA device                       */
    KVSMC_ERR_CAPACITY = 6,          /* caller buffer too small; sizes are returned */
    KVSMC_ERR_TOO_LARGE = 7,         /* result does not fit the 32-bit vertex ids   */
    KVSMC_ERR_TIMEOUT = 8,           /* a bounded device-side wait gave up          */
    KVSMC_ERR_BUDGET = 9             /* serving: request larger than the budget     */
} kvsmc_status;

/* Scalar types, numbered as the reference's type switch (MarchingCubes.cpp:115-124). */
typedef enum kvsmc_dtype {
    KVSMC_I8 = 0, KVSMC_I16 = 1, KVSMC_I32 = 2, KVSMC_I64 = 3,
    KVSMC_U8 = 4, KVSMC_U16 = 5, KVSMC_U32 = 6, KVSMC_U64 = 7,
    KVSMC_F32 = 8, KVSMC_F64 = 9
} kvsmc_dtype;

/* Extraction modes: the reference's (duplication, normal type) combinations.
 * VertexNormal forces shared vertices (MarchingCubes.cpp:69-73). */
typedef enum kvsmc_mode {
    KVSMC_DUP_POLYGON_NORMAL = 0,    /* duplication=true,  PolygonNormal */
    KVSMC_SHARED_POLYGON_NORMAL = 1, /* duplication=false, PolygonNormal */
    KVSMC_SHARED_VERTEX_NORMAL = 2   /* VertexNormal (either duplication) */
} kvsmc_mode;

/* Unstructured cell types of the marching mappers (the reference's
 * UnstructuredVolumeObject::CellType Tetrahedra, Hexahedra, Pyramid, Prism). */
typedef enum kvsmc_cell_type {
    KVSMC_TETRAHEDRA = 0, KVSMC_HEXAHEDRA = 1, KVSMC_PYRAMID = 2, KVSMC_PRISM = 3
} kvsmc_cell_type;

typedef struct kvsmc_context kvsmc_context;
typedef struct kvsmc_volume kvsmc_volume;

/* Per-request parameters.  min/max and the coordinate transform are decided by
 * the host layer exactly as MapperBase::setRange / setMinMaxCoords do
 * (MapperBase.cpp:54-122); the library only applies them. */
typedef struct kvsmc_params {
    double isolevel;       /* MarchingCubes::m_isolevel                          */
    int32_t mode;          /* kvsmc_mode                                         */
    int32_t has_minmax;    /* 1: use min_value/max_value; 0: use the volume's
                              device-computed min/max (GetMinMaxValues,
                              StructuredVolumeObject.cpp:66-85)                 */
    double min_value;      /* clamp range of interpolate_vertex (:347-348)       */
    double max_value;
    float min_coord[3];    /* volume->minObjectCoord()      (MarchingCubes.cpp:166) */
    float scale[3];        /* (max_coord-min_coord)/ncells  (MarchingCubes.cpp:168) */
} kvsmc_params;

/* Sizes of one extraction (counts of elements, not bytes). */
typedef struct kvsmc_sizes {
    uint64_t ntriangles;
    uint64_t nvertices;     /* 3*T in duplicated mode                             */
    uint64_t ncoords;       /* floats                                             */
    uint64_t nnormals;      /* floats                                             */
    uint64_t nconnections;  /* uint32 (0 in duplicated mode)                      */
    double min_value;       /* min/max actually used                              */
    double max_value;
    int32_t extracted;      /* 0: Math::Equal(min,max) early exit (MarchingCubes.cpp:108-110) */
    int32_t reserved;
} kvsmc_sizes;

/* ------------------------------------------------------------------ context */

/* One context per (host thread, device).  Owns a CUDA stream, the scratch
 * arena and the device-resident volumes.  device < 0 picks the current one. */
kvsmc_status kvsmc_create(int device, kvsmc_context** ctx);
void kvsmc_destroy(kvsmc_context* ctx);
const char* kvsmc_status_string(kvsmc_status st);
/* Text of the last error on this context ("" if none). */
const char* kvsmc_last_error(const kvsmc_context* ctx);
/* The context's CUDA stream (a cudaStream_t), for event timing by callers. */
void* kvsmc_stream(kvsmc_context* ctx);
/* Run all later work of this context on a caller stream (NULL = own stream). */
kvsmc_status kvsmc_set_stream(kvsmc_context* ctx, void* cuda_stream);
kvsmc_status kvsmc_synchronize(kvsmc_context* ctx);
/* Number of kernels this context has launched since creation. */
uint64_t kvsmc_kernel_launches(const kvsmc_context* ctx);
/* Kernel family: 0 (default) = streaming kernels for requests on 8/16-bit and
 * float32 volumes (duplicated mode; in the shared-vertex modes the node and
 * connection passes), gather kernels for the rest; 1 = gather kernels for
 * everything.  Both give identical results.  No counterpart in the reference
 * (which has one CPU loop). */
kvsmc_status kvsmc_set_kernel_path(kvsmc_context* ctx, int32_t path);

/* ------------------------------------------------------------------ volumes */

/* Copy a host volume (x fastest) into a device-resident, row-padded buffer.
 * Replaces the borrowed StructuredVolumeObject values of MapperBase::attachVolume
 * (MapperBase.h:54) with a resident device copy. */
kvsmc_status kvsmc_volume_upload(kvsmc_context* ctx, const void* host_values, kvsmc_dtype dtype,
                                 uint32_t nx, uint32_t ny, uint32_t nz, kvsmc_volume** vol);
/* Same, from a dense device buffer (x fastest, no padding). */
kvsmc_status kvsmc_volume_from_device(kvsmc_context* ctx, const void* dev_values, kvsmc_dtype dtype,
                                      uint32_t nx, uint32_t ny, uint32_t nz, kvsmc_volume** vol);
/* Overwrite the values of an existing volume from host memory (same shape/type). */
kvsmc_status kvsmc_volume_update(kvsmc_context* ctx, kvsmc_volume* vol, const void* host_values);
void kvsmc_volume_free(kvsmc_context* ctx, kvsmc_volume* vol);
/* Copy a volume's values back to host memory (dense, x fastest). */
kvsmc_status kvsmc_volume_download(kvsmc_context* ctx, const kvsmc_volume* vol, void* host_values);
/* Min/max of the values, computed on the device once and cached
 * (StructuredVolumeObject::updateMinMaxValues, StructuredVolumeObject.cpp:431-450). */
kvsmc_status kvsmc_volume_minmax(kvsmc_context* ctx, kvsmc_volume* vol, double* min_value, double* max_value);

/* ------------------------------------------------------------- extraction */

/* Count pass: exact output sizes for one request (no output written). */
kvsmc_status kvsmc_count(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p, kvsmc_sizes* sizes);

/* Count + emit into caller-provided DEVICE buffers.  Capacities are element
 * counts; on KVSMC_ERR_CAPACITY nothing is written and *sizes holds the need.
 * d_connections may be NULL in duplicated mode. */
kvsmc_status kvsmc_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p,
                                  float* d_coords, uint64_t coords_capacity,
                                  float* d_normals, uint64_t normals_capacity,
                                  uint32_t* d_connections, uint64_t connections_capacity,
                                  kvsmc_sizes* sizes);

/* Host-side allocator for the output arrays: which = 0 coords (float),
 * 1 normals (float), 2 connections (uint32), 3 colours (uint8, slice plane);
 * count = elements (> 0).
 * Return NULL to fail the call with KVSMC_ERR_OUT_OF_MEMORY. */
typedef void* (*kvsmc_host_alloc_fn)(void* user, int32_t which, uint64_t count);

/* The whole mapper call on host buffers: upload the volume, min/max when not
 * given, count, allocate the outputs through `alloc`, emit, copy back.  This is
 * what kvs::cuda::MarchingCubes::exec calls
 * (replaces MarchingCubes::mapping + extract_surfaces<T>, MarchingCubes.cpp:87-147). */
kvsmc_status kvsmc_marching_cubes_host(kvsmc_context* ctx, const void* host_values, kvsmc_dtype dtype,
                                       uint32_t nx, uint32_t ny, uint32_t nz, const kvsmc_params* p,
                                       kvsmc_host_alloc_fn alloc, void* alloc_user, kvsmc_sizes* sizes);

/* --------------------------------------------------------------- batching */

/* One (volume, isolevel) request of a batch.  Outputs are device pointers with
 * capacities as in kvsmc_extract_device. */
typedef struct kvsmc_request {
    kvsmc_volume* volume;
    kvsmc_params params;
    float* d_coords;       uint64_t coords_capacity;
    float* d_normals;      uint64_t normals_capacity;
    uint32_t* d_connections; uint64_t connections_capacity;
    kvsmc_sizes sizes;     /* out */
    kvsmc_status status;   /* out */
} kvsmc_request;

/* Several isolevels (or modes) of one HOST volume in one call: the volume is
 * uploaded once, all requests run batched, and each request's arrays are
 * allocated through `alloc` (user pointer `alloc_user`, `which` as above plus
 * 3 * request index) and copied back: duplicated-mode triangles in plane
 * ranges while later ranges are written, a shared-vertex request's vertices,
 * connections and normals as soon as the pass that writes each is done, so
 * the copies overlap the remaining passes.  sizes: n entries.  The reference
 * equivalent is n kvs::MarchingCubes constructions on the same volume
 * (Tool/kvsview/Isosurface.cpp:238-249 re-extracts per isolevel). */
kvsmc_status kvsmc_extract_batch_host(kvsmc_context* ctx, const void* host_values, kvsmc_dtype dtype,
                                      uint32_t nx, uint32_t ny, uint32_t nz, const kvsmc_params* params,
                                      int32_t n, kvsmc_host_alloc_fn alloc, void* alloc_user, kvsmc_sizes* sizes);

/* Count every request of a batch in one fused launch (all volumes and
 * isolevels); fills reqs[i].sizes. */
kvsmc_status kvsmc_count_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n);
/* Count + emit a whole batch: fused launches over all requests, so each
 * volume is read once per pass however many isolevels share it. */
kvsmc_status kvsmc_extract_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n);

/* ------------------------------------------------------- replayable plans */

/* A fixed batch extracted again and again (the same volumes, isolevels and
 * output buffers; the volume contents may change in place): the work tables
 * are planned and uploaded once and every launch of one extraction (count,
 * unit scan, plane scan, totals, emit, for every value type present) plus
 * the read-back of the totals is captured into ONE CUDA graph, so a replay
 * costs one cudaGraphLaunch and no host round trip between the passes.
 * No counterpart in the reference (one kvs::MarchingCubes per request).
 *   - every extracted request must be one the streaming kernels take
 *     (duplicated mode, int8/uint8/int16/uint16/float32, width <= 4097),
 *     else KVSMC_ERR_INVALID_ARGUMENT;
 *   - min/max are decided at creation (preset, or the volume's cache, filled
 *     by a min/max pass if needed) and frozen in the plan;
 *   - outputs are bound by address: each request writes at most
 *     min(coords_capacity / 9, normals_capacity / 3) triangles (checked on the
 *     device), and kvsmc_plan_wait reports KVSMC_ERR_CAPACITY with the full
 *     sizes for a request whose result did not fit;
 *   - volumes and outputs must outlive the plan; one replay in flight per plan. */
typedef struct kvsmc_plan kvsmc_plan;
kvsmc_status kvsmc_plan_create(kvsmc_context* ctx, const kvsmc_request* reqs, int32_t n, kvsmc_plan** out);
/* Enqueue one replay on `cuda_stream` (NULL: the context's stream); returns at once. */
kvsmc_status kvsmc_plan_launch(kvsmc_plan* plan, void* cuda_stream);
/* Wait for the last replay and fill reqs[i].sizes / reqs[i].status (n = the
 * plan's request count, same order as at creation); returns the first error. */
kvsmc_status kvsmc_plan_wait(kvsmc_plan* plan, kvsmc_request* reqs, int32_t n);
/* Kernel launches one replay performs. */
uint64_t kvsmc_plan_kernels(const kvsmc_plan* plan);
void kvsmc_plan_destroy(kvsmc_plan* plan);

/* ---------------------------------------------------------------- serving */

/* A request loop over resident volumes with continuous batching.  No
 * counterpart in the reference (one kvs::MarchingCubes call at a time on the
 * caller's thread).  Clients submit (volume, params) requests from any
 * thread; `workers` worker threads, each with its own context and stream,
 * take every pending request (up to `max_batch`) as soon as they are free,
 * count them in one fused pass, admit them against the output budget (48
 * bytes per triangle of device memory held until the client releases the
 * result), carve their outputs from a device arena of the budget's size
 * (allocated once, at creation), and emit them in one fused
 * pass; batches of different workers overlap on the GPU, so requests that
 * arrive while others run start without waiting for them.  A request whose
 * output alone exceeds the budget completes with KVSMC_ERR_BUDGET.  Served
 * requests: duplicated vertices + polygon normals on int8/uint8/int16/uint16/
 * float32 volumes of width <= 4097 (the streaming kernels); others are refused
 * at submit.  Results are identical to kvsmc_extract_device's. */
typedef struct kvsmc_server kvsmc_server;

typedef struct kvsmc_server_config {
    uint64_t output_budget_bytes;  /* device memory for results not yet released (0: 40 GiB) */
    int32_t max_batch;             /* requests per batch (0: 256) */
    int32_t workers;               /* batches in flight at once (0: 3) */
} kvsmc_server_config;

typedef struct kvsmc_completion {
    uint64_t ticket;
    kvsmc_status status;
    int32_t batch_size;            /* requests in the batch it ran in */
    kvsmc_sizes sizes;
    const float* d_coords;         /* device; valid until kvsmc_server_release(ticket) */
    const float* d_normals;
    double submit_s, start_s, done_s;  /* host clock, seconds since the server was created:
                                        * submitted, its batch started counting, results ready */
} kvsmc_completion;

/* The server runs on ctx's device; volumes must stay alive and unchanged
 * while requests on them are pending.  The first request on a volume waits
 * for ctx's stream (so an upload on ctx is complete); a volume uploaded on
 * another context must be complete before it is submitted. */
kvsmc_status kvsmc_server_create(kvsmc_context* ctx, const kvsmc_server_config* cfg, kvsmc_server** out);
/* Queue one request; never blocks on the GPU beyond the first-use wait above
 * (the volume's min/max is filled first if not cached).  *ticket identifies
 * its completion. */
kvsmc_status kvsmc_server_submit(kvsmc_server* s, kvsmc_volume* vol, const kvsmc_params* p, uint64_t* ticket);
/* Up to `max` completions, waiting up to `timeout_ms` (0: do not wait) for
 * the first one; returns how many were written. */
int32_t kvsmc_server_poll(kvsmc_server* s, kvsmc_completion* out, int32_t max, int32_t timeout_ms);
/* Free a completed result's device outputs and return its bytes to the budget. */
kvsmc_status kvsmc_server_release(kvsmc_server* s, uint64_t ticket);
/* Counters: [0] requests submitted, [1] completed, [2] batches, [3] kernel
 * launches, [4] output bytes held now, [5] peak bytes held, [6] times a batch
 * waited for budget. */
kvsmc_status kvsmc_server_stats(kvsmc_server* s, uint64_t* out7);
/* Drain (every submitted request completes), stop the workers, free every
 * result still held. */
void kvsmc_server_destroy(kvsmc_server* s);

/* Copy `bytes` of device memory (a result's d_coords / d_normals) to host
 * memory on the context's stream and wait; for callers without a CUDA
 * runtime of their own. */
kvsmc_status kvsmc_copy_to_host(kvsmc_context* ctx, void* host, const void* device, uint64_t bytes);

/* ------------------------------------------------- no-allocation variant */

/* For callers that may not allocate device memory: a plugin whose host
 * application owns the whole device-memory budget, or an interactive frame
 * loop in which cudaMalloc/cudaFree (which can synchronize the device) would
 * stall.  No counterpart in the reference; this is the duplicated-vertex,
 * polygon-normal extraction (p->mode must be KVSMC_DUP_POLYGON_NORMAL) run
 * by the streaming kernels, with no context and no allocation of any kind:
 *   - the caller passes the volume (dense device array, x fastest; its rows,
 *     nx * sizeof(value), must be 16-byte multiples and d_values 16-byte
 *     aligned), the output arrays with their capacities (floats), and a
 *     CUDA stream (NULL = the legacy default stream);
 *   - dtype is int8, uint8, int16, uint16 or float32; 2 <= nx <= 4097;
 *     ny, nz >= 2; the isolevel is finite;
 *   - the intermediates live in a 4 MiB static device array that every GPU
 *     loading this library holds until exit; a volume whose intermediates do
 *     not fit (beyond about 512^3) is refused with KVSMC_ERR_TOO_LARGE;
 *   - the first call on each device looks up that array's device address
 *     (cudaGetSymbolAddress) with the device current: make that first call
 *     before starting any stream capture;  the address is kept for the life
 *     of the process, so after a cudaDeviceReset (or anything else that
 *     destroys and recreates the device's primary context) it is stale:
 *     do not call this entry point again on that device;
 *   - each call waits for its stream (cudaStreamSynchronize) to read back
 *     the triangle count: twice, three times when the min/max is not
 *     preset;
 *   - all calls share the array: calls that overlap on the GPU race on it
 *     and must be serialized by the caller.
 * Returns KVSMC_ERR_CAPACITY (with *sizes filled) when the outputs are too
 * small.  Results are identical to kvsmc_extract_device's. */
kvsmc_status kvsmc_extract_noalloc(const void* d_values, kvsmc_dtype dtype, uint32_t nx, uint32_t ny,
                                   uint32_t nz, const kvsmc_params* p, float* d_coords,
                                   uint64_t coords_capacity, float* d_normals, uint64_t normals_capacity,
                                   void* cuda_stream, kvsmc_sizes* sizes);

/* ------------------------------------------------------ unstructured volumes */

/* kvs::MarchingTetrahedra / MarchingHexahedra / MarchingPyramid /
 * MarchingPrism (Source/Core/Visualization/Mapper/) on an unstructured volume
 * in host memory: nnodes values and float coords[3 nnodes], ncells cells of
 * 4 / 8 / 5 / 6 connections each.  Duplicated vertices, one normal per
 * triangle (the reference builds nothing in shared-vertex mode), cells in
 * order, table order inside a cell, same bits.  The isolevel and the clamp
 * range (has_minmax: min/max given, else the device scan over values[0] and
 * the cells' nodes, UnstructuredVolumeObject.cpp:82-143, or over the nodes
 * when there are no cells) decide as in the reference; sizes->min_value /
 * max_value return the range used; the Math::Equal(min, max) early exit
 * gives sizes->extracted = 0.  Outputs come from `alloc` (which: 0 coords,
 * 1 normals).  A connection index >= nnodes is KVSMC_ERR_INVALID_ARGUMENT
 * (checked on the device, nothing read out of range); more than 2^31 - 1
 * nodes or 2^32 - 1 cells is KVSMC_ERR_TOO_LARGE (the reference's int node
 * ids and UInt32 cell counter).  An isolevel of NaN classifies every node
 * below it: only the min/max scan and an empty count run. */
kvsmc_status kvsmc_marching_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                       kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                       const uint32_t* connections, uint64_t ncells, double isolevel,
                                       int32_t has_minmax, double min_value, double max_value,
                                       kvsmc_host_alloc_fn alloc, void* user, kvsmc_sizes* sizes);
/* An isolevel sweep of one unstructured volume on DEVICE arrays: niso (at
 * most 64) extractions, each the same as kvsmc_marching_cells_device at its
 * isolevel, sharing one count pass (connections and node values read once for
 * all isolevels), one scan and one emit launch.  out_coords[k] /
 * out_normals[k] with capacities coords_capacity[k] / normals_capacity[k]
 * (floats) receive isolevel k's triangles; sizes[k] its counts (all get the
 * min/max used).  If any isolevel's triangles do not fit, nothing is written
 * and the call returns KVSMC_ERR_CAPACITY with every sizes[k] filled. */
kvsmc_status kvsmc_marching_cells_sweep_device(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* d_values,
                                               kvsmc_dtype dtype, uint64_t nnodes, const float* d_coords,
                                               const uint32_t* d_connections, uint64_t ncells,
                                               const double* isolevels, int32_t niso, int32_t has_minmax,
                                               double min_value, double max_value, float* const* d_out_coords,
                                               const uint64_t* coords_capacity, float* const* d_out_normals,
                                               const uint64_t* normals_capacity, kvsmc_sizes* sizes);
/* The volume's bounding box as UnstructuredVolumeObject::updateMinMaxCoords
 * (UnstructuredVolumeObject.cpp:396-466) folds it, on the GPU: per axis
 * Math::Min / Math::Max from the first connected node over every connection
 * (over the nodes when ncells is 0); a NaN coordinate is taken and the next
 * replaces it, ties keep the later value.  Host arrays in, six floats out. */
kvsmc_status kvsmc_cells_bounds(kvsmc_context* ctx, kvsmc_cell_type cell_type, const float* coords, uint64_t nnodes,
                                const uint32_t* connections, uint64_t ncells, float* min_coord, float* max_coord);
/* The same on DEVICE arrays (values, coords, connections) into caller-provided
 * device outputs (capacities in floats: 9 T coords, 3 T normals); on
 * KVSMC_ERR_CAPACITY nothing is written and *sizes holds the need. */
kvsmc_status kvsmc_marching_cells_device(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* d_values,
                                         kvsmc_dtype dtype, uint64_t nnodes, const float* d_coords,
                                         const uint32_t* d_connections, uint64_t ncells, double isolevel,
                                         int32_t has_minmax, double min_value, double max_value,
                                         float* d_out_coords, uint64_t coords_capacity, float* d_out_normals,
                                         uint64_t normals_capacity, kvsmc_sizes* sizes);

/* -------------------------------------------------------------- slice plane */

/* kvs::SlicePlane on a structured volume (Source/Core/Visualization/Mapper/
 * SlicePlane.cpp): marching cubes on the plane a x + b y + c z + d (cases
 * from its sign at the corners), one RGB colour per vertex from the
 * transfer function at the interpolated volume value, one normal per
 * triangle; duplicated vertices, coords float[9T], colours uint8[9T],
 * normals float[3T], in the reference's cell and table order, same bits.
 * The host decides what MapperBase decides (the colour map range, the
 * coordinate transform) and passes it here. */
typedef struct kvsmc_slice_params {
    float coefficients[4];      /* a, b, c, d (SlicePlane::setPlane; point p, normal n -> (n, -p.n)) */
    float min_coord[3];         /* volume->minObjectCoord() */
    float scale[3];             /* (max_coord - min_coord) / ncells */
    float tf_min, tf_max;       /* the colour map's range (MapperBase::setRange) */
    int32_t tf_resolution;      /* colour table entries */
    const uint8_t* tf_table;    /* host, tf_resolution x RGB */
} kvsmc_slice_params;

/* Triangles of the slice (count pass only). */
kvsmc_status kvsmc_slice_count(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               uint64_t* ntriangles);
/* Count + emit into DEVICE buffers (capacities in elements); on
 * KVSMC_ERR_CAPACITY nothing is written and *ntriangles holds the need. */
kvsmc_status kvsmc_slice_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                                        float* d_coords, uint64_t coords_capacity, uint8_t* d_colors,
                                        uint64_t colors_capacity, float* d_normals, uint64_t normals_capacity,
                                        uint64_t* ntriangles);
/* Count + emit into host arrays from `alloc` (which: 0 coords, 1 normals,
 * 3 colours (uint8)); nothing is allocated for an empty slice. */
kvsmc_status kvsmc_slice_plane(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles);

/* ------------------------------------------------------------ volume ingest */

/* A KVSML structured volume (.kvsml) as the reference reads it
 * (StructuredVolumeObject::read, StructuredVolumeObject.cpp:171-229). */
typedef struct kvsmc_kvsml_info {
    int32_t dtype;                  /* kvsmc_dtype of <DataArray type> */
    uint32_t nx, ny, nz;            /* resolution */
    uint32_t veclen;
    int32_t grid_uniform;           /* 1: grid_type="uniform" */
    int32_t data_format;            /* 0: inline ASCII, 1: external ASCII, 2: external binary */
    int32_t byte_swap;              /* external binary of the other endianness */
    int32_t has_min_value, has_max_value;
    double min_value, max_value;    /* the file's <Value min_value max_value> */
    double volume_min, volume_max;  /* the loaded volume's min/max (set by the load) */
    int32_t has_object_coord, has_external_coord;
    float min_object_coord[3], max_object_coord[3];     /* the file's, or [0, res - 1] */
    float min_external_coord[3], max_external_coord[3]; /* the file's, or the object coords */
} kvsmc_kvsml_info;

/* The header of a .kvsml file (no data read, no GPU needed). */
kvsmc_status kvsmc_kvsml_read_info(const char* path, kvsmc_kvsml_info* info);
/* Load a .kvsml uniform scalar volume straight into a resident device volume:
 * external binary values stream from the file through pinned memory into the
 * padded device rows (byte-swapped on the GPU when the file's endianness
 * differs); ASCII values are parsed as the reference does (atof, cast).  The
 * volume's min/max cache is set as StructuredVolumeObject::read sets it, the
 * brick table is built.  Non-uniform grids and veclen != 1 are
 * KVSMC_ERR_INVALID_ARGUMENT; fewer values than nodes too (the reference
 * leaves them uninitialised). */
kvsmc_status kvsmc_volume_load_kvsml(kvsmc_context* ctx, const char* path, kvsmc_volume** vol,
                                     kvsmc_kvsml_info* info);
/* The same for an AVS field file (.fld, kvs::AVSField, FileFormat/AVSField/
 * AVSField.cpp, imported as StructuredVolumeImporter.cpp:155-189 does):
 * uniform fields of byte/short/integer/float/double, the values after the
 * header's "\f\f" streamed into the device rows; min/max by the device scan;
 * info->data_format is 2 (binary). */
kvsmc_status kvsmc_avs_read_info(const char* path, kvsmc_kvsml_info* info);
kvsmc_status kvsmc_volume_load_avs(kvsmc_context* ctx, const char* path, kvsmc_volume** vol,
                                   kvsmc_kvsml_info* info);

/* kvs::SlicePlane on an unstructured volume (SlicePlane.cpp:291-800): per
 * cell, the case from the plane's sign at the node coordinates, the cell
 * type's triangle table in table order, vertices (1 - r) v0 + r v1 with
 * r = |p0 / (p1 - p0)| in float, per-vertex colours from the transfer
 * function at the value interpolated in the value type's arithmetic, one
 * normal -((v2 - v0) x (v1 - v0)) per triangle; coords float[9T], colours
 * uint8[9T], normals float[3T] through `alloc` (which: 0 coords, 1 normals,
 * 3 colours).  Arrays as kvsmc_marching_cells_host; p->min_coord and
 * p->scale are not used (the reference slices the node coordinates as they
 * are).  A connection index >= nnodes is KVSMC_ERR_INVALID_ARGUMENT. */
kvsmc_status kvsmc_slice_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                    kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                    const uint32_t* connections, uint64_t ncells, const kvsmc_slice_params* p,
                                    kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles);

/* ---------------------------------------------------------- polygon export */

/* Binary STL records of a triangle mesh in device memory: what
 * kvs::PolygonExporter<kvs::Stl>::exec (PolygonExporter.cpp:78-176) and
 * kvs::Stl::write_binary (Stl.cpp:490-540) write after the 84-byte header --
 * per triangle its normal (3 floats; with vertex normals the mean
 * (n0 + n1 + n2) / 3 of its vertices' normals), its 3 vertices (9 floats)
 * and 2 zero bytes: 50 bytes, little-endian.  mode is the kvsmc_mode the mesh
 * was extracted with:
 *   KVSMC_DUP_POLYGON_NORMAL:    d_coords 9T floats, d_normals 3T (d_connections unused);
 *   KVSMC_SHARED_POLYGON_NORMAL: d_coords 3V, d_connections 3T, d_normals 3T;
 *   KVSMC_SHARED_VERTEX_NORMAL:  d_coords 3V, d_connections 3T, d_normals 3V.
 * d_out: 50 * ntriangles bytes of 16-byte aligned device memory.  Runs on the
 * context's stream and waits for it.  A connection index >= nvertices is
 * KVSMC_ERR_INVALID_ARGUMENT (checked on the device; nothing is read out of
 * range). */
kvsmc_status kvsmc_stl_records(kvsmc_context* ctx, int32_t mode, const float* d_coords, const float* d_normals,
                               const uint32_t* d_connections, uint64_t nvertices, uint64_t ntriangles,
                               void* d_out);
/* The binary STL file of a device mesh, written to `path`: the 80-byte header
 * "Generated by KVS" (zero-padded), the uint32 triangle count, the records --
 * serialised on the GPU in chunks of 2^20 triangles, each copied to pinned
 * memory and written while the next is serialised.  The reference's
 * kvs::Stl defaults to ASCII; this is its Binary file type.  More than
 * 2^32 - 1 triangles is KVSMC_ERR_TOO_LARGE (the format's count would wrap). */
kvsmc_status kvsmc_write_stl(kvsmc_context* ctx, const char* path, int32_t mode, const float* d_coords,
                             const float* d_normals, const uint32_t* d_connections, uint64_t nvertices,
                             uint64_t ntriangles);
/* Same for a mesh in HOST memory (a PolygonObject's arrays; sizes in
 * elements): uploaded, then serialised on the GPU as above.  Triangles:
 * ncoords / 9 (duplicated) or nconnections / 3. */
kvsmc_status kvsmc_write_stl_host(kvsmc_context* ctx, const char* path, int32_t mode, const float* coords,
                                  uint64_t ncoords, const float* normals, uint64_t nnormals,
                                  const uint32_t* connections, uint64_t nconnections);
/* The ASCII STL file of a device mesh, kvs::Stl's default file type
 * (Stl.cpp:86): what Stl::write_ascii (Stl.cpp:447-480) prints for the
 * triangles PolygonExporter<kvs::Stl> hands it -- "solid Generated by KVS",
 * per triangle "facet normal %f %f %f", "outer loop", three "vertex %f %f %f",
 * "endloop", "endfacet", then "endsolid", byte for byte.  The text is
 * formatted on the GPU (exact "%f": the float's binary value rounded to six
 * decimals, ties to even) in chunks of 2^20 triangles, each copied to pinned
 * memory and written while the next is formatted.  Same meshes and modes as
 * kvsmc_write_stl. */
kvsmc_status kvsmc_write_stl_ascii(kvsmc_context* ctx, const char* path, int32_t mode, const float* d_coords,
                                   const float* d_normals, const uint32_t* d_connections, uint64_t nvertices,
                                   uint64_t ntriangles);
/* The KVSML polygon file of a device mesh: what PolygonExporter<
 * kvs::KVSMLPolygonObject> (PolygonExporter.cpp:22-68) and
 * KVSMLPolygonObject::write (KVSMLPolygonObject.cpp:349-492) write for a
 * marching-cubes result, byte for byte.  writing_type is the reference's
 * WritingDataType: 0 Ascii (arrays inside the .kvsml), 1 ExternalAscii,
 * 2 ExternalBinary (arrays in <base>_coord.dat, _normal.dat, _connect.dat
 * beside `path`, binary arrays streamed from the device through pinned
 * buffers).  mode sets normal_type (vertex for KVSMC_SHARED_VERTEX_NORMAL,
 * else polygon); sizes are elements (floats, uint32); color (3 bytes) and
 * opacity (1 byte), when not null, are the object's single colour and
 * opacity, written as <DataValue>s. */
kvsmc_status kvsmc_write_kvsml_polygon(kvsmc_context* ctx, const char* path, int32_t writing_type, int32_t mode,
                                       const float* d_coords, uint64_t ncoords, const float* d_normals,
                                       uint64_t nnormals, const uint32_t* d_connections, uint64_t nconnections,
                                       const uint8_t* color, const uint8_t* opacity);
/* Same for a mesh in HOST memory (uploaded first), as kvsmc_write_stl_host. */
kvsmc_status kvsmc_write_stl_ascii_host(kvsmc_context* ctx, const char* path, int32_t mode, const float* coords,
                                        uint64_t ncoords, const float* normals, uint64_t nnormals,
                                        const uint32_t* connections, uint64_t nconnections);


/* Binary PLY (little endian) of a triangle mesh without connections: what
 * kvs::PolygonExporter<kvs::Ply>::exec (PolygonExporter.cpp:178-361) and
 * kvs::Ply::write with the Binary file type (Ply.cpp:389-488, header of
 * PlyFile.cpp:399-460) write -- the header ("element vertex N", the x/y/z,
 * red/green/blue and nx/ny/nz properties present, "element face 0") and one
 * packed record per vertex.  color_mode: 0 no colour, 1 the one RGB colour at
 * colors[0..2] for every vertex (a PolygonObject with a single colour), 2 one
 * RGB per vertex (VertexColor).  normal_mode: 0 none, 1 zeros (PolygonNormal:
 * the exporter averages polygon normals over connections, of which there are
 * none), 2 one normal per vertex (VertexNormal).  Meshes with connections are
 * not taken: the reference's writer stores face indices through a null
 * pointer (Ply.cpp:470-480).  More than 2^31 - 1 vertices is
 * KVSMC_ERR_TOO_LARGE (the header's int count). */
uint32_t kvsmc_ply_record_bytes(int32_t color_mode, int32_t normal_mode);
/* The header text; returns its length (written to buf when size > length). */
int64_t kvsmc_ply_header(uint64_t nvertices, int32_t color_mode, int32_t normal_mode, char* buf, uint64_t size);
/* The records of a device mesh into a 16-byte aligned device buffer of
 * nvertices * kvsmc_ply_record_bytes() bytes. */
kvsmc_status kvsmc_ply_records(kvsmc_context* ctx, const float* d_coords, uint64_t nvertices, const uint8_t* d_colors,
                               int32_t color_mode, const float* d_normals, int32_t normal_mode, uint8_t* d_out);
/* The file of a device mesh (records in chunks through pinned memory), or of a
 * host mesh (uploaded first). */
kvsmc_status kvsmc_write_ply(kvsmc_context* ctx, const char* path, const float* d_coords, uint64_t nvertices,
                             const uint8_t* d_colors, int32_t color_mode, const float* d_normals, int32_t normal_mode);
kvsmc_status kvsmc_write_ply_host(kvsmc_context* ctx, const char* path, const float* coords, uint64_t nvertices,
                                  const uint8_t* colors, int32_t color_mode, const float* normals, int32_t normal_mode);

/* ------------------------------------------------------------- autotuning */

/* Launch shape of the streaming kernels for one (value type, volume size
 * class).  Every field 0 = the built-in rule for that field.  Results are
 * identical under every shape; only the speed differs.  The reference has one
 * CPU loop and nothing to tune. */
typedef struct kvsmc_tune_choice {
    int32_t rows;          /* cell rows per warp task: 1 (256-cell row segments) or 2 (two 128-cell rows) */
    int32_t tasks_per_sm;  /* warp tasks per SM a launch is cut into (sets cell planes per task, 4..64) */
    int32_t ctas_per_sm;   /* resident CTAs per SM of the persistent launches (capped by what fits) */
    int32_t scan_threads;  /* unit-scan tile: 64, 128 or 256 units per CTA pass */
} kvsmc_tune_choice;

/* One row of a tuning table. */
typedef struct kvsmc_tune_entry {
    int32_t dtype;            /* kvsmc_dtype */
    int32_t size_class;       /* kvsmc_size_class() of the volumes it applies to */
    kvsmc_tune_choice choice;
    double tuned_ms;          /* measured count + emit time of the choice (0: not measured) */
    double default_ms;        /* measured time of the built-in rule on the same work */
} kvsmc_tune_entry;

#define KVSMC_SIZE_CLASSES 5

/* Size class of a volume by its cell count C = (nx-1)(ny-1)(nz-1):
 * 0: C < 2^18, 1: < 2^21, 2: < 2^24, 3: < 2^27, 4: larger. */
int32_t kvsmc_size_class(uint32_t nx, uint32_t ny, uint32_t nz);

/* The launch shape a streaming batch uses for a volume, given a tuning table
 * (NULL / 0 rows: built-in rules): the entry for (dtype, size class) with
 * its zero fields filled by the built-in rules.  Pure host function.
 * KVSMC_ERR_INVALID_ARGUMENT when a table entry holds an invalid value. */
kvsmc_status kvsmc_tune_resolve(const kvsmc_tune_entry* table, int32_t n, kvsmc_dtype dtype, uint32_t nx,
                                uint32_t ny, uint32_t nz, kvsmc_tune_choice* out);

/* Install a tuning table on a context (copied; n = 0 clears it).  Every
 * later streaming batch, plan and server round of the context follows it. */
kvsmc_status kvsmc_tuning_set(kvsmc_context* ctx, const kvsmc_tune_entry* table, int32_t n);
/* Copy out the installed table; returns its length (fills at most cap rows). */
int32_t kvsmc_tuning_get(const kvsmc_context* ctx, kvsmc_tune_entry* out, int32_t cap);
/* Use one launch shape for every volume (NULL: back to the table). */
kvsmc_status kvsmc_tuning_force(kvsmc_context* ctx, const kvsmc_tune_choice* choice);

typedef struct kvsmc_autotune_config {
    const int32_t* dtypes;    /* value types to tune (NULL: uint8, uint16, float32, int8, int16) */
    int32_t ndtypes;
    int32_t max_class;        /* tune size classes 0 .. max_class (<= 4) */
    int32_t isovalues;        /* isovalues per batch on the tuning volumes (1..16) */
    int32_t reps;             /* timed runs per candidate; the median counts */
    uint64_t seed;            /* seed of the synthetic tuning volumes */
} kvsmc_autotune_config;

/* The autotuner: for every (dtype, size class) asked for, build a seeded
 * synthetic volume of that class on the device, time count + emit of a
 * batch of isovalues under candidate launch shapes (coordinate descent over
 * rows x tasks per SM, then CTAs per SM, then the scan tile), and keep a
 * shape only where it beats the built-in rules by more than 3 %.  Installs
 * the table on the context and copies it to out (at most cap rows, *nout
 * rows written).  Takes seconds; allocates and frees its own buffers. */
kvsmc_status kvsmc_autotune(kvsmc_context* ctx, const kvsmc_autotune_config* cfg, kvsmc_tune_entry* out,
                            int32_t cap, int32_t* nout);

/* ------------------------------------------------------------ diagnostics */

/* Per-kernel timing: with profiling on, every kernel family launched by this
 * context is bracketed by CUDA events on its own stream.  enable() clears the
 * totals.  read() waits for the recorded events and returns the number of
 * kernel families; for the first `max` it fills the name, the launch count
 * and the summed device milliseconds.  The reference times whole calls on
 * the host (kvs::Timer, Utility/Timer.h); this is the device-side analogue. */
kvsmc_status kvsmc_profile_enable(kvsmc_context* ctx, int32_t on);
int32_t kvsmc_profile_read(kvsmc_context* ctx, int32_t max, const char** names, uint64_t* launches, double* ms);

/* Device self-check of the FP32 interpolation path: n random straddling edges
 * (several value distributions) interpolated both by the FP32 path and by the
 * reference's FP64 sequence (interpolate_vertex, MarchingCubes.cpp:327-356).
 * Reports how many were tested, how many float results differ (must be 0)
 * and how many fell back to FP64.  No counterpart in the reference. */
kvsmc_status kvsmc_selftest_interpolation(kvsmc_context* ctx, uint64_t n, uint64_t seed, uint64_t* tested,
                                          uint64_t* mismatches, uint64_t* fallbacks);
/* The same for the unstructured mappers' vertex on random float endpoints
 * (interpolate_vertex, MarchingTetrahedra.cpp:325-346): the FP32 certificate
 * of the cells' emit pass against the FP64 sequence. */
kvsmc_status kvsmc_selftest_cells(kvsmc_context* ctx, uint64_t n, uint64_t seed, uint64_t* tested,
                                  uint64_t* mismatches, uint64_t* fallbacks);

/* Position-keyed checksums of a device array of 32-bit words, for checking
 * outputs too large to copy back against a CPU run of the same extraction:
 * sums[c] = sum over the words i of chunk c (words [c*chunk_words,
 * (c+1)*chunk_words) of the array) of mix(i, w_i) mod 2^64, with
 *   x = (i * 0x9E3779B97F4A7C15) ^ (w * 0xC2B2AE3D27D4EB4F);
 *   x ^= x >> 31;  x *= 0xBF58476D1CE4E5B9;  x ^= x >> 29;  mix = x
 * (64-bit unsigned arithmetic).  nchunks (at most 65535) must cover the
 * array; sums is host memory.  No counterpart in the reference. */
kvsmc_status kvsmc_checksum_words(kvsmc_context* ctx, const void* d_words, uint64_t nwords, uint64_t chunk_words,
                                  uint64_t* sums, uint64_t nchunks);

/* Test hook: cap the polls of the streaming count / emit kernels' bounded
 * waits for a staged node plane (negative = the built-in limit, 2^22).  With
 * a cap of 0 every such wait gives up at once, so an extraction returns
 * KVSMC_ERR_TIMEOUT the way a stalled copy would make it; the kernels still
 * drain their copies in flight under their own limit, and the context stays
 * usable.  No counterpart in the reference (whose loop has no device waits);
 * its error convention is a message and a null result
 * (MarchingCubes.cpp:50-67). */
kvsmc_status kvsmc_set_wait_limit(kvsmc_context* ctx, int64_t count_polls, int64_t emit_polls);

#ifdef __cplusplus
}
#endif

#endif /* KVSMC_H */
