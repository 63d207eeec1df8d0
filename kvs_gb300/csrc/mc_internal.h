// mc_internal.h -- host-side declarations shared by the library's .cu files.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mc_device.cuh"
#include "mc_interp.cuh"

namespace kvsmc {

struct Profiler;

// Polls of the streaming kernels' waits for a staged node plane before they
// give up (KVSMC_ERR_TIMEOUT); a plane normally lands within a few polls.
constexpr uint32_t kStreamWaitPolls = 1u << 22;

// Launch bookkeeping passed to every launcher.
struct Launch {
    cudaStream_t stream;
    int num_sms;
    uint64_t* counter;   // incremented once per kernel launch
    Profiler* prof;      // per-kernel CUDA-event timing when enabled (may be null)
    // plane-wait poll limit of the streaming count [0] and emit [1] kernels
    uint32_t wait_polls[2] = {kStreamWaitPolls, kStreamWaitPolls};
};

// CUDA events on the launching stream around one kernel family's launch.
void prof_begin(const Launch& L, const char* name);
void prof_end(const Launch& L);

// Size in bytes of one value of a dtype code (0 if unknown).
size_t dtype_size(int dtype);

// ---- min/max scan (GetMinMaxValues, StructuredVolumeObject.cpp:66-85)
// scratch: minmax_scratch_bytes() device bytes; out: 2 doubles (device).
size_t minmax_scratch_bytes(int num_sms);
cudaError_t launch_minmax(const VolumeView& v, void* scratch, double* d_out, const Launch& L);

// ---- exclusive scan of uint32 counts -> uint64 offsets, total in *d_total.
size_t scan_scratch_bytes(uint64_t n);
cudaError_t launch_scan(const uint32_t* counts, uint64_t* offsets, uint64_t n, void* scratch,
                        uint64_t* d_total, const Launch& L);

// ---- gather-form kernels (mc_gather.cu): every mode and dtype
cudaError_t launch_cell_count(const Job& j, const Launch& L);
cudaError_t launch_emit_dup(const Job& j, const Launch& L);
cudaError_t launch_node_count(const Job& j, const Launch& L);
cudaError_t launch_node_emit(const Job& j, const Launch& L);
cudaError_t launch_connect(const Job& j, const Launch& L);
// vertex normals (mode 2) from the connections and per-triangle normals
// (k_connect writes them to j.tri_normals): scratch of
// vertex_normals_scratch_bytes, carved into j by vertex_normals_carve
size_t vertex_normals_scratch_bytes(uint64_t ntri, uint64_t nvert);
void vertex_normals_carve(Job& j, uint64_t ntri, uint64_t nvert, void* scratch);
cudaError_t launch_vertex_normals(const Job& j, uint64_t ntri, uint64_t nvert, const Launch& L);

// ---- streaming kernels (mc_stream.cu): duplicated mode, batched
constexpr int kStreamThreads = 256;   // 8 independent warps per CTA
constexpr int kStreamMaxIso = 16;     // isolevels of one volume per group
constexpr int kStreamBuckets = 128;   // threshold lookup buckets
constexpr int kStreamSegCells = 256;  // cells per warp step (one 256-cell row segment, or two of 128)
constexpr int kStreamMaxCells = 4096; // cells per row (width <= 4097 nodes)

// One isolevel request inside a streaming launch.
struct StreamIso {
    FastIso f;
    Interp ip;
    uint64_t plane_index;  // its first (isolevel, z) plane in the plane arrays
    float* coords;         // outputs (null: not written)
    float* normals;
    uint64_t cap_tris;     // triangles the outputs hold: later ones are not written
};

// One volume with up to kStreamMaxIso isolevels, sorted by threshold.
// Warp tasks (z-chunk, row y, segment) are numbered segment fastest, then y,
// then z-chunk; units (z, y, segment) likewise, each with niso counters.
struct StreamGroup {
    VolumeView vol;
    int32_t iso_begin, niso;
    uint32_t rows;           // cell rows per warp task: 1 (256-cell segments) or 2 (128-cell segments)
    uint32_t wpr;            // segments per cell row
    uint32_t zchunk;         // cell planes per warp task
    uint64_t task_begin;     // first warp task of this group in its launch
    uint64_t unit_base;      // first element of its (unit, isolevel) counters
    uint32_t plane_begin;    // first unit-scan block of this group (one per z)
    uint32_t seg_elems;      // staged elements per node row (16-byte multiple)
    uint32_t seg_copy_bytes; // bytes copied per node row (last segment: fewer)
    uint32_t warp_smem_bytes;
    uint32_t warp_smem_offset;
    float bs, bo;            // bucket(v) = floor(kStreamBuckets * sat(v * bs + bo)), in [0, kStreamBuckets]
    const float2* bricks;    // the volume's brick min/max table, or null
    int32_t skip_emit;       // 1: no isolevel of the group is written by this emit launch
    uint32_t brick_wpr;      // bricks per row pair (128-cell brick segments per row)
    // shared-vertex vertex counts from the count pass (one-row tasks only):
    // per isolevel k, node unit u = (plane, node row, 256-node segment) at
    // node_base + k * node_units + u; node_units == 0: not counted
    uint64_t node_base;
    uint64_t node_units;
};

// Brick min/max table of a volume: one float2 per (8 cell planes, 2 cell
// rows, 128 cells) brick, the min and max of its node box ((-inf, +inf) when
// it holds a NaN), bricks numbered segment fastest, then row pair, then plane
// group.  A two-row warp task covers one brick per plane group, a one-row
// task (256 cells) two neighbouring bricks; the table serves both.
constexpr int kBrickPlanes = 8;
constexpr uint32_t kBrickCells = 128;
uint64_t brick_count(const VolumeView& v);
cudaError_t launch_bricks(const VolumeView& v, float2* out, const Launch& L);

size_t stream_shared_bytes(int dtype, bool emit, int rows);
size_t stream_warp_smem_bytes(int dtype, bool emit, int rows);
size_t stream_warp_smem_offset();
size_t stream_row_elems(int dtype, int rows);
// d_next_task: a zeroed u64 per launch (the persistent warps' task counter).
// d_unit_counts: written by the count launch; read by the emit launch to skip
// steps without triangles.  ctas_per_sm: resident CTAs per SM of the
// persistent grid (0: as many as fit; never more than fit).  The launch runs
// the warp tasks [task0, ntasks) of its groups (task0 > 0: a later part of a
// launch split by z-chunks).
cudaError_t launch_stream(bool emit, int dtype, int rows, const StreamGroup* d_groups, int ngroups, uint64_t ntasks,
                          const StreamIso* d_isos, uint16_t* d_unit_counts, const uint32_t* d_unit_offsets,
                          const uint64_t* d_plane_base, int* d_status, unsigned long long* d_next_task,
                          const Launch& L, int ctas_per_sm = 0, uint64_t task0 = 0,
                          uint32_t* d_node_counts = nullptr);
// scan_threads: units per CTA pass (64, 128 or 256; 0 = 256).
cudaError_t launch_unit_scan(const StreamGroup* d_groups, int ngroups, uint32_t nplanes, const StreamIso* d_isos,
                             const uint16_t* d_unit_counts, uint32_t* d_unit_offsets, uint32_t* d_plane_totals,
                             const Launch& L, int scan_threads = 0);
cudaError_t launch_iso_totals(const StreamIso* d_isos, int n, const uint64_t* d_plane_base, const uint64_t* d_total,
                              uint64_t* d_totals, const Launch& L);

// ---- shared-vertex node passes on the streaming kernels (mc_snode.cu):
// node units (plane, row, 256-node segment) numbered in node order; the count
// pass writes one vertex count per unit, the emit pass (unit_offsets: the
// exclusive scan of the counts) the rank words j.rank and the vertices
// j.coords.  One isolevel; 8/16-bit and float32 volumes.
size_t snode_shared_bytes(int dtype);

// One request of the multi-isolevel node emit: a batch's shared-vertex
// requests on one volume (at most kStreamMaxIso, sorted by threshold) written
// by one pass over the volume.
struct NodeIso {
    FastIso f;
    Interp ip;
    float* coords;              // the request's vertices
    uint4* rank;                // its rank words (nz * ny * words_per_row)
    const uint64_t* offsets;    // per node unit: its first vertex id
    const uint32_t* counts;     // per node unit: its vertices
};
size_t snode_multi_shared_bytes(int dtype);

// One request of the multi-isolevel connection pass (the requests of one
// streaming count group, in its isolevel order).
struct ConnIso {
    const uint4* rank;       // its rank words
    const float* coords;     // its vertices
    uint32_t* connections;   // its triangles' vertex ids
    float* tri_out;          // polygon normals, or the per-triangle normals its vertex normals sum
    uint64_t nvert, ntri;
    uint32_t enabled;        // 0: nothing of it is written
    uint32_t pad;
};
size_t sconnect_multi_shared_bytes(int dtype);
// The connection pass of every enabled request of streaming count group
// d_group (one-row tasks) at once: the group's tasks, its counters and scans.
cudaError_t launch_sconnect_multi(const StreamGroup* d_group, const StreamIso* d_isos, const ConnIso* d_conn, int dtype,
                                  const uint16_t* unit_counts, const uint32_t* unit_offsets, const uint64_t* plane_base,
                                  uint64_t ntasks, int* status, unsigned long long* next_task, const Launch& L);
// vol: the volume; d_isos: niso requests; bs, bo: the bucket map of their
// thresholds; wprn, zchunk, ntasks: the node-unit task shape of the single
// request passes; words_per_row: rank words per node row.
cudaError_t launch_snode_multi(const VolumeView& vol, const NodeIso* d_isos, int niso, float bs, float bo,
                               uint32_t wprn, uint32_t zchunk, uint64_t ntasks, uint32_t words_per_row, int* status,
                               unsigned long long* next_task, const Launch& L);
cudaError_t launch_snode(bool emit, const Job& j, const FastIso& f, uint32_t wprn, uint32_t zchunk, uint64_t ntasks,
                         uint32_t* unit_counts, const uint64_t* unit_offsets, int* status,
                         unsigned long long* next_task, const Launch& L);

// connect_isopoints on the streaming cell tasks of a one-group, one-isolevel,
// one-row-per-task streaming count (its unit counts and offsets, plane
// bases): connections, and polygon normals (mode 1) or per-triangle normals
// for the vertex normals (mode 2); the node emit pass must have written
// j.rank and j.coords.
size_t sconnect_shared_bytes(int dtype);
cudaError_t launch_sconnect(const Job& j, const StreamGroup* d_groups, const StreamIso* d_isos,
                            const uint16_t* unit_counts, const uint32_t* unit_offsets, const uint64_t* plane_base,
                            uint32_t iso_k, uint64_t ntasks, uint64_t nvert, uint64_t ntri, int* status,
                            unsigned long long* next_task, const Launch& L);

// ---- SlicePlane on structured volumes (slice.cu): one warp per cell row
// (y, z), rows numbered y fastest
struct SliceJob {
    VolumeView vol;
    float coef[4];            // a x + b y + c z + d
    float min_coord[3], scale[3];
    float tf_min, tf_max;     // colour map range
    int32_t tf_res;
    const uint8_t* table;     // device colour table, tf_res x RGB
    uint64_t nrows;           // (ny - 1) (nz - 1)
    uint32_t* row_counts;     // count pass: triangles per row
    uint64_t* row_offsets;    // emit pass: exclusive scan of row_counts
    float* coords;            // 9 T
    uint8_t* colors;          // 9 T (RGB per vertex)
    float* normals;           // 3 T
    uint64_t cap_tris;        // triangles the outputs hold
};
cudaError_t launch_slice_count(const SliceJob& j, const Launch& L);
cudaError_t launch_slice_emit(const SliceJob& j, const Launch& L);

// ---- marching cells on unstructured volumes (cells.cu)
// One isolevel of a cells extraction: its exact thresholds, its vertex
// certificate constants and its outputs.
struct CellIso {
    double iso;
    Classifier cls;
    FastIso f;
    float* out_coords;        // 9 T
    float* out_normals;       // 3 T
    uint64_t cap_tris;
    uint64_t base;            // sweep: its first slot in the scanned group offsets
};
constexpr int kCellSweepMax = 64;   // isolevels of one sweep
struct CellJob {
    int32_t cell_type;        // kvsmc_cell_type
    int32_t dtype;
    const void* values;
    uint64_t nnodes;
    const float* coords;      // 3 nnodes
    const uint32_t* conn;     // nodes-per-cell x ncells
    uint64_t ncells;
    double iso, vmin, vmax;
    Classifier cls;           // exact thresholds of the isolevel (no FP64 for float / 32-bit values)
    FastIso f;                // constants of the FP32 vertex certificate (emit pass)
    int32_t conn_vec16;       // connections 16-byte aligned: vector loads for tetrahedra / hexahedra
    uint32_t* tile_counts;    // per 32-cell group
    uint64_t* tile_offsets;
    float* out_coords;        // 9 T
    float* out_normals;       // 3 T
    uint64_t cap_tris;
    const uint64_t* d_total;  // emit: the scanned total (device); nothing is written when it exceeds cap_tris
    int* bad_index;           // set to 1 by a connection index >= nnodes
    // slice plane (kvs::SlicePlane on unstructured volumes)
    float coef[4];            // a x + b y + c z + d
    float tf_min, tf_max;     // colour map range
    int32_t tf_res;
    const uint8_t* table;     // device colour table, tf_res x RGB
    uint8_t* out_colors;      // 9 T (RGB per vertex)
    // isolevel sweep: niso records in device memory, group counts / offsets
    // of isolevel k at [k * groups, (k + 1) * groups)
    const CellIso* isos;
    int32_t niso;
};
cudaError_t launch_cells_count(const CellJob& j, const Launch& L);
cudaError_t launch_cells_emit(const CellJob& j, const Launch& L);
uint64_t cells_tiles(uint64_t ncells);
cudaError_t launch_cells_sweep_count(const CellJob& j, const Launch& L);
cudaError_t launch_cells_sweep_emit(const CellJob& j, const Launch& L);
cudaError_t launch_sweep_bases(const uint64_t* offsets, uint64_t groups, int niso, const uint64_t* total,
                               uint64_t* out, const Launch& L);
cudaError_t launch_cells_slice_count(const CellJob& j, const Launch& L);
cudaError_t launch_cells_slice_emit(const CellJob& j, const Launch& L);
// bounding box of the cells' nodes (updateMinMaxCoords' fold), d_out[0..2] min, [3..5] max
size_t cells_bounds_scratch_bytes(int num_sms);
cudaError_t launch_cells_bounds(const CellJob& j, bool has_conn, void* scratch, float* d_out, const Launch& L);
// min/max over values[0] and the connected nodes' values, as doubles in d_out[0..1]
size_t cells_minmax_scratch_bytes(int num_sms);
cudaError_t launch_cells_minmax(const CellJob& j, void* scratch, double* d_out, const Launch& L);

// ---- binary STL records (export.cu): 50 bytes per triangle; bad_index: a
// device word set to 1 when a connection index is >= nverts (that vertex
// then reads as vertex 0)
constexpr uint64_t kStlRecordBytes = 50;
// ---- binary PLY vertex records (ply.cu): colour mode 0 none / 1 one colour /
// 2 per vertex; normal mode 0 none / 1 zeros / 2 per vertex
int ply_record_bytes(int color_mode, int normal_mode);
cudaError_t launch_ply_vertices(const float* coords, const uint8_t* colors, int color_mode, const float* normals,
                                int normal_mode, uint64_t nverts, uint8_t* out, const Launch& L);
cudaError_t launch_stl_records(const float* coords, const float* normals, const uint32_t* conn, uint64_t nverts,
                               uint64_t ntri, int mode, uint8_t* out, int* bad_index, const Launch& L);

// ---- ASCII STL text (stl_ascii.cu): per triangle its record length, then
// the records at scanned offsets; triangles [t0, t0 + n) of the mesh
cudaError_t launch_stl_ascii_len(const float* coords, const float* normals, const uint32_t* conn, uint64_t nverts,
                                 uint64_t t0, uint64_t n, int mode, uint32_t* lens, int* bad_index, const Launch& L);
cudaError_t launch_stl_ascii_write(const float* coords, const float* normals, const uint32_t* conn,
                                   uint64_t nverts, uint64_t t0, uint64_t n, int mode, const uint64_t* offsets,
                                   char* out, int* bad_index, const Launch& L);

// ---- diagnostics (selftest.cu)
cudaError_t launch_selftest(uint64_t n, uint64_t seed, unsigned long long* d_counters, const Launch& L);
cudaError_t launch_selftest_cells(uint64_t n, uint64_t seed, unsigned long long* d_counters, const Launch& L);

}  // namespace kvsmc
