// batch.h -- the streaming batch runner (batch.cu).
#pragma once
#include <functional>
#include <vector>

#include "context.h"

namespace kvsmc_host {

kvsmc::FastIso make_fast(double iso, double vmin, double vmax, int dtype);

// Bucket parameters of a group's sorted thresholds.
void bucket_params(float t0, float t1, float& bs, float& bo);

// Cell planes per warp task for a launch of `warp_steps` (row segment, plane)
// steps in all: about tasks_per_sm tasks per SM (the built-in rule: 96),
// 4 to 64 planes per task (the one-plane halo a task re-reads stays small).
constexpr int kDefaultTasksPerSm = 96;
uint32_t stream_zchunk(uint64_t warp_steps, int num_sms, int tasks_per_sm = kDefaultTasksPerSm);

// Cell rows per warp task for rows of cx cells: 2 (128-cell segments) when
// that idles fewer lanes than 256-cell segments, else 1.
int stream_rows(uint32_t cx);

// Row segments per cell row of a volume tiled with `rows` cell rows per warp
// task (256 / rows cells per segment).
inline uint32_t segments_per_row(const kvsmc::VolumeView& v, int rows)
{
    const uint32_t seg = kvsmc::kStreamSegCells / rows;
    return (v.nx - 1 + seg - 1) / seg;
}

// Warp tasks of one volume: (cell-row groups) x segments x z-chunks.
inline uint64_t stream_tasks(const kvsmc::VolumeView& v, int rows, uint32_t wpr, uint32_t zchunk)
{
    const uint32_t cy = v.ny - 1, cz = v.nz - 1;
    return (uint64_t)((cy + rows - 1) / rows) * wpr * ((cz + zchunk - 1) / zchunk);
}

// (unit, isolevel) counters of one volume: one per (z, cell row, segment, isolevel).
inline uint64_t stream_units(const kvsmc::VolumeView& v, uint32_t wpr, int niso)
{
    return (uint64_t)(v.nz - 1) * (v.ny - 1) * wpr * (uint64_t)niso;
}

// A batch of streaming-eligible requests.  plan() builds the work tables,
// count() fills every item's sizes, emit() writes the outputs of the items
// with emit set and enough capacity (status OK), finish() waits for them.
// The tables live in the context's scratch arena from plan() to finish().
struct StreamBatch {
    kvsmc_context* ctx = nullptr;
    std::vector<Item*> items;

    struct Launch1 {
        int dtype;
        int rows;
        int g0, ng;
        uint64_t ntasks;
        int ctas_per_sm;   // 0: as many as fit
    };
    std::vector<kvsmc::StreamGroup> groups;
    std::vector<kvsmc::StreamIso> isos;
    std::vector<Item*> iso_item;
    std::vector<Launch1> launches;
    uint64_t unit_elems = 0;     // (unit, isolevel) counters
    uint32_t scan_blocks = 0;    // unit-scan blocks: one per (group, z)
    int scan_threads = 256;      // unit-scan tile
    uint64_t iso_planes = 0;     // (isolevel, z) planes
    // the count pass also counts the shared-vertex modes' vertices per
    // (isolevel, node unit) for the groups that take one row per task and
    // whose node segments are its cell segments (set before plan_tables)
    bool want_nodes = false;
    uint64_t node_elems = 0;
    uint32_t* d_node_counts = nullptr;

    kvsmc::StreamGroup* d_groups = nullptr;
    kvsmc::StreamIso* d_isos = nullptr;
    uint16_t* d_unit_counts = nullptr;
    uint32_t* d_unit_offsets = nullptr;
    uint32_t* d_plane_totals = nullptr;
    uint64_t* d_plane_base = nullptr;
    void* d_scan = nullptr;
    uint64_t* d_totals = nullptr;
    uint64_t* d_total = nullptr;
    int* d_status = nullptr;
    unsigned long long* d_next = nullptr;   // per launch: [2 i] count, [2 i + 1] emit task counter

    unsigned long long* d_next_parts = nullptr;   // task counters of a split emit (kMaxParts)
    static constexpr int kMaxParts = 16;

    kvsmc_status plan();
    kvsmc_status count();
    kvsmc_status emit();
    kvsmc_status finish();

    // The emit as up to `parts` launches over consecutive ranges of cell
    // planes, so the outputs of a finished range can leave while the next
    // range is written.  Splits only a batch of one group (one volume, at
    // most 16 isolevels); otherwise one launch.  After enqueueing each launch
    // on the context's stream it calls after(z_begin, z_end, whole): the
    // outputs of cell planes [z_begin, z_end) (every output when whole) are
    // complete once the stream reaches that point.
    kvsmc_status emit_parts(int parts, const std::function<kvsmc_status(uint32_t, uint32_t, bool)>& after);

    // The pieces of plan(): host tables, their device footprint, and the
    // device pointers carved from a region of scratch_bytes().
    void plan_tables();
    size_t scratch_bytes() const;
    void carve(char* base);
    kvsmc_status upload_tables();
};

// Triangles an item's output buffers hold (coords / 9, normals / 3).
uint64_t cap_triangles(const Item& it);

}  // namespace kvsmc_host
