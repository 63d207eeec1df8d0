// batch.h -- the streaming batch runner (batch.cu).
#pragma once
#include <vector>

#include "context.h"

namespace kvsmc_host {

kvsmc::FastIso make_fast(double iso, double vmin, double vmax, int dtype);

// Bucket parameters of a group's sorted thresholds.
void bucket_params(float t0, float t1, float& bs, float& bo);

// Cell planes per warp task for a volume (enough tasks to fill the GPU, at
// most 64 planes so the one-plane halo of a task stays small).
uint32_t stream_zchunk(const kvsmc::VolumeView& v, uint32_t wpr, int num_sms);

// A batch of streaming-eligible requests.  plan() builds the work tables,
// count() fills every item's sizes, emit() writes the outputs of the items
// with emit set and enough capacity (status OK), finish() waits for them.
// The tables live in the context's scratch arena from plan() to finish().
struct StreamBatch {
    kvsmc_context* ctx = nullptr;
    std::vector<Item*> items;

    struct Launch1 {
        int dtype;
        int g0, ng;
        uint64_t ntasks;
    };
    std::vector<kvsmc::StreamGroup> groups;
    std::vector<kvsmc::StreamIso> isos;
    std::vector<Item*> iso_item;
    std::vector<Launch1> launches;
    uint64_t unit_elems = 0;     // (unit, isolevel) counters
    uint32_t scan_blocks = 0;    // unit-scan blocks: one per (group, z)
    uint64_t iso_planes = 0;     // (isolevel, z) planes

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

    kvsmc_status plan();
    kvsmc_status count();
    kvsmc_status emit();
    kvsmc_status finish();

  private:
    kvsmc_status upload_tables();
};

}  // namespace kvsmc_host
