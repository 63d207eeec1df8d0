// batch.h -- the streaming batch runner (batch.cu).
#pragma once
#include <vector>

#include "context.h"

namespace kvsmc_host {

kvsmc::FastIso make_fast(double iso, double vmin, double vmax, int dtype);
// Warps per row, cell rows per y-tile and staged plane size of a volume.
void tiling(const kvsmc::VolumeView& v, uint32_t& wpr, uint32_t& rows, uint64_t& plane_elems);

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
        uint32_t nctas;
        size_t smem_count, smem_emit;
    };
    std::vector<kvsmc::StreamGroup> groups;
    std::vector<kvsmc::StreamIso> isos;
    std::vector<Item*> iso_item;
    std::vector<Launch1> launches;
    uint64_t total_tiles = 0;

    kvsmc::StreamGroup* d_groups = nullptr;
    kvsmc::StreamIso* d_isos = nullptr;
    uint32_t* d_counts = nullptr;
    uint64_t* d_offsets = nullptr;
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
