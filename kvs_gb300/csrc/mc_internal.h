// mc_internal.h -- host-side declarations shared by the library's .cu files.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mc_device.cuh"

namespace kvsmc {

// Launch bookkeeping passed to every launcher.
struct Launch {
    cudaStream_t stream;
    int num_sms;
    uint64_t* counter;   // incremented once per kernel launch
};

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

// ---- gather-form kernels (mc_gather.cu)
cudaError_t launch_cell_count(const Job& j, const Launch& L);
cudaError_t launch_emit_dup(const Job& j, const Launch& L);
cudaError_t launch_node_count(const Job& j, const Launch& L);
cudaError_t launch_node_emit(const Job& j, const Launch& L);
cudaError_t launch_connect(const Job& j, const Launch& L);
cudaError_t launch_vertex_normals(const Job& j, const Launch& L);

}  // namespace kvsmc
