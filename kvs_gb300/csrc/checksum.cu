// checksum.cu -- position-keyed checksums of device arrays, and the test hook
// that caps the streaming kernels' plane waits.
//
// The checksum lets a caller compare outputs of billions of triangles with a
// CPU run of the same extraction without copying them back: per chunk of
// `chunk_words` 32-bit words, the sum (mod 2^64) of mix(i, w_i) over the
// chunk's words, i the word's index from the start of the array.  Because
// the index enters every term, the sum changes when words are permuted as
// well as when any bit changes; because it is a sum, blocks add their parts
// in any order and the result is deterministic.
#include <cstring>

#include "context.h"

namespace kvsmc {

namespace {

// mix(i, w): a 64-bit multiply-xorshift finaliser of the index and the word.
__device__ __forceinline__ uint64_t mix_word(uint64_t i, uint32_t w)
{
    uint64_t x = (i * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)w * 0xC2B2AE3D27D4EB4Full);
    x ^= x >> 31;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 29;
    return x;
}

constexpr int kSumThreads = 256;

// grid (blocks per chunk, chunks): each block sums a strided share of its chunk
__global__ void __launch_bounds__(kSumThreads)
    k_checksum(const uint32_t* __restrict__ words, uint64_t n, uint64_t chunk_words,
               unsigned long long* __restrict__ sums)
{
    const uint64_t c = blockIdx.y;
    const uint64_t lo = c * chunk_words;
    const uint64_t hi = lo + chunk_words < n ? lo + chunk_words : n;
    uint64_t acc = 0;
    for (uint64_t i = lo + (uint64_t)blockIdx.x * kSumThreads + threadIdx.x; i < hi;
         i += (uint64_t)gridDim.x * kSumThreads)
        acc += mix_word(i, __ldcs(words + i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ uint64_t part[kSumThreads / 32];
    if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t s = 0;
        for (int w = 0; w < kSumThreads / 32; ++w) s += part[w];
        atomicAdd(sums + c, (unsigned long long)s);
    }
}

}  // namespace

}  // namespace kvsmc

extern "C" {

kvsmc_status kvsmc_checksum_words(kvsmc_context* ctx, const void* d_words, uint64_t nwords, uint64_t chunk_words,
                                  uint64_t* sums, uint64_t nchunks)
{
    using namespace kvsmc_host;
    if (!ctx || !sums || (!d_words && nwords) || chunk_words == 0) return KVSMC_ERR_INVALID_ARGUMENT;
    if ((nwords + chunk_words - 1) / chunk_words > nchunks || nchunks > 65535)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "checksum: %llu chunks do not fit %llu",
                    (unsigned long long)((nwords + chunk_words - 1) / chunk_words), (unsigned long long)nchunks);
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    std::memset(sums, 0, nchunks * sizeof(uint64_t));
    if (nwords == 0) return KVSMC_OK;
    kvsmc_status st = ensure_scratch(ctx, nchunks * sizeof(uint64_t));
    if (st) return st;
    unsigned long long* d = static_cast<unsigned long long*>(ctx->scratch);
    KVSMC_CUDA(ctx, cudaMemsetAsync(d, 0, nchunks * sizeof(uint64_t), ctx->stream));
    const uint64_t used = (nwords + chunk_words - 1) / chunk_words;
    // about 8 blocks per SM over all chunks, at least one block per chunk
    uint64_t per = ((uint64_t)ctx->num_sms * 8 + used - 1) / used;
    const uint64_t cap = (chunk_words + kvsmc::kSumThreads - 1) / kvsmc::kSumThreads;
    if (per > cap) per = cap;
    if (per < 1) per = 1;
    const kvsmc::Launch L = launch_of(ctx);
    kvsmc::prof_begin(L, "checksum");
    kvsmc::k_checksum<<<dim3((unsigned)per, (unsigned)used), kvsmc::kSumThreads, 0, ctx->stream>>>(
        static_cast<const uint32_t*>(d_words), nwords, chunk_words, d);
    kvsmc::prof_end(L);
    ctx->launches += 1;
    KVSMC_CUDA(ctx, cudaGetLastError());
    KVSMC_CUDA(ctx, cudaMemcpyAsync(sums, d, used * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

kvsmc_status kvsmc_set_wait_limit(kvsmc_context* ctx, int64_t count_polls, int64_t emit_polls)
{
    if (!ctx || count_polls > 0xffffffffLL || emit_polls > 0xffffffffLL) return KVSMC_ERR_INVALID_ARGUMENT;
    ctx->wait_polls[0] = count_polls < 0 ? kvsmc::kStreamWaitPolls : (uint32_t)count_polls;
    ctx->wait_polls[1] = emit_polls < 0 ? kvsmc::kStreamWaitPolls : (uint32_t)emit_polls;
    return KVSMC_OK;
}

}  // extern "C"
