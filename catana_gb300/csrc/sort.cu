// sort.cu -- stable LSD radix sort of (uint32 key, uint32 index) pairs on the GPU.
//
// Used to group points: by HEALPix pixel for the binned catalog (the reference
// appends radii to per-pixel vectors in point order, PixelizedPointContainer.cpp:27-30,
// so the sort must be stable) and by quantised radius for the split form (points
// with nearly equal r share j_l table intervals, which turns the shared-memory table
// reads into broadcasts).
//
// One pass per 8-bit digit:
//   k_radix_hist     per-tile digit histogram (tile = 4096 consecutive pairs)
//   k_radix_scan     exclusive scan of the (digit-major, tile-minor) histogram
//   k_radix_scatter  each tile re-reads its pairs in order, 256 at a time, ranks equal
//                    digits with __match_any_sync within a warp and with per-warp
//                    counts across warps, and scatters -- a stable, deterministic order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace catana_gpu {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_TILE = 4096;  // pairs per tile (16 rounds of 256)
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void k_radix_hist(const uint32_t *__restrict__ keys, int64_t n, int shift, uint32_t *__restrict__ hist,
                             int ntiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int k = threadIdx.x; k < RS_TILE; k += RS_THREADS) {
        const int64_t i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Single-CTA exclusive scan of count entries (1024 threads, contiguous segments).
__global__ void k_radix_scan(uint32_t *__restrict__ data, int64_t count) {
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    const int64_t seg = (count + 1023) / 1024;
    const int64_t b = t * seg, e = min(count, b + seg);
    uint32_t s = 0;
    for (int64_t i = b; i < e; ++i) s += data[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - s;  // exclusive prefix of this segment
    for (int64_t i = b; i < e; ++i) {
        const uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
}

__global__ void k_radix_scatter(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, int64_t n,
                                int shift, const uint32_t *__restrict__ offs, int ntiles,
                                uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[RS_WARPS][256];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    base[t] = offs[(size_t)t * ntiles + blockIdx.x];
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t tile0 = (int64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_TILE / RS_THREADS; ++r) {
        const int64_t i = tile0 + (int64_t)r * RS_THREADS + t;
        const bool valid = i < n;
        uint32_t key = 0, val = 0, d = 0xFFFFFFFFu;  // invalid lanes form their own group
        if (valid) {
            key = keys[i];
            val = vals[i];
            d = (key >> shift) & 255u;
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (int w = 0; w < warp; ++w) before += wcnt[w][d];
            const uint32_t dst = base[d] + before + rank;
            keys_out[dst] = key;
            vals_out[dst] = val;
        }
        __syncthreads();
        uint32_t tot = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
            tot += wcnt[w][t];
            wcnt[w][t] = 0;
        }
        base[t] += tot;
        __syncthreads();
    }
}

}  // namespace

// In-place exclusive scan of count uint32 words (single CTA; counts up to a few
// million entries).
catana_status_t scan_u32(uint32_t *data, int64_t count, cudaStream_t st) {
    if (count <= 0) return CATANA_OK;
    k_radix_scan<<<1, 1024, 0, st>>>(data, count);
    count_launch();
    CG_CUDA_TRY(cudaGetLastError());
    return CATANA_OK;
}

// Sorts (keys, vals) by the low `key_bits` bits of the keys, stably.  The result
// ends in (keys, vals); tmp_keys / tmp_vals are scratch of n entries; hist_scratch
// holds 256 * ceil(n / 4096) words.
catana_status_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tmp_keys, uint32_t *tmp_vals, int64_t n,
                                 int key_bits, uint32_t *hist_scratch, cudaStream_t st) {
    if (n <= 1) return CATANA_OK;
    const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    uint32_t *ka = keys, *va = vals, *kb = tmp_keys, *vb = tmp_vals;
    int passes = 0;
    for (int shift = 0; shift < key_bits; shift += 8, ++passes) {
        k_radix_hist<<<ntiles, RS_THREADS, 0, st>>>(ka, n, shift, hist_scratch, ntiles);
        k_radix_scan<<<1, 1024, 0, st>>>(hist_scratch, (int64_t)256 * ntiles);
        k_radix_scatter<<<ntiles, RS_THREADS, 0, st>>>(ka, va, n, shift, hist_scratch, ntiles, kb, vb);
        count_launch(3);
        CG_CUDA_TRY(cudaGetLastError());
        uint32_t *t;
        t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
    }
    if (passes & 1) {  // result sits in the scratch arrays: copy back
        CG_CUDA_TRY(cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        CG_CUDA_TRY(cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    }
    return CATANA_OK;
}

}  // namespace catana_gpu
