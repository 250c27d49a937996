// radix_sort.cu — onesweep LSD radix sort of (key, uint32 index) pairs.
//
// One histogram kernel reads the keys once and counts every 8-bit digit of
// every pass; passes whose digit is constant over all keys are skipped. Each
// remaining pass is one kernel: a tile of 2048 keys is ranked per digit with
// warp match (stable, in index order), each tile publishes its 256 digit
// counts and resolves its global offsets by a per-digit decoupled look-back,
// then the tile is staged in shared memory in digit order so that the global
// scatter is written as contiguous runs. Per pass the HBM traffic is one read
// and one write of (key, index).
#include <algorithm>
#include <cstring>
#include <vector>

#include "lookback.cuh"
#include "sq_internal.cuh"

namespace sq {

constexpr int kRsBlock = 256;
constexpr int kRsWarps = kRsBlock / 32;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsBlock * kRsItems;
constexpr int kRadix = 256;

template <typename KeyT>
__global__ void __launch_bounds__(kRsBlock) rs_histogram_kernel(const KeyT* __restrict__ keys, uint64_t n,
                                                                int passes, unsigned* __restrict__ hist) {
    __shared__ unsigned s_h[8][kRadix];
    for (int i = threadIdx.x; i < 8 * kRadix; i += kRsBlock) (&s_h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const KeyT k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&s_h[p][(unsigned)(k >> (8 * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += kRsBlock) {
        const unsigned v = (&s_h[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

template <typename KeyT>
__global__ void __launch_bounds__(kRsBlock) rs_onesweep_kernel(const KeyT* __restrict__ kin,
                                                               const unsigned* __restrict__ vin,
                                                               KeyT* __restrict__ kout, unsigned* __restrict__ vout,
                                                               uint64_t n, int shift,
                                                               const unsigned* __restrict__ digit_base,
                                                               unsigned* status, unsigned* counter, unsigned* err) {
    __shared__ unsigned s_tile;
    __shared__ unsigned s_whist[kRsWarps][kRadix];
    __shared__ unsigned s_tstart[kRadix];
    __shared__ unsigned s_gbase[kRadix];
    __shared__ unsigned s_wsum[kRsWarps];
    __shared__ KeyT s_k[kRsTile];
    __shared__ unsigned s_v[kRsTile];

    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    for (int i = tid; i < kRsWarps * kRadix; i += kRsBlock) (&s_whist[0][0])[i] = 0;
    __syncthreads();
    const unsigned tile = s_tile;
    const uint64_t base = (uint64_t)tile * kRsTile;

    KeyT key[kRsItems];
    unsigned val[kRsItems], rank[kRsItems], dg[kRsItems];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        const uint64_t i = base + (uint64_t)warp * (32 * kRsItems) + (uint64_t)j * 32 + lane;
        const bool valid = i < n;
        key[j] = valid ? kin[i] : (KeyT)0;
        val[j] = valid ? vin[i] : 0u;
        dg[j] = valid ? ((unsigned)(key[j] >> shift) & 0xffu) : 0xffffffffu;
    }
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        const bool valid = dg[j] != 0xffffffffu;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        const unsigned peers = __match_any_sync(0xffffffffu, dg[j]) & vmask;
        const int leader = valid ? (__ffs(peers) - 1) : (int)lane;
        unsigned b = 0;
        if (valid && (int)lane == leader) {
            b = s_whist[warp][dg[j]];
            s_whist[warp][dg[j]] = b + __popc(peers);
        }
        b = __shfl_sync(0xffffffffu, b, leader);
        rank[j] = b + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // digit d = tid: exclusive prefix over warps, tile count, look-back
    const unsigned d = tid;
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
        const unsigned t = s_whist[w][d];
        s_whist[w][d] = run;
        run += t;
    }
    const unsigned cnt = run;
    unsigned excl = 0;
    if (tile == 0) {
        lb32_store(&status[d], kFlag32Pre | cnt);
    } else {
        lb32_store(&status[(size_t)tile * kRadix + d], kFlag32Agg | cnt);
        long long t = (long long)tile - 1;
        unsigned spins = 0;
        while (t >= 0) {
            const unsigned s = lb32_load(&status[(size_t)t * kRadix + d]);
            const unsigned flag = s >> 30;
            if (flag == 0u) {
                if (++spins > kSpinLimit) {
                    atomicOr(err, 1u);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            excl += s & kVal32Mask;
            if (flag == 2u) break;
            --t;
            spins = 0;
        }
        lb32_store(&status[(size_t)tile * kRadix + d], kFlag32Pre | (excl + cnt));
    }
    // block exclusive scan of cnt over digits -> tile-local digit start
    unsigned inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) s_wsum[warp] = inc;
    __syncthreads();
    unsigned wpre = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w)
        if ((unsigned)w < warp) wpre += s_wsum[w];
    const unsigned tstart = wpre + inc - cnt;
    s_tstart[d] = tstart;
    s_gbase[d] = digit_base[d] + excl;
    __syncthreads();

#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        if (dg[j] == 0xffffffffu) continue;
        const unsigned pos = s_tstart[dg[j]] + s_whist[warp][dg[j]] + rank[j];
        s_k[pos] = key[j];
        s_v[pos] = val[j];
    }
    __syncthreads();
    const uint64_t rem = n - base;
    const unsigned tile_n = rem < (uint64_t)kRsTile ? (unsigned)rem : (unsigned)kRsTile;
    for (unsigned p = tid; p < tile_n; p += kRsBlock) {
        const KeyT k = s_k[p];
        const unsigned dd = (unsigned)(k >> shift) & 0xffu;
        const uint64_t o = (uint64_t)s_gbase[dd] + (p - s_tstart[dd]);
        // digit bases computed on the host from this sort's histogram: a
        // replayed graph whose keys differ from the recorded ones could point
        // past the end (its replay is reported invalid; nothing is written there)
        if (o < n) {
            kout[o] = k;
            vout[o] = s_v[p];
        } else {
            atomicOr(err, 32u);
        }
    }
}

// Sorts (k[0], v[0]) by the low `bits` bits of the key; returns 0 or 1: the
// buffer pair holding the result. Buffers k[1], v[1] are scratch.
template <typename KeyT>
int radix_sort_pairs(KeyT* k[2], unsigned* v[2], uint64_t n, int bits) {
    if (n >= (1ull << 30)) fail(SQ_ERR_CAPACITY, "radix sort limited to < 2^30 keys");
    if (n <= 1 || bits <= 0) return 0;
    const int passes = (bits + 7) / 8;
    unsigned* hist = (unsigned*)ws().get(WS_HIST, (size_t)2 * 8 * kRadix * 4);
    SQ_CUDA(cudaMemsetAsync(hist, 0, (size_t)passes * kRadix * 4, stream()));
    prof_begin("radix_histogram");
    rs_histogram_kernel<KeyT><<<grid_for(n, kRsBlock, 4), kRsBlock, 0, stream()>>>(k[0], n, passes, hist);
    prof_end((double)n * sizeof(KeyT));
    SQ_CUDA(cudaGetLastError());
    std::vector<unsigned> h((size_t)passes * kRadix);
    host_read(h.data(), hist, h.size() * 4);
    std::vector<int> live;
    std::vector<unsigned> bases((size_t)passes * kRadix);
    for (int p = 0; p < passes; ++p) {
        unsigned run = 0;
        bool trivial = false;
        for (int d = 0; d < kRadix; ++d) {
            const unsigned c = h[(size_t)p * kRadix + d];
            if (c == n) trivial = true;
            bases[(size_t)p * kRadix + d] = run;
            run += c;
        }
        if (!trivial) live.push_back(p);
    }
    if (live.empty()) return 0;
    unsigned* dbase = hist + (size_t)8 * kRadix;
    h2d_small(dbase, bases.data(), bases.size() * 4);
    const unsigned ntiles = (unsigned)((n + kRsTile - 1) / kRsTile);
    const size_t per_pass = (size_t)ntiles * kRadix + 64;  // status + counter
    unsigned* lb = (unsigned*)ws().get(WS_LOOKBACK, per_pass * live.size() * 4);
    SQ_CUDA(cudaMemsetAsync(lb, 0, per_pass * live.size() * 4, stream()));
    int cur = 0;
    for (size_t q = 0; q < live.size(); ++q) {
        const int p = live[q];
        unsigned* st = lb + q * per_pass;
        unsigned* counter = st + (size_t)ntiles * kRadix;
        prof_begin(sizeof(KeyT) == 8 ? "radix_onesweep_u64" : "radix_onesweep_u32");
        rs_onesweep_kernel<KeyT><<<ntiles, kRsBlock, 0, stream()>>>(k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, 8 * p,
                                                                   dbase + (size_t)p * kRadix, st, counter,
                                                                   device_error_word());
        prof_end(2.0 * n * (sizeof(KeyT) + 4));  // one read and one write of (key, index)
        SQ_CUDA(cudaGetLastError());
        cur ^= 1;
    }
    return cur;
}

template int radix_sort_pairs<uint32_t>(uint32_t* k[2], unsigned* v[2], uint64_t n, int bits);
template int radix_sort_pairs<uint64_t>(uint64_t* k[2], unsigned* v[2], uint64_t n, int bits);

}  // namespace sq
