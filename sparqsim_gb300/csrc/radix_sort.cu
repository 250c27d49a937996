// radix_sort.cu — onesweep LSD radix sort of (key, uint32 index) pairs.
//
// One histogram kernel reads the keys once and counts every 8-bit digit of
// every pass; passes whose digit is constant over all keys are skipped. Each
// remaining pass is one kernel: a tile of 2048 or 4096 keys is ranked per
// digit with warp match (stable, in index order), each tile publishes its 256
// digit counts and resolves its global offsets by a per-digit decoupled
// look-back (16 predecessors per read), then the tile is staged in shared
// memory in digit order so that the global scatter is written as contiguous
// runs. Per pass the HBM traffic is one read and one write of (key, index).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "lookback.cuh"
#include "sq_internal.cuh"

namespace sq {

constexpr int kRsBlock = 256;
constexpr int kRsWarps = kRsBlock / 32;
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

// Exclusive prefix of digit d over the tiles before `tile`: the tile's count
// is published first (flag 1), then the predecessors are read kRsWindow at a
// time (independent loads, so one window costs one L2 round trip) and their
// counts summed back to the first inclusive prefix (flag 2), which ends the
// walk; the tile then publishes its own inclusive prefix. A status word holds
// flag and count together, so relaxed loads and stores suffice.
constexpr int kRsWindow = 16;
__device__ __forceinline__ unsigned rs_lookback(unsigned* status, unsigned tile, unsigned d, unsigned cnt,
                                                unsigned* err) {
    if (tile == 0) {
        lb32_store_relaxed(&status[d], kFlag32Pre | cnt);
        return 0;
    }
    lb32_store_relaxed(&status[(size_t)tile * kRadix + d], kFlag32Agg | cnt);
    unsigned excl = 0, spins = 0;
    const unsigned limit = spin_limit(err);
    long long t = (long long)tile - 1;  // next predecessor to read
    while (true) {
        unsigned s[kRsWindow];
#pragma unroll
        for (int q = 0; q < kRsWindow; ++q)
            s[q] = t - q >= 0 ? lb32_load_relaxed(&status[(size_t)(t - q) * kRadix + d]) : kFlag32Pre;
        bool stop = false, found = false;
        int take = 0;
#pragma unroll
        for (int q = 0; q < kRsWindow; ++q) {
            if (stop) continue;
            const unsigned flag = s[q] >> 30;
            if (flag == 0u) {
                stop = true;  // not published yet: read it again
            } else {
                excl += s[q] & kVal32Mask;
                ++take;
                if (flag == 2u) stop = found = true;
            }
        }
        if (found) break;
        t -= take;
        if (take == kRsWindow) {
            spins = 0;
            continue;
        }
        if (++spins > limit) {  // count the missing predecessors as zero
            atomicOr(err, 1u);
            break;
        }
        __nanosleep(32);
    }
    lb32_store_relaxed(&status[(size_t)tile * kRadix + d], kFlag32Pre | (excl + cnt));
    return excl;
}

// Reduce-then-scan form of a pass (no chain between tiles): the upsweep
// counts each tile's digits, counts[d * ntiles + tile]; rs_scan_kernel turns
// them into each tile's first output position per digit; the rank-and-scatter
// kernel (rs_onesweep_kernel, CHAINED = false) reads those. Tiles are the
// same 256 * ITEMS consecutive keys in all three.
template <typename KeyT, int ITEMS>
__global__ void __launch_bounds__(kRsBlock) rs_upsweep_kernel(const KeyT* __restrict__ kin, uint64_t n, int shift,
                                                              unsigned* __restrict__ counts) {
    __shared__ unsigned s_h[kRadix];
    const unsigned tid = threadIdx.x, lane = tid & 31u;
    s_h[tid] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * (kRsBlock * ITEMS);
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint64_t i = base + (uint64_t)j * kRsBlock + tid;
        const bool valid = i < n;
        const unsigned dg = valid ? ((unsigned)(kin[i] >> shift) & 0xffu) : 0xffffffffu;
        // one shared atomic per distinct digit in the warp: sorted or skewed
        // keys would otherwise serialise 32 lanes on one counter
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        if (valid && (int)lane == __ffs(peers) - 1) atomicAdd(&s_h[dg], (unsigned)__popc(peers));
    }
    __syncthreads();
    counts[(size_t)tid * gridDim.x + blockIdx.x] = s_h[tid];
}

// One CTA per digit d: offs[d * ntiles + t] = digit_base[d] + the digit's
// count over tiles 0..t-1 (an exclusive scan along the digit's row, 1024
// tiles per step with a running carry). `offs` may alias `counts`.
__global__ void __launch_bounds__(kRsBlock) rs_scan_kernel(const unsigned* counts, unsigned ntiles,
                                                           const unsigned* __restrict__ digit_base, unsigned* offs) {
    __shared__ unsigned s_w[kRsWarps];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, d = blockIdx.x;
    const unsigned* row = counts + (size_t)d * ntiles;
    unsigned* orow = offs + (size_t)d * ntiles;
    unsigned carry = digit_base[d];
    for (unsigned t0 = 0; t0 < ntiles; t0 += 4 * kRsBlock) {
        unsigned v[4], sum = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const unsigned t = t0 + tid * 4 + q;
            v[q] = t < ntiles ? row[t] : 0u;
            sum += v[q];
        }
        unsigned inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned x = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (unsigned)o) inc += x;
        }
        if (lane == 31) s_w[warp] = inc;
        __syncthreads();
        unsigned wpre = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kRsWarps; ++w) {
            if ((unsigned)w < warp) wpre += s_w[w];
            total += s_w[w];
        }
        unsigned run = carry + wpre + inc - sum;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const unsigned t = t0 + tid * 4 + q;
            if (t < ntiles) orow[t] = run;
            run += v[q];
        }
        carry += total;
        __syncthreads();  // s_w is rewritten by the next step
    }
}

// Peer masks of a warp's equal digits: MATCH_ANY = __match_any_sync (the
// default); MATCH_OR = each lane ORs its bit into a per-warp shared word of
// its digit and reads the word back (the leader, its lowest lane, clears it),
// 7 % slower over a QDA walk step's sorts; SPARQ_RADIX_RANK=1 selects it.
enum { RANK_MATCH_ANY = 0, RANK_MATCH_OR = 1 };

// CHAINED: the tile's digit offsets come from the look-back (status words,
// tile order from `counter`). Otherwise tile = blockIdx.x and its offsets are
// read from `status` laid out digit-major, offs[d * ntiles + tile], as written
// by rs_scan_kernel (`digit_base` and `counter` unused).
template <typename KeyT, int ITEMS, int RANK, bool CHAINED>
__global__ void __launch_bounds__(kRsBlock) rs_onesweep_kernel(const KeyT* __restrict__ kin,
                                                               const unsigned* __restrict__ vin,
                                                               KeyT* __restrict__ kout, unsigned* __restrict__ vout,
                                                               uint64_t n, int shift,
                                                               const unsigned* __restrict__ digit_base,
                                                               unsigned* status, unsigned* counter, unsigned* err) {
    constexpr int kTile = kRsBlock * ITEMS;
    extern __shared__ __align__(16) unsigned char rs_smem[];
    KeyT* s_k = reinterpret_cast<KeyT*>(rs_smem);                       // kTile keys
    unsigned* s_v = reinterpret_cast<unsigned*>(rs_smem + sizeof(KeyT) * kTile);  // kTile indices
    __shared__ unsigned s_tile;
    __shared__ unsigned s_whist[kRsWarps][kRadix];
    __shared__ unsigned s_tstart[kRadix];
    __shared__ unsigned s_gbase[kRadix];
    __shared__ unsigned s_wsum[kRsWarps];
    __shared__ unsigned s_match[RANK == RANK_MATCH_OR ? kRsWarps : 1][kRadix];

    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (CHAINED && tid == 0) s_tile = atomicAdd(counter, 1u);
    for (int i = tid; i < kRsWarps * kRadix; i += kRsBlock) (&s_whist[0][0])[i] = 0;
    if (RANK == RANK_MATCH_OR)
        for (int i = tid; i < kRsWarps * kRadix; i += kRsBlock) (&s_match[0][0])[i] = 0;
    __syncthreads();
    const unsigned tile = CHAINED ? s_tile : blockIdx.x;
    const uint64_t base = (uint64_t)tile * kTile;

    // a warp owns 32 * ITEMS consecutive keys; item j of lane l is key j * 32 + l
    KeyT key[ITEMS];
    unsigned val[ITEMS], rank[ITEMS];
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t wbase = base + (uint64_t)warp * (32 * ITEMS) + lane;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint64_t i = wbase + (uint64_t)j * 32;
        key[j] = i < n ? kin[i] : (KeyT)0;
        val[j] = i < n ? vin[i] : 0u;
    }
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const bool valid = wbase + (uint64_t)j * 32 < n;
        const unsigned dg = valid ? ((unsigned)(key[j] >> shift) & 0xffu) : 0xffffffffu;
        unsigned peers;
        if (RANK == RANK_MATCH_OR) {
            if (valid) atomicOr(&s_match[warp][dg], 1u << lane);
            __syncwarp();
            peers = valid ? s_match[warp][dg] : 0u;
            __syncwarp();
        } else {
            peers = __match_any_sync(0xffffffffu, dg) & __ballot_sync(0xffffffffu, valid);
        }
        const int leader = valid ? (__ffs(peers) - 1) : (int)lane;
        unsigned b = 0;
        if (valid && (int)lane == leader) {
            b = s_whist[warp][dg];
            s_whist[warp][dg] = b + __popc(peers);
            if (RANK == RANK_MATCH_OR) s_match[warp][dg] = 0u;
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
    const unsigned gbase = CHAINED ? digit_base[d] + rs_lookback(status, tile, d, cnt, err)
                                   : status[(size_t)d * gridDim.x + tile];
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
    s_gbase[d] = gbase;
    __syncthreads();

#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        if (wbase + (uint64_t)j * 32 >= n) continue;
        const unsigned dg = (unsigned)(key[j] >> shift) & 0xffu;
        const unsigned pos = s_tstart[dg] + s_whist[warp][dg] + rank[j];
        s_k[pos] = key[j];
        s_v[pos] = val[j];
    }
    __syncthreads();
    const uint64_t rem = n - base;
    const unsigned tile_n = rem < (uint64_t)kTile ? (unsigned)rem : (unsigned)kTile;
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

// Keys per thread of a onesweep tile: 8 (2048-key tiles, four CTAs of 64
// registers per SM). The 16-key form (4096-key tiles, half the look-back
// chains, 128 registers and two CTAs per SM) measured 7 % slower over the
// sorts of a QDA walk step at 2^20 (4M entries); SPARQ_RADIX_ITEMS=16 selects it.
static int radix_rank_mode() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("SPARQ_RADIX_RANK");
        mode = e && atoi(e) == 1 ? RANK_MATCH_OR : RANK_MATCH_ANY;
    }
    return mode;
}

static int radix_tile_items(uint64_t n) {
    static int forced = -1;
    if (forced < 0) {
        const char* e = getenv("SPARQ_RADIX_ITEMS");
        forced = e && (atoi(e) == 8 || atoi(e) == 16) ? atoi(e) : 0;
    }
    (void)n;
    return forced ? forced : 8;
}

// How a pass finds each tile's output offsets: 0 (default) the chained
// onesweep, one launch with a per-digit look-back; 1 reduce-then-scan, three
// launches with no dependence between tiles. Over the sorts of a QDA walk
// step at 2^20 (4M entries, 46 passes) the chained form took 2.48 ms and the
// three-launch form 3.3 ms (its rank-and-scatter alone 1.89 ms, the upsweep
// 1.08 ms): the ranking inside a tile, not the look-back, dominates a pass.
// SPARQ_RADIX_MODE=1 selects the three-launch form.
static int radix_mode() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("SPARQ_RADIX_MODE");
        mode = e && atoi(e) == 1 ? 1 : 0;
    }
    return mode;
}

template <typename KeyT, bool CH>
static auto rs_pick(int items, int rank) {
    if (rank == RANK_MATCH_OR)
        return items == 16 ? rs_onesweep_kernel<KeyT, 16, RANK_MATCH_OR, CH> : rs_onesweep_kernel<KeyT, 8, RANK_MATCH_OR, CH>;
    return items == 16 ? rs_onesweep_kernel<KeyT, 16, RANK_MATCH_ANY, CH> : rs_onesweep_kernel<KeyT, 8, RANK_MATCH_ANY, CH>;
}

template <typename KeyT>
static void radix_set_smem() {
    static bool done = false;
    if (done) return;
    for (int items : {8, 16})
        for (int rank : {RANK_MATCH_ANY, RANK_MATCH_OR}) {
            const int bytes = kRsBlock * items * (int)(sizeof(KeyT) + 4);
            SQ_CUDA(cudaFuncSetAttribute(rs_pick<KeyT, true>(items, rank), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            SQ_CUDA(cudaFuncSetAttribute(rs_pick<KeyT, false>(items, rank), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        }
    done = true;
}

// Sorts (k[0], v[0]) by the low `bits` bits of the key; returns 0 or 1: the
// buffer pair holding the result. Buffers k[1], v[1] are scratch.
template <typename KeyT>
int radix_sort_pairs(KeyT* k[2], unsigned* v[2], uint64_t n, int bits) {
    if (n >= (1ull << 30)) fail(SQ_ERR_CAPACITY, "radix sort limited to < 2^30 keys");
    if (n <= 1 || bits <= 0) return 0;
    radix_set_smem<KeyT>();
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
    const int items = radix_tile_items(n);
    const int rank = radix_rank_mode();
    const bool chained = radix_mode() == 0;
    const unsigned tile = (unsigned)(kRsBlock * items);
    const unsigned ntiles = (unsigned)((n + tile - 1) / tile);
    const size_t smem = (size_t)tile * (sizeof(KeyT) + 4);
    cudaStream_t st = stream();
    int cur = 0;
    if (chained) {
        const size_t per_pass = (size_t)ntiles * kRadix + 64;  // status + counter
        unsigned* lb = (unsigned*)ws().get(WS_LOOKBACK, per_pass * live.size() * 4);
        SQ_CUDA(cudaMemsetAsync(lb, 0, per_pass * live.size() * 4, st));
        for (size_t q = 0; q < live.size(); ++q) {
            const int p = live[q];
            unsigned* status = lb + q * per_pass;
            unsigned* counter = status + (size_t)ntiles * kRadix;
            prof_begin(sizeof(KeyT) == 8 ? "radix_onesweep_u64" : "radix_onesweep_u32");
            rs_pick<KeyT, true>(items, rank)<<<ntiles, kRsBlock, smem, st>>>(
                k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, 8 * p, dbase + (size_t)p * kRadix, status, counter,
                device_error_word());
            prof_end(2.0 * n * (sizeof(KeyT) + 4));  // one read and one write of (key, index)
            SQ_CUDA(cudaGetLastError());
            cur ^= 1;
        }
        return cur;
    }
    // reduce-then-scan: per-tile digit counts, turned in place into offsets
    unsigned* offs = (unsigned*)ws().get(WS_LOOKBACK, (size_t)ntiles * kRadix * 4);
    for (size_t q = 0; q < live.size(); ++q) {
        const int p = live[q];
        prof_begin("radix_upsweep");
        (items == 16 ? rs_upsweep_kernel<KeyT, 16> : rs_upsweep_kernel<KeyT, 8>)<<<ntiles, kRsBlock, 0, st>>>(
            k[cur], n, 8 * p, offs);
        prof_end((double)n * sizeof(KeyT));
        SQ_CUDA(cudaGetLastError());
        prof_begin("radix_tile_scan");
        rs_scan_kernel<<<kRadix, kRsBlock, 0, st>>>(offs, ntiles, dbase + (size_t)p * kRadix, offs);
        prof_end(2.0 * ntiles * kRadix * 4);
        SQ_CUDA(cudaGetLastError());
        prof_begin(sizeof(KeyT) == 8 ? "radix_scatter_u64" : "radix_scatter_u32");
        rs_pick<KeyT, false>(items, rank)<<<ntiles, kRsBlock, smem, st>>>(
            k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, 8 * p, nullptr, offs, nullptr, device_error_word());
        prof_end(2.0 * n * (sizeof(KeyT) + 4));
        SQ_CUDA(cudaGetLastError());
        cur ^= 1;
    }
    return cur;
}

template int radix_sort_pairs<uint32_t>(uint32_t* k[2], unsigned* v[2], uint64_t n, int bits);
template int radix_sort_pairs<uint64_t>(uint64_t* k[2], unsigned* v[2], uint64_t n, int bits);

}  // namespace sq
