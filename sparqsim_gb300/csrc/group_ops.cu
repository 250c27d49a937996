// group_ops.cu — split / merge operators: Hadamard_Int, Hadamard_Int_Full,
// Hadamard_Bool, Rot_Bool (general matrix), CondRot_Rational_Bool and the
// equal-key merge of add_systems.
//
// All of them act on groups of entries that agree on every active key bit
// except a few target bits (reference grouping: sort_state.cpp:10-36,
// compare_equal :173-188; StateLessExceptKey buckets in the SAFE_HASH paths).
// Pipeline, every step on the GPU:
//   1. stats: OR/AND of the group-key bits over all entries (which bits vary)
//      and the number of entries failing the control conditions;
//   2. extract: pack only the varying group-key bits (plus a condition-fail
//      bit on top) into a 32- or 64-bit sort key per entry;
//   3. onesweep radix sort of (sort key, entry index);
//   4. segment heads -> group starts (order-preserving compaction);
//   5. emit, count pass: per group, the number of outputs with |a|^2 >= eps;
//      exclusive scan -> output offsets (exact count-then-scan);
//   6. emit, write pass: recompute and write keys + amplitudes; entries that
//      fail the conditions are copied through unchanged.
// Output amplitudes are computed in exactly the reference's arithmetic order
// (stage-ascending FWHT butterflies (a0 + a1) * sqrt2inv, the singleton
// a * 2^{-n/2} shortcut, the pair formulas), so results do not depend on the
// order entries arrive in.
#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "lookback.cuh"
#include "sq_internal.cuh"

namespace sq {

template <typename KeyT>
int radix_sort_pairs(KeyT* k[2], unsigned* v[2], uint64_t n, int bits);
void check_device_error();

constexpr int kMaxRuns = 64;

// Kernels and device helpers have internal linkage: the file is compiled once
// per key width K (-DSQ_GROUP_K=K) plus once for the dispatcher, in parallel.
namespace {

struct Run {
    uint8_t word;
    uint8_t shift;
    uint8_t len;
    uint8_t dst;
};
struct Extract {
    uint32_t nruns;
    uint32_t flag_bit;  // 0xff: no condition bit in this chunk
    Run runs[kMaxRuns];
};

__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ bool keep_amp(double2 a, double eps) { return sq_keep_amp(a.x, a.y, eps); }
// Store of a or -a (the bits of a * -1.0 for every non-NaN a) as integer
// bits: a negation kept in double registers would be issued as an FP64 add.
template <int K>
__device__ __forceinline__ void store_entry_sign(const KeyPtrs& kp, double2* amp, unsigned long long o,
                                                 const uint64_t (&k)[K], double2 a, bool negate) {
#pragma unroll
    for (int w = 0; w < K; ++w) kp.w[w][o] = k[w];
    const unsigned long long s = negate ? 0x8000000000000000ull : 0ull;
    reinterpret_cast<ulonglong2*>(amp)[o] = make_ulonglong2((unsigned long long)__double_as_longlong(a.x) ^ s,
                                                            (unsigned long long)__double_as_longlong(a.y) ^ s);
}

// ------------------------------------------------------------------ exact-sum FWHT arithmetic
// FP64 runs at a small fraction of the integer rate on this part, and an
// n-stage butterfly network costs 4n FP64 operations per slot. In the
// exact-sum arithmetic a group's amplitudes are put on one integer grid,
//     X = round(x * 2^(F - E)),  E = emax - 1022,  F = 62 - n,
// where emax is the largest biased exponent among the group's components (so
// every |x| < 2^E and |X| < 2^F); the n stages of sums and differences are then
// exact in int64 (|partial sum| < 2^62), and each output is rounded once:
//     y = Y * 2^(E - F) * 2^(-n/2)  (times 1/sqrt(2) once more for odd n).
// The only other error is the grid rounding of each input, at most
// 2^(E - F - 1) per component. Zero or subnormal components count as biased
// exponent 1; a group holding inf or NaN gives unspecified amplitudes.
__device__ __forceinline__ int amp_exp(double2 v) {
    const int ex = (int)((unsigned long long)__double_as_longlong(v.x) >> 52) & 0x7ff;
    const int ey = (int)((unsigned long long)__double_as_longlong(v.y) >> 52) & 0x7ff;
    const int e = ex > ey ? ex : ey;
    return e ? e : 1;
}
__device__ __forceinline__ long long to_fixed(double x, int emax, int F) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)(b >> 52) & 0x7ff;
    unsigned long long mant = b & 0xfffffffffffffull;
    if (ex) mant |= 1ull << 52;
    const int r = emax - (ex ? ex : 1) + 53 - F;  // right shift; >= n - 9
    unsigned long long q;
    if (r <= 0) q = mant << (-r);
    else if (r >= 64) q = 0;
    else q = (mant + (1ull << (r - 1))) >> r;  // half away from zero
    return (b >> 63) ? -(long long)q : (long long)q;
}
// The same for F <= 52 (n >= 10), where the shift is always a right shift:
// branch-free (a shift past the mantissa rounds to 0 at 63 just as at 64+).
__device__ __forceinline__ long long to_fixed_right(double x, int emax, int F) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)(b >> 52) & 0x7ff;
    const unsigned long long mant = (b & 0xfffffffffffffull) | (ex ? (1ull << 52) : 0ull);
    const int r = min(emax - (ex ? ex : 1) + 53 - F, 63);
    const unsigned long long q = (mant + (1ull << (r - 1))) >> r;
    const unsigned long long sg = 0ull - (b >> 63);  // all ones when negative
    return (long long)((q ^ sg) - sg);
}
__device__ __forceinline__ longlong2 to_fixed2(double2 v, int emax, int F) {
    return make_longlong2(to_fixed(v.x, emax, F), to_fixed(v.y, emax, F));
}
// outside the normal range (two roundings); a call of its own, so that the
// conversion is not issued for every slot
static __device__ __noinline__ double fixed_to_double_scaled(long long Y, int e2) { return scalbn((double)Y, e2); }
// Y * 2^e2 rounded to nearest even (|Y| < 2^63)
__device__ __forceinline__ double fixed_to_double(long long Y, int e2) {
    if (Y == 0) return 0.0;
    const unsigned long long sign = (unsigned long long)Y & 0x8000000000000000ull;
    const unsigned long long m = sign ? 0ull - (unsigned long long)Y : (unsigned long long)Y;
    const int top = 63 - __clzll((long long)m);
    int ex = top;
    unsigned long long q;
    if (top > 52) {
        const int sh = top - 52;
        q = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
        if (q >> 53) {
            q >>= 1;
            ++ex;
        }
    } else {
        q = m << (52 - top);
    }
    const int be = ex + e2 + 1023;
    if (be <= 0 || be >= 2047) return fixed_to_double_scaled(Y, e2);
    return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (q & 0xfffffffffffffull)));
}
// An exactly zero component stays +0.0 without the FP64 multiply (0 * s2 is
// +0.0): merges leave most slots zero, and FP64 issue is scarce on GB300.
__device__ __forceinline__ double2 from_fixed2(longlong2 v, int e2, bool odd, double s2) {
    double2 r = make_double2(fixed_to_double(v.x, e2), fixed_to_double(v.y, e2));
    if (odd && (v.x | v.y)) r = cscale(r, s2);
    return r;
}
// 1/sqrt(2^n) for a batched group's width n (0..63), as 1.0 / sqrt(2^n)
// rounds it, built from exponent bits instead of an FP64 square root and
// division: 2^(-n/2) for even n; for odd n sqrt(2^n) = 2^((n-1)/2) sqrt(2)
// scales exactly, so the quotient is sqrt2inv (= 1/sqrt(2) rounded) times
// 2^(-(n-1)/2).
__device__ __forceinline__ double inv_sqrt_pow2(int n, double sqrt2inv) {
    if (n & 1) return __longlong_as_double(__double_as_longlong(sqrt2inv) - ((long long)(n >> 1) << 52));
    return __longlong_as_double((long long)(1023 - (n >> 1)) << 52);
}
__device__ __forceinline__ longlong2 ladd(longlong2 a, longlong2 b) { return make_longlong2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ longlong2 lsub(longlong2 a, longlong2 b) { return make_longlong2(a.x - b.x, a.y - b.y); }
// output scale exponent of an n-stage exact-sum FWHT: E - F - floor(n/2)
__device__ __forceinline__ int fix_out_exp(int emax, int n) { return emax - 1022 - (62 - n) - (n >> 1); }

// ------------------------------------------------------------------ 1. stats
template <int K>
__global__ void __launch_bounds__(256) stats_kernel(ConstKeyPtrs keys, uint64_t n, DCondSet cond,
                                                    const uint64_t* __restrict__ gmask_in,
                                                    unsigned long long* __restrict__ out /* [K or, K and, fail] */) {
    __shared__ unsigned long long s_or[K], s_and[K];
    __shared__ unsigned long long s_fail;
    uint64_t gm[K];
#pragma unroll
    for (int w = 0; w < K; ++w) gm[w] = gmask_in[w];
    if (threadIdx.x < K) {
        s_or[threadIdx.x] = 0;
        s_and[threadIdx.x] = ~0ull;
    }
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    uint64_t o[K], a[K];
#pragma unroll
    for (int w = 0; w < K; ++w) {
        o[w] = 0;
        a[w] = ~0ull;
    }
    unsigned long long fails = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = keys.w[w][i];
        if (!cond_ok<K>(k, cond)) {
            ++fails;
            continue;
        }
#pragma unroll
        for (int w = 0; w < K; ++w) {
            o[w] |= k[w] & gm[w];
            a[w] &= k[w] & gm[w];
        }
    }
#pragma unroll
    for (int w = 0; w < K; ++w) {
        for (int s = 16; s > 0; s >>= 1) {
            o[w] |= __shfl_xor_sync(0xffffffffu, o[w], s);
            a[w] &= __shfl_xor_sync(0xffffffffu, a[w], s);
        }
    }
    for (int s = 16; s > 0; s >>= 1) fails += __shfl_xor_sync(0xffffffffu, fails, s);
    if ((threadIdx.x & 31u) == 0) {
#pragma unroll
        for (int w = 0; w < K; ++w) {
            atomicOr(&s_or[w], (unsigned long long)o[w]);
            atomicAnd(&s_and[w], (unsigned long long)a[w]);
        }
        atomicAdd(&s_fail, fails);
    }
    __syncthreads();
    if (threadIdx.x < K) {
        atomicOr(&out[threadIdx.x], s_or[threadIdx.x]);
        atomicAnd(&out[K + threadIdx.x], s_and[threadIdx.x]);
    }
    if (threadIdx.x == 0) atomicAdd(&out[2 * K], s_fail);
}

// ------------------------------------------------------------------ 2. extract
template <int K, typename KeyT, bool GATHER>
__global__ void __launch_bounds__(256) extract_kernel(ConstKeyPtrs keys, uint64_t n, const __grid_constant__ Extract ex,
                                                      DCondSet cond, KeyT* __restrict__ sk, unsigned* __restrict__ idx) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned e = GATHER ? idx[i] : (unsigned)i;
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = keys.w[w][e];
        uint64_t v = 0;
        for (uint32_t r = 0; r < ex.nruns; ++r) {
            const Run ru = ex.runs[r];
            v |= ((kword<K>(k, ru.word) >> ru.shift) & wmask(ru.len)) << ru.dst;
        }
        if (ex.flag_bit != 0xffu && !cond_ok<K>(k, cond)) v |= 1ull << ex.flag_bit;
        sk[i] = (KeyT)v;
        if (!GATHER) idx[i] = (unsigned)i;
    }
}

__global__ void iota_kernel(unsigned* __restrict__ idx, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) idx[i] = (unsigned)i;
}

// ------------------------------------------------------------------ 4. segment heads
struct LbWs {
    unsigned long long* status;
    unsigned* counter;
    unsigned long long* total;
};
static LbWs make_lb(long long ntiles, int slot_offset_bytes = 0) {
    size_t bytes = 256 + (size_t)ntiles * 8;
    char* p = (char*)ws().get(WS_MISC, bytes);
    SQ_CUDA(cudaMemsetAsync(p, 0, bytes, stream()));
    LbWs w;
    w.counter = (unsigned*)p;
    w.total = (unsigned long long*)(p + 8);
    w.status = (unsigned long long*)(p + 256);
    (void)slot_offset_bytes;
    return w;
}

constexpr int kSelBlock = 256;
constexpr int kSelItems = 8;
constexpr int kSelTile = kSelBlock * kSelItems;

// Head of a group: first entry, or group key differs from the previous entry.
// KEYCMP: compare sorted 1-chunk keys; otherwise gather full masked keys.
template <int K, typename KeyT, bool KEYCMP>
__device__ __forceinline__ bool is_head(uint64_t i, const KeyT* sk, const unsigned* idx, ConstKeyPtrs keys,
                                        const uint64_t* gm) {
    if (i == 0) return true;
    if (KEYCMP) return sk[i] != sk[i - 1];
    const unsigned a = idx[i], b = idx[i - 1];
    bool diff = false;
#pragma unroll
    for (int w = 0; w < K; ++w) diff = diff || (((keys.w[w][a] ^ keys.w[w][b]) & gm[w]) != 0);
    return diff;
}

// Order-preserving select of head positions in [0, n) into seg[]; the count
// lands in *lb.total.
template <int K, typename KeyT, bool KEYCMP>
__global__ void __launch_bounds__(kSelBlock) heads_kernel(const KeyT* __restrict__ sk, const unsigned* __restrict__ idx,
                                                          ConstKeyPtrs keys, const uint64_t* __restrict__ gmask,
                                                          uint64_t n, unsigned* __restrict__ seg, LbWs lb,
                                                          long long ntiles, unsigned* err) {
    __shared__ unsigned s_tile;
    __shared__ unsigned s_cnt[kSelItems][kSelBlock / 32];
    __shared__ unsigned long long s_prefix;
    uint64_t gm[K];
#pragma unroll
    for (int w = 0; w < K; ++w) gm[w] = gmask[w];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(lb.counter, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const uint64_t base = (uint64_t)tile * kSelTile;
    unsigned ball[kSelItems];
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        const uint64_t i = base + (uint64_t)j * kSelBlock + tid;
        const bool h = i < n && is_head<K, KeyT, KEYCMP>(i, sk, idx, keys, gm);
        ball[j] = __ballot_sync(0xffffffffu, h);
        if (lane == 0) s_cnt[j][warp] = __popc(ball[j]);
    }
    __syncthreads();
    if (warp == 0) {
        constexpr int W = kSelBlock / 32;
        unsigned v0 = s_cnt[(2 * lane) / W][(2 * lane) % W];
        unsigned v1 = s_cnt[(2 * lane + 1) / W][(2 * lane + 1) % W];
        unsigned sum = v0 + v1, inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (unsigned)o) inc += t;
        }
        const unsigned excl = inc - sum;
        const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
        s_cnt[(2 * lane) / W][(2 * lane) % W] = excl;
        s_cnt[(2 * lane + 1) / W][(2 * lane + 1) % W] = excl + v0;
        unsigned long long pre = lb_warp_exclusive(lb.status, tile, total, err);
        if (lane == 0) {
            s_prefix = pre;
            if (tile == ntiles - 1) *lb.total = pre + total;
        }
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        if (!((ball[j] >> lane) & 1u)) continue;
        const uint64_t i = base + (uint64_t)j * kSelBlock + tid;
        seg[s_prefix + s_cnt[j][warp] + __popc(ball[j] & lt)] = (unsigned)i;
    }
}

// Exclusive scan of per-group counts (u32) into u64 offsets; total in *lb.total.
__global__ void __launch_bounds__(kSelBlock) scan_counts_kernel(const unsigned* __restrict__ cnt,
                                                                unsigned long long* __restrict__ off, uint64_t n,
                                                                LbWs lb, long long ntiles, unsigned* err) {
    __shared__ unsigned s_tile;
    __shared__ unsigned long long s_w[kSelBlock / 32];
    __shared__ unsigned long long s_prefix;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(lb.counter, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const uint64_t base = (uint64_t)tile * kSelTile + (uint64_t)tid * kSelItems;  // blocked: thread owns 8 consecutive
    unsigned long long v[kSelItems];
    unsigned long long sum = 0;
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        const uint64_t i = base + j;
        v[j] = i < n ? cnt[i] : 0ull;
        sum += v[j];
    }
    unsigned long long inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned long long wv = lane < kSelBlock / 32 ? s_w[lane] : 0ull;
        unsigned long long wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (unsigned)o) wi += t;
        }
        const unsigned long long total = __shfl_sync(0xffffffffu, wi, kSelBlock / 32 - 1);
        if (lane < kSelBlock / 32) s_w[lane] = wi - wv;
        unsigned long long pre = lb_warp_exclusive(lb.status, tile, total, err);
        if (lane == 0) {
            s_prefix = pre;
            if (tile == ntiles - 1) *lb.total = pre + total;
        }
    }
    __syncthreads();
    unsigned long long run = s_prefix + s_w[warp] + inc - sum;
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        const uint64_t i = base + j;
        if (i < n) off[i] = run;
        run += v[j];
    }
}

// ------------------------------------------------------------------ 5/6. emit
struct EmitArgs {
    ConstKeyPtrs in_keys;
    const double2* in_amp;
    KeyPtrs out_keys;
    double2* out_amp;
    const unsigned* idx;       // sort path: entry index of each member, grouped
    const unsigned* btgt;      // hash path: target value of each member, grouped
    const double2* bamp;       // hash path: amplitude of each member, grouped
    const unsigned* ghead;     // hash path: one member's entry index per group (its key)
    const unsigned* seg;       // group starts, seg[G] = end
    uint64_t groups;
    unsigned* cnt;             // count pass output
    const unsigned long long* off;  // write pass input
    unsigned long long* cursor;     // single-pass mode: output slots reserved so far
    Field target;
    Field aux;
    int mode;
    int nbits;                 // target width (1 for pair modes)
    double extra;              // 1/sqrt(2^n)
    double sqrt2inv;
    double eps;
    double sign2pi;            // CondRot: +-2*pi
    double2 m[4];
    const double2* mtable;     // CondRot_General_Bool: 4 matrix elements per input value
    const double2* umat;       // Rot_GeneralUnitary: S x S row-major
    int udag;                  // Rot_GeneralUnitary: apply the conjugate transpose
    Field varw;                // batched Hadamard: each group's digit count is this field of its key
    const unsigned long long* rstart;  // cached group ranges (access mode 2)
    const unsigned* rcnt;
    unsigned long long* ostart;  // single-pass mode: each group's output range, for the next split
    unsigned* ocnt;
    unsigned long long capacity;  // single-pass mode: output entries available; a group whose
                                  // reservation ends past it writes nothing (the host reruns exactly)
    int fix;                   // FWHT arithmetic: 0 the reference's FP64 butterflies, 1 exact sums
    unsigned long long* ticket;  // dynamic group order: next group, CTAs finished (zero between launches)
    unsigned* err;               // device error word
    unsigned* glist;             // groups left by a singleton fan-out, and their number (glist_n);
    unsigned* glist_n;           // emit_hadamard_kernel then runs over these groups only
};

// Dynamic group order for the persistent emit kernels. A grid of two CTAs
// per SM fills the register file; when another stream's blocks hold part of
// an SM (an overlapped download), a CTA may become resident only when they
// finish. With groups handed out by a counter such a CTA finds the work done
// instead of holding back the launch with a fixed share. Thread 0 fetches
// the next group while the CTA works on the current one (two shared slots,
// alternating per iteration, each rewritten only after a barrier that
// follows its last read); the last CTA to finish zeroes the counters.
__device__ __forceinline__ uint64_t ticket_first(unsigned long long* t, unsigned long long (&s_g)[2]) {
    if (threadIdx.x == 0) s_g[0] = atomicAdd(&t[0], 1ull);
    __syncthreads();
    return s_g[0];
}
__device__ __forceinline__ void ticket_prefetch(unsigned long long* t, unsigned long long (&s_g)[2], unsigned it) {
    if (threadIdx.x == 0) s_g[(it + 1) & 1] = atomicAdd(&t[0], 1ull);
}
__device__ __forceinline__ uint64_t ticket_next(unsigned long long (&s_g)[2], unsigned& it) {
    __syncthreads();
    ++it;
    return s_g[it & 1];
}
__device__ __forceinline__ void ticket_exit(unsigned long long* t) {
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&t[1], 1ull) == (unsigned long long)gridDim.x - 1ull) {
            atomicExch(&t[0], 0ull);
            atomicExch(&t[1], 0ull);
        }
    }
}

template <int K>
__device__ __forceinline__ void load_key(const ConstKeyPtrs& kp, unsigned e, uint64_t (&k)[K]) {
#pragma unroll
    for (int w = 0; w < K; ++w) k[w] = kp.w[w][e];
}
template <int K>
__device__ __forceinline__ void store_entry(const KeyPtrs& kp, double2* amp, unsigned long long o, const uint64_t (&k)[K],
                                            double2 a) {
#pragma unroll
    for (int w = 0; w < K; ++w) kp.w[w][o] = k[w];
    amp[o] = a;
}

// An output entry of a split or merge. Outputs past a.capacity are not
// written: in a consistent run that never happens (the single pass reserves
// within its capacity, the exact path's offsets sum to its total); a replayed
// graph fed other data than it recorded could compute offsets past the
// buffer, and is reported invalid by its count checks.
template <int K>
__device__ __forceinline__ void store_out(const EmitArgs& a, unsigned long long o, const uint64_t (&k)[K],
                                          double2 v) {
    if (o < a.capacity) store_entry<K>(a.out_keys, a.out_amp, o, k, v);
}
template <int K>
__device__ __forceinline__ void store_out_sign(const EmitArgs& a, unsigned long long o, const uint64_t (&k)[K],
                                               double2 v, bool negate) {
    if (o < a.capacity) store_entry_sign<K>(a.out_keys, a.out_amp, o, k, v, negate);
}

__device__ __forceinline__ double as_rational(uint64_t v, unsigned w) {
    if (w >= 64) return v * 1.0 / 2 / 9223372036854775808.0;
    return 1.0 * v / (double)(1ull << w);
}

// Member `pos` of the grouped order: its target value and amplitude. The
// sort path gathers them through the sorted index; the hash path reads the
// bucket arrays, which hold them contiguously per group.
// Member access: AM 0 = sort path (entry index per member), 1 = hash path
// (bucketed target + amplitude per member), 2 = cached group ranges (members
// are the entries start[g] .. start[g] + cnt[g] - 1 themselves).
template <int AM>
__device__ __forceinline__ void member_at(const EmitArgs& a, unsigned pos, uint64_t& t, double2& amp) {
    if (AM == 1) {
        t = a.btgt[pos];
        amp = a.bamp[pos];
    } else {
        const unsigned e = AM == 2 ? pos : a.idx[pos];
        t = (a.in_keys.w[a.target.word][e] >> a.target.shift) & wmask(a.target.width);
        amp = a.in_amp[e];
    }
}
template <int AM>
__device__ __forceinline__ unsigned group_head(const EmitArgs& a, uint64_t g, unsigned s0) {
    return AM == 1 ? a.ghead[g] : AM == 2 ? s0 : a.idx[s0];
}
template <int AM>
__device__ __forceinline__ void group_range(const EmitArgs& a, uint64_t g, unsigned& s0, unsigned& m) {
    if (AM == 2) {
        s0 = (unsigned)a.rstart[g];
        m = a.rcnt[g];
    } else {
        s0 = a.seg[g];
        m = a.seg[g + 1] - s0;
    }
}

// Pair modes (1-bit target): the two outputs of a pair (az: the member
// with target bit 0, ao: bit 1; either may be absent) and whether each
// survives the prune. k0 is a member's key (the other registers).
template <int K>
__device__ __forceinline__ void pair_math(const EmitArgs& a, const uint64_t (&k0)[K], double2 az, double2 ao,
                                          bool has_z, bool has_o, double2& rz, double2& ro, bool& kz, bool& ko) {
    {
        const double2 zero = make_double2(0.0, 0.0);
        if (a.mode == GM_HADAMARD_BOOL) {
            const double s = a.sqrt2inv;
            if (has_z && has_o) {
                rz = cadd(cscale(az, s), cscale(ao, s));
                ro = csub(cscale(az, s), cscale(ao, s));
            } else if (has_z) {
                rz = cscale(az, s);
                ro = cscale(az, s);
            } else {
                rz = cscale(ao, s);
                ro = cscale(ao, -s);
            }
        } else if (a.mode == GM_ROT) {
            double2 m0 = a.m[0], m1 = a.m[1], m2 = a.m[2], m3 = a.m[3];
            if (a.mtable) {  // CondRot_General_Bool: matrix chosen by the input register's value
                const double2* mt = a.mtable + 4 * fget<K>(k0, a.aux);
                m0 = mt[0];
                m1 = mt[1];
                m2 = mt[2];
                m3 = mt[3];
            }
            if (has_z && has_o) {
                rz = cadd(cmul2(az, m0), cmul2(ao, m1));
                ro = cadd(cmul2(az, m2), cmul2(ao, m3));
            } else if (has_z) {
                rz = cmul2(az, m0);
                ro = cmul2(az, m2);
            } else {
                rz = cmul2(ao, m1);
                ro = cmul2(ao, m3);
            }
        } else {  // GM_CONDROT: partner amplitude 0 for singletons, as the reference inserts it
            const double rot = as_rational(fget<K>(k0, a.aux), a.aux.width) * a.sign2pi;
            double sn, cs;
            sincos(rot, &sn, &cs);
            if (!has_z) az = zero;
            if (!has_o) ao = zero;
            rz = csub(cscale(az, cs), cscale(ao, sn));
            ro = cadd(cscale(az, sn), cscale(ao, cs));
        }
        kz = keep_amp(rz, a.eps);
        ko = keep_amp(ro, a.eps);
    }
}

// Pair modes: one thread per group of the grouping.
template <int K, bool BUCKET>
__device__ __forceinline__ void pair_outputs(const EmitArgs& a, uint64_t g, uint64_t (&k0)[K], double2& rz,
                                             double2& ro, bool& kz, bool& ko) {
    const unsigned s0 = a.seg[g], s1 = a.seg[g + 1];
    const unsigned m = s1 - s0;
    load_key<K>(a.in_keys, group_head<BUCKET>(a, g, s0), k0);
    uint64_t t0;
    double2 v0;
    member_at<BUCKET>(a, s0, t0, v0);
    const bool b0 = t0 & 1ull;
    double2 az = make_double2(0.0, 0.0), ao = make_double2(0.0, 0.0);
    bool has_z = false, has_o = false;
    if (b0) { ao = v0; has_o = true; } else { az = v0; has_z = true; }
    if (m >= 2) {
        uint64_t t1;
        double2 v1;
        member_at<BUCKET>(a, s0 + 1, t1, v1);
        if (b0) { az = v1; has_z = true; } else { ao = v1; has_o = true; }
    }
    pair_math<K>(a, k0, az, ao, has_z, has_o, rz, ro, kz, ko);
}

// One thread per group of at most two members (the target is one bit). In
// the single-pass mode (WRITE with a cursor) the lanes of a warp reserve
// their outputs with one atomic, in lane order.
template <int K, bool WRITE, bool BUCKET>
__global__ void __launch_bounds__(256) emit_pair_kernel(const __grid_constant__ EmitArgs a) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t gb = (uint64_t)blockIdx.x * blockDim.x; gb < a.groups; gb += stride) {  // warp-uniform trips
        const uint64_t g = gb + threadIdx.x;
        const bool valid = g < a.groups;
        bool kz = false, ko = false;
        double2 rz = make_double2(0.0, 0.0), ro = make_double2(0.0, 0.0);
        uint64_t k0[K];
        if (valid) pair_outputs<K, BUCKET>(a, g, k0, rz, ro, kz, ko);
        if (!WRITE) {
            if (valid) a.cnt[g] = (unsigned)kz + (unsigned)ko;
            continue;
        }
        unsigned long long o = 0;
        bool fits = true;
        if (a.cursor) {
            const unsigned c = (unsigned)kz + (unsigned)ko;
            unsigned inc = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned t = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= (unsigned)d) inc += t;
            }
            const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
            unsigned long long base = 0;
            if (lane == 31 && total) base = atomicAdd(a.cursor, (unsigned long long)total);
            base = __shfl_sync(0xffffffffu, base, 31);
            fits = base + total <= a.capacity;
            o = base + (inc - c);
        } else if (valid) {
            o = a.off[g];
        }
        if (!valid || !fits) continue;
        uint64_t kk[K];
#pragma unroll
        for (int w = 0; w < K; ++w) kk[w] = k0[w];
        if (kz) {
            fset<K>(kk, a.target, 0);
            store_out<K>(a, o++, kk, rz);
        }
        if (ko) {
            fset<K>(kk, a.target, 1);
            store_out<K>(a, o, kk, ro);
        }
    }
}



// add_systems merge: sum each run of equal keys in sorted (stable) order.
template <int K, bool WRITE>
__global__ void __launch_bounds__(256) emit_merge_kernel(const __grid_constant__ EmitArgs a) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.groups; g += stride) {
        const unsigned s0 = a.seg[g], s1 = a.seg[g + 1];
        const unsigned e0 = a.idx[s0];
        double2 acc = a.in_amp[e0];
        for (unsigned j = s0 + 1; j < s1; ++j) acc = cadd(acc, a.in_amp[a.idx[j]]);
        const bool keep = keep_amp(acc, a.eps);
        if (!WRITE) {
            a.cnt[g] = keep ? 1u : 0u;
        } else if (keep) {
            uint64_t k0[K];
            load_key<K>(a.in_keys, e0, k0);
            store_out<K>(a, a.off[g], k0, acc);
        }
    }
}

// Hadamard groups: one worker (a warp, or a whole block) per group, the 2^n
// slots of the group in shared memory.
template <int W>
__device__ __forceinline__ void worker_sync() {
    if (W == 32) __syncwarp();
    else __syncthreads();
}

// max of an int over a worker (a warp or the whole block); s_tmp holds 8 words
template <int W>
__device__ __forceinline__ int worker_max(int v, unsigned* s_tmp) {
    v = (int)__reduce_max_sync(0xffffffffu, (unsigned)v);
    if (W == 32) return v;
    __syncthreads();
    if ((threadIdx.x & 31u) == 0) s_tmp[threadIdx.x >> 5] = (unsigned)v;
    __syncthreads();
    unsigned r = s_tmp[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) r = max(r, s_tmp[i]);
    __syncthreads();
    return (int)r;
}

// Single-pass output: one thread of the worker reserves `total` output slots
// with an atomic on the cursor and publishes the range for the next split.
// `fits` is false when the range ends past the output capacity.
template <int W>
__device__ __forceinline__ unsigned long long reserve_out(const EmitArgs& a, uint64_t g, unsigned total, bool& fits,
                                                          unsigned long long* s_base) {
    const unsigned t = W == 32 ? (threadIdx.x & 31u) : threadIdx.x;
    unsigned long long base = 0;
    if (t == 0) {
        base = total ? atomicAdd(a.cursor, (unsigned long long)total) : 0ull;
        if (a.ocnt) {
            a.ostart[g] = base;
            a.ocnt[g] = total;
        }
    }
    if (W == 32) {
        base = __shfl_sync(0xffffffffu, base, 0);
    } else {
        if (t == 0) *s_base = base;
        __syncthreads();
        base = *s_base;
        __syncthreads();
    }
    fits = base + total <= a.capacity;
    return base;
}

// exclusive scan of a per-thread flag over a worker, in thread order; returns
// (exclusive prefix, total) for this round.
template <int W>
__device__ __forceinline__ unsigned worker_rank(bool f, unsigned* s_tmp, unsigned& total) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const unsigned in_warp = __popc(b & ((1u << lane) - 1u));
    if (W == 32) {
        total = __popc(b);
        return in_warp;
    }
    const unsigned warp = threadIdx.x >> 5;
    if (lane == 0) s_tmp[warp] = __popc(b);
    __syncthreads();
    unsigned pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < W / 32; ++w) {
        const unsigned c = s_tmp[w];
        if ((unsigned)w < warp) pre += c;
        tot += c;
    }
    __syncthreads();
    total = tot;
    return pre + in_warp;
}

// Single-pass integer Hadamard of up to 8 bits (or a batched width) whose
// groups are all singletons (a fresh grouping with as many groups as
// condition-passing entries). Each lane of a warp fetches one of 32
// consecutive groups (their chains of dependent reads run side by side), the
// warp reserves the 32 groups' outputs with one atomic on the output cursor
// (a reservation per group put up to a million same-address atomics in one
// launch), then fans the groups out one after another, 32 outputs per store
// instruction. Arithmetic and per-group output order are those of the
// singleton case of emit_hadamard_kernel; groups land in the output in lane
// order within a warp.
template <int K, int AM>
__global__ void __launch_bounds__(256) emit_fanout_kernel(const __grid_constant__ EmitArgs a) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t step = (uint64_t)gridDim.x * 256u;  // groups per grid-wide round (32 per warp)
    for (uint64_t gb = ((uint64_t)blockIdx.x * 8u + (threadIdx.x >> 5)) * 32u; gb < a.groups; gb += step) {
        const uint64_t g = gb + lane;
        const bool valid = g < a.groups;
        unsigned s0 = 0, m = 0;
        uint64_t v0 = 0;
        double2 a0 = make_double2(0.0, 0.0);
        uint64_t gk[K] = {};
        if (valid) {
            group_range<AM>(a, g, s0, m);
            if (m == 1u) {
                member_at<AM>(a, s0, v0, a0);
                load_key<K>(a.in_keys, group_head<AM>(a, g, s0), gk);
            }
        }
        // a group of several members (a few collisions among mostly singleton
        // groups) is listed for emit_hadamard_kernel; without a list it only
        // arises in a graph replayed on other data: nothing is written for it
        // and the replay is reported
        const bool one = valid && m == 1u;
        if (valid && !one) {
            if (a.glist) a.glist[atomicAdd(a.glist_n, 1u)] = (unsigned)g;  // several members: left for the next kernel
            else atomicOr(a.err, 32u);
        }
        const int nbits = a.varw.width ? (int)fget<K>(gk, a.varw) : a.nbits;
        const unsigned S = 1u << nbits;
        const double extra = a.varw.width ? inv_sqrt_pow2(nbits, a.sqrt2inv) : a.extra;
        // singleton: a * 2^{-n/2}, sign (-1)^{popcount(t & v)} (hadamard.cpp:27-42)
        const double2 base = cscale(a0, extra);
        // batched width 0: the entry is left as it is, never pruned
        const bool keep = one && ((a.varw.width && nbits == 0) || keep_amp(base, a.eps));
        const unsigned cnt = keep ? S : 0u;
        unsigned inc = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= (unsigned)d) inc += t;
        }
        const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
        unsigned long long wbase = 0;
        if (lane == 31 && total) wbase = atomicAdd(a.cursor, (unsigned long long)total);
        wbase = __shfl_sync(0xffffffffu, wbase, 31);
        const unsigned long long o = wbase + (inc - cnt);
        if (valid && a.ocnt) {
            a.ostart[g] = keep ? o : 0ull;
            a.ocnt[g] = cnt;
        }
        // past the output capacity (uniform over the warp): nothing is
        // written, the host sees the cursor beyond it and reruns exactly
        if (wbase + total > a.capacity) continue;
        for (unsigned j = 0; j < 32u; ++j) {
            const unsigned cj = __shfl_sync(0xffffffffu, cnt, j);
            if (!cj) continue;  // uniform: the group is empty or pruned
            const unsigned long long oj = __shfl_sync(0xffffffffu, o, j);
            const uint64_t vj = __shfl_sync(0xffffffffu, v0, j);
            const double2 bj = make_double2(__shfl_sync(0xffffffffu, base.x, j), __shfl_sync(0xffffffffu, base.y, j));
            const int nj = __shfl_sync(0xffffffffu, nbits, j);
            uint64_t kj[K];
#pragma unroll
            for (int w = 0; w < K; ++w) kj[w] = __shfl_sync(0xffffffffu, gk[w], j);
            Field tg = a.target;
            tg.width = (uint8_t)nj;
            for (unsigned c = lane; c < cj; c += 32u) {
                uint64_t kk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) kk[w] = kj[w];
                fset<K>(kk, tg, (uint64_t)c);
                store_out_sign<K>(a, oj + c, kk, bj, __popcll((uint64_t)c & vj) & 1);
            }
        }
    }
}

__device__ __forceinline__ double2 shfl_xor_d2(double2 v, int m) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// A warp per group (W = 32, targets up to 8 bits) or a CTA per group. The
// warp form is latency-bound (a chain of dependent loads and shared-memory
// stages per group), so it asks for 4 CTAs per SM at one key word and 3 at
// two (a few bytes of spills outside the stage loops), to keep more groups
// in flight.
template <int K, int W, bool WRITE, int AM>
__global__ void __launch_bounds__(256, W == 32 ? (K == 1 ? 4 : K == 2 ? 3 : 1) : 1) emit_hadamard_kernel(const __grid_constant__ EmitArgs a) {
    extern __shared__ double2 s_slots[];
    __shared__ unsigned s_tmp[8];
    __shared__ uint64_t s_member_t[8][64];
    __shared__ double2 s_member_a[8][64];
    __shared__ unsigned long long s_base;
    const unsigned Smax = 1u << a.nbits;
    const unsigned wid = W == 32 ? (threadIdx.x >> 5) : 0u;
    const unsigned t = W == 32 ? (threadIdx.x & 31u) : threadIdx.x;
    double2* slots = s_slots + (size_t)wid * Smax;
    const uint64_t workers_per_block = blockDim.x / W;
    const uint64_t stride = (uint64_t)gridDim.x * workers_per_block;
    // a group's range and key are a chain of dependent reads: the next
    // group's are issued while the current one is transformed
    // every group, or the groups a fan-out listed (their number written by
    // that kernel, earlier on the same stream)
    const uint64_t ng = a.glist ? (uint64_t)*a.glist_n : a.groups;
    uint64_t i = (uint64_t)blockIdx.x * workers_per_block + wid;
    unsigned s0_next = 0, m_next = 0;
    uint64_t gk_next[K] = {};
    if (i < ng) {
        const uint64_t gn = a.glist ? (uint64_t)a.glist[i] : i;
        group_range<AM>(a, gn, s0_next, m_next);
        if (m_next) load_key<K>(a.in_keys, group_head<AM>(a, gn, s0_next), gk_next);
    }
    for (; i < ng; i += stride) {
        const uint64_t g = a.glist ? (uint64_t)a.glist[i] : i;
        const unsigned s0 = s0_next, m = m_next;
        uint64_t gk[K];
#pragma unroll
        for (int w = 0; w < K; ++w) gk[w] = gk_next[w];
        if (i + stride < ng) {
            const uint64_t gn = a.glist ? (uint64_t)a.glist[i + stride] : i + stride;
            group_range<AM>(a, gn, s0_next, m_next);
            if (m_next) load_key<K>(a.in_keys, group_head<AM>(a, gn, s0_next), gk_next);
        }
        if (m == 0) {  // an emptied cached range
            if (!WRITE && t == 0) a.cnt[g] = 0u;
            continue;
        }
        // batched Hadamard: this group's digit count comes from its key
        const int nbits = a.varw.width ? (int)fget<K>(gk, a.varw) : a.nbits;
        const unsigned S = 1u << nbits;
        const double extra = a.varw.width ? inv_sqrt_pow2(nbits, a.sqrt2inv) : a.extra;
        Field tg = a.target;
        tg.width = (uint8_t)nbits;
        const bool sparse_full = a.mode == GM_HADAMARD_FULL && m <= (unsigned)(nbits - 1);
        if (a.mode == GM_HADAMARD_INT && m == 1) {
            // singleton: a * 2^{-n/2}, sign (-1)^{popcount(t & v)} (hadamard.cpp:27-42)
            uint64_t v0;
            double2 a0;
            member_at<AM>(a, s0, v0, a0);
            const double2 base = cscale(a0, extra);
            // batched width 0: the entry is left as it is, never pruned
            const bool keep = (a.varw.width && nbits == 0) || keep_amp(base, a.eps);
            bool fits = true;
            unsigned long long o = 0;
            if (WRITE) o = a.cursor ? reserve_out<W>(a, g, keep ? S : 0u, fits, &s_base) : a.off[g];
            if (!WRITE) {
                if (t == 0) a.cnt[g] = keep ? S : 0u;
            } else if (keep && fits) {
                for (unsigned c = t; c < S; c += W) {
                    uint64_t kk[K];
#pragma unroll
                    for (int w = 0; w < K; ++w) kk[w] = gk[w];
                    fset<K>(kk, tg, (uint64_t)c);
                    store_out_sign<K>(a, o + c, kk, base, __popcll((uint64_t)c & v0) & 1);
                }
            }
            worker_sync<W>();
            continue;
        }
        if (sparse_full) {
            // Hadamard_Int_Full sparse bucket (hadamard.cpp:267-304): direct
            // 2^n x m product, members summed in ascending target value.
            for (unsigned j = t; j < m; j += W) {
                uint64_t tj;
                double2 aj;
                member_at<AM>(a, s0 + j, tj, aj);
                s_member_t[wid][j] = tj;
                s_member_a[wid][j] = aj;
            }
            worker_sync<W>();
            if (t == 0) {  // order members by target value (m <= 63)
                for (unsigned i = 1; i < m; ++i) {
                    const uint64_t kt = s_member_t[wid][i];
                    const double2 ka = s_member_a[wid][i];
                    int j = (int)i - 1;
                    while (j >= 0 && s_member_t[wid][j] > kt) {
                        s_member_t[wid][j + 1] = s_member_t[wid][j];
                        s_member_a[wid][j + 1] = s_member_a[wid][j];
                        --j;
                    }
                    s_member_t[wid][j + 1] = kt;
                    s_member_a[wid][j + 1] = ka;
                }
            }
            worker_sync<W>();
            for (unsigned c = t; c < S; c += W) {
                double2 acc = make_double2(0.0, 0.0);
                for (unsigned j = 0; j < m; ++j) {
                    double2 term = cscale(s_member_a[wid][j], (__popcll((uint64_t)c & s_member_t[wid][j]) & 1) ? -1. : 1.);
                    term = cscale(term, extra);
                    acc = cadd(acc, term);
                }
                slots[c] = acc;
            }
            worker_sync<W>();
        } else {
            // zero-filled slots, scatter members, stage-ascending FWHT (hadamard.cpp:44-59, 100-131)
            int emax = 1;
            if (AM == 2 && m == S) {
                // a full cached range: member c has target c, read as amplitudes only
                for (unsigned c = t; c < S; c += W) {
                    const double2 ac = __ldcs(a.in_amp + s0 + c);
                    slots[c] = ac;
                    emax = max(emax, amp_exp(ac));
                }
            } else {
                for (unsigned c = t; c < S; c += W) slots[c] = make_double2(0.0, 0.0);
                worker_sync<W>();
                for (unsigned j = t; j < m; j += W) {
                    uint64_t tj;
                    double2 aj;
                    member_at<AM>(a, s0 + j, tj, aj);
                    slots[tj & (S - 1u)] = aj;  // cached ranges of a batched split: only the group's own n bits
                    emax = max(emax, amp_exp(aj));
                }
            }
            const bool fix = a.fix && a.mode != GM_UNITARY;
            if (fix) emax = worker_max<W>(emax, s_tmp);
            worker_sync<W>();
            if (fix) {
                // exact-sum arithmetic: integer grid, n exact stages, one rounding
                longlong2* ls = reinterpret_cast<longlong2*>(slots);
                const int F = 62 - nbits;
                for (unsigned c = t; c < S; c += W) ls[c] = to_fixed2(slots[c], emax, F);
                worker_sync<W>();
                for (int qn = 0; qn < nbits; ++qn) {
                    const unsigned h = 1u << qn;
                    for (unsigned p = t; p < S / 2; p += W) {
                        const unsigned i0 = ((p >> qn) << (qn + 1)) | (p & (h - 1u));
                        const unsigned i1 = i0 + h;
                        const longlong2 x0 = ls[i0], x1 = ls[i1];
                        ls[i0] = ladd(x0, x1);
                        ls[i1] = lsub(x0, x1);
                    }
                    worker_sync<W>();
                }
                const int e2 = fix_out_exp(emax, nbits);
                for (unsigned c = t; c < S; c += W) slots[c] = from_fixed2(ls[c], e2, nbits & 1, a.sqrt2inv);
                worker_sync<W>();
            }
            if (a.mode == GM_UNITARY) {
                // Rot_GeneralUnitary (rot.cpp:353-389): out[i] = sum_j M(i,j) * amp[j], j ascending
                double2 r[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned c = t + (unsigned)q * W;
                    double2 acc = make_double2(0.0, 0.0);
                    if (c < S)
                        for (unsigned j = 0; j < S; ++j) {
                            const double2 mij = a.udag ? make_double2(a.umat[(size_t)j * S + c].x, -a.umat[(size_t)j * S + c].y)
                                                       : a.umat[(size_t)c * S + j];
                            acc = cadd(acc, cmul2(mij, slots[j]));
                        }
                    r[q] = acc;
                }
                worker_sync<W>();
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned c = t + (unsigned)q * W;
                    if (c < S) slots[c] = r[q];
                }
                worker_sync<W>();
            }
            for (int qn = 0; a.mode != GM_UNITARY && !fix && qn < nbits; ++qn) {
                const unsigned h = 1u << qn;
                for (unsigned p = t; p < S / 2; p += W) {
                    const unsigned i0 = ((p >> qn) << (qn + 1)) | (p & (h - 1u));
                    const unsigned i1 = i0 + h;
                    const double2 x0 = slots[i0], x1 = slots[i1];
                    slots[i0] = cscale(cadd(x0, x1), a.sqrt2inv);
                    slots[i1] = cscale(csub(x0, x1), a.sqrt2inv);
                }
                worker_sync<W>();
            }
        }
        // count / write the kept slots in ascending target order
        unsigned long long o = 0;
        bool fits = true;
        if (W == 32 && WRITE && a.cursor) {
            // single pass, a warp per group (S <= 256): the rows' keep masks
            // stay in registers between the count and the write
            unsigned ball[8];
            unsigned total = 0;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const unsigned c = (unsigned)r * 32u + t;
                ball[r] = (unsigned)r * 32u < S ? __ballot_sync(0xffffffffu, c < S && keep_amp(slots[c], a.eps)) : 0u;
                total += __popc(ball[r]);
            }
            o = reserve_out<W>(a, g, total, fits, &s_base);
            unsigned kept = 0;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const unsigned c = (unsigned)r * 32u + t;
                if (fits && ((ball[r] >> t) & 1u)) {
                    uint64_t kk[K];
#pragma unroll
                    for (int w = 0; w < K; ++w) kk[w] = gk[w];
                    fset<K>(kk, tg, (uint64_t)c);
                    store_out<K>(a, o + kept + __popc(ball[r] & ((1u << t) - 1u)), kk, slots[c]);
                }
                kept += __popc(ball[r]);
            }
            worker_sync<W>();
            continue;
        }
        if (WRITE && a.cursor) {  // single pass: count, reserve, then write
            unsigned total = 0;
            for (unsigned r = 0; r < S; r += W) {
                const unsigned c = r + t;
                unsigned tot;
                worker_rank<W>(c < S && keep_amp(slots[c], a.eps), s_tmp, tot);
                total += tot;
            }
            o = reserve_out<W>(a, g, total, fits, &s_base);
        } else if (WRITE) {
            o = a.off[g];
        }
        unsigned kept = 0;
        for (unsigned r = 0; r < S; r += W) {
            const unsigned c = r + t;
            const bool keep = c < S && keep_amp(slots[c], a.eps);
            unsigned tot;
            const unsigned rank = worker_rank<W>(keep, s_tmp, tot);
            if (WRITE && keep && fits) {
                uint64_t kk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) kk[w] = gk[w];
                fset<K>(kk, tg, (uint64_t)c);
                store_out<K>(a, o + kept + rank, kk, slots[c]);
            }
            kept += tot;
        }
        if (!WRITE && t == 0) a.cnt[g] = kept;
        worker_sync<W>();
    }
}

// Hadamard_Int and Hadamard_Int_Full on targets of 1 to 4 bits, and
// Rot_GeneralUnitary on 1 to 3 bits: one thread per group, the group's 2^NB
// slots in registers. The
// arithmetic and its order are those of emit_hadamard_kernel, so the results
// are bit-identical; what changes is that millions of small groups no longer
// run one after another on a warp (a chain of dependent loads per group, with
// most lanes idle), and that in the single-pass mode the lanes of a warp
// reserve their outputs with one atomic, in lane order.
template <int K, int NB, bool WRITE, int AM, bool UNI>
__global__ void __launch_bounds__(256) emit_small_kernel(const __grid_constant__ EmitArgs a) {
    constexpr unsigned S = 1u << NB;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t gb = (uint64_t)blockIdx.x * blockDim.x; gb < a.groups; gb += stride) {  // warp-uniform trips
        const uint64_t g = gb + threadIdx.x;
        const bool valid = g < a.groups;
        double2 v[S];
        uint64_t gk[K];
        unsigned keepm = 0;  // bit c: output slot c survives the prune
        bool single = false;
        uint64_t v0 = 0;
        double2 base = make_double2(0.0, 0.0);
        unsigned s0 = 0, m = 0;
        if (valid) group_range<AM>(a, g, s0, m);
        if (m) {
            load_key<K>(a.in_keys, group_head<AM>(a, g, s0), gk);
            if (!UNI && a.mode == GM_HADAMARD_INT && m == 1) {
                // singleton: a * 2^{-n/2}, sign (-1)^{popcount(t & v)} (hadamard.cpp:27-42)
                double2 a0;
                member_at<AM>(a, s0, v0, a0);
                base = cscale(a0, a.extra);
                single = true;
                keepm = keep_amp(base, a.eps) ? (1u << S) - 1u : 0u;
            } else if (!UNI && a.mode == GM_HADAMARD_FULL && m <= (unsigned)(NB - 1)) {
                // Hadamard_Int_Full sparse bucket (hadamard.cpp:267-304): at most
                // NB - 1 members, summed in ascending target value
                constexpr int MM = NB > 1 ? NB - 1 : 1;
                uint64_t ts[MM];
                double2 as[MM];
#pragma unroll
                for (int j = 0; j < MM; ++j) {
                    ts[j] = ~0ull;  // absent members sort last
                    as[j] = make_double2(0.0, 0.0);
                    if ((unsigned)j < m) member_at<AM>(a, s0 + j, ts[j], as[j]);
                }
#pragma unroll
                for (int i = 0; i < MM - 1; ++i) {  // bubble passes over at most three registers
#pragma unroll
                    for (int j = 0; j < MM - 1 - i; ++j) {
                        if (ts[j + 1] < ts[j]) {
                            const uint64_t tt = ts[j];
                            ts[j] = ts[j + 1];
                            ts[j + 1] = tt;
                            const double2 ta = as[j];
                            as[j] = as[j + 1];
                            as[j + 1] = ta;
                        }
                    }
                }
#pragma unroll
                for (unsigned c = 0; c < S; ++c) {
                    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
                    for (int j = 0; j < MM; ++j) {
                        if ((unsigned)j < m) {
                            const double2 term = cscale(as[j], (__popcll((uint64_t)c & ts[j]) & 1) ? -1. : 1.);
                            acc = cadd(acc, cscale(term, a.extra));
                        }
                    }
                    v[c] = acc;
                }
            } else {
                // zero-filled slots, members scattered, then the FWHT or the unitary
#pragma unroll
                for (unsigned c = 0; c < S; ++c) v[c] = make_double2(0.0, 0.0);
                int emax = 1;
                unsigned filled = 0;  // bit c: slot c holds a member
#pragma unroll
                for (unsigned j = 0; j < S; ++j) {
                    if (j < m) {
                        uint64_t tj;
                        double2 aj;
                        member_at<AM>(a, s0 + j, tj, aj);
#pragma unroll
                        for (unsigned c = 0; c < S; ++c)
                            if (c == (unsigned)(tj & (S - 1u))) v[c] = aj;
                        filled |= 1u << (unsigned)(tj & (S - 1u));
                        emax = max(emax, amp_exp(aj));
                    }
                }
                if (UNI) {
                    // Rot_GeneralUnitary (rot.cpp:353-389): out[i] = sum_j M(i,j) * amp[j], j ascending.
                    // An empty slot's terms are +-0 and leave every nonzero sum as it is (an all-zero
                    // output is pruned), so column j is skipped when no lane of the warp holds slot j:
                    // FP64 is the limit of this kernel, and partly filled groups are common.
                    double2 r[S];
#pragma unroll
                    for (unsigned c = 0; c < S; ++c) r[c] = make_double2(0.0, 0.0);
#pragma unroll
                    for (unsigned j = 0; j < S; ++j) {
                        if (!__any_sync(__activemask(), (filled >> j) & 1u)) continue;
#pragma unroll
                        for (unsigned c = 0; c < S; ++c) {
                            const double2 mij = a.udag ? make_double2(a.umat[j * S + c].x, -a.umat[j * S + c].y)
                                                       : a.umat[c * S + j];
                            r[c] = cadd(r[c], cmul2(mij, v[j]));
                        }
                    }
#pragma unroll
                    for (unsigned c = 0; c < S; ++c) v[c] = r[c];
                } else if (a.fix) {
                    // exact-sum arithmetic: integer grid, NB exact stages, one rounding
                    longlong2 ls[S];
#pragma unroll
                    for (unsigned c = 0; c < S; ++c) ls[c] = to_fixed2(v[c], emax, 62 - NB);
#pragma unroll
                    for (int qn = 0; qn < NB; ++qn) {
                        const unsigned h = 1u << qn;
#pragma unroll
                        for (unsigned p = 0; p < S / 2; ++p) {
                            const unsigned i0 = ((p >> qn) << (qn + 1)) | (p & (h - 1u));
                            const unsigned i1 = i0 + h;
                            const longlong2 x0 = ls[i0], x1 = ls[i1];
                            ls[i0] = ladd(x0, x1);
                            ls[i1] = lsub(x0, x1);
                        }
                    }
                    const int e2 = fix_out_exp(emax, NB);
#pragma unroll
                    for (unsigned c = 0; c < S; ++c) v[c] = from_fixed2(ls[c], e2, NB & 1, a.sqrt2inv);
                } else {
                    // stage-ascending butterflies (hadamard.cpp:44-59, 100-131)
#pragma unroll
                    for (int qn = 0; qn < NB; ++qn) {
                        const unsigned h = 1u << qn;
#pragma unroll
                        for (unsigned p = 0; p < S / 2; ++p) {
                            const unsigned i0 = ((p >> qn) << (qn + 1)) | (p & (h - 1u));
                            const unsigned i1 = i0 + h;
                            const double2 x0 = v[i0], x1 = v[i1];
                            v[i0] = cscale(cadd(x0, x1), a.sqrt2inv);
                            v[i1] = cscale(csub(x0, x1), a.sqrt2inv);
                        }
                    }
                }
            }
            if (!single) {
#pragma unroll
                for (unsigned c = 0; c < S; ++c)
                    if (keep_amp(v[c], a.eps)) keepm |= 1u << c;
            }
        }
        const unsigned cnt = (unsigned)__popc(keepm);
        if (!WRITE) {
            if (valid) a.cnt[g] = cnt;
            continue;
        }
        unsigned long long o = 0;
        bool fits = true;
        if (a.cursor) {
            unsigned inc = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned t = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= (unsigned)d) inc += t;
            }
            const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
            unsigned long long wbase = 0;
            if (lane == 31 && total) wbase = atomicAdd(a.cursor, (unsigned long long)total);
            wbase = __shfl_sync(0xffffffffu, wbase, 31);
            fits = wbase + total <= a.capacity;
            o = wbase + (inc - cnt);
            if (valid && a.ocnt) {  // this group's output range, for the next split
                a.ostart[g] = o;
                a.ocnt[g] = cnt;
            }
        } else if (valid) {
            o = a.off[g];
        }
        if (!valid || !fits || !cnt) continue;
#pragma unroll
        for (unsigned c = 0; c < S; ++c) {
            if (!((keepm >> c) & 1u)) continue;
            uint64_t kk[K];
#pragma unroll
            for (int w = 0; w < K; ++w) kk[w] = gk[w];
            fset<K>(kk, a.target, (uint64_t)c);
            if (single) store_out_sign<K>(a, o, kk, base, __popcll((uint64_t)c & v0) & 1);
            else store_out<K>(a, o, kk, v[c]);
            ++o;
        }
    }
}

// Hadamard on 12 bits (4096 slots), one CTA of 256 threads per group. The
// stage-ascending FWHT runs mostly in registers: each thread holds 16 slots.
// Layout A: slot = j << 8 | warp << 5 | lane (j = 0..15); layout B:
// slot = warp << 9 | j << 5 | lane. Stages 0-4 are warp shuffles in layout A,
// stages 5-8 are in-register in layout B, stages 9-11 in-register in layout A;
// shared memory is used only to scatter the members and for two transposes.
// Every butterfly is (x0 + x1) * sqrt2inv, (x0 - x1) * sqrt2inv in the
// reference's stage order, so results are bit-identical to the smem version.
// MODE 0 counts kept outputs, 1 writes at offsets from the count pass, 2
// reserves each group's range with one atomic (single pass; the order of
// groups in the output is then not fixed, the values are).
enum { EMIT_COUNT = 0, EMIT_WRITE = 1, EMIT_ATOMIC = 2 };

// lower ? p : -v, chosen on the bit patterns
__device__ __forceinline__ double2 sel_neg(bool lower, double2 p, double2 v) {
    const unsigned long long sx = (unsigned long long)__double_as_longlong(v.x) ^ 0x8000000000000000ull;
    const unsigned long long sy = (unsigned long long)__double_as_longlong(v.y) ^ 0x8000000000000000ull;
    return make_double2(__longlong_as_double((long long)(lower ? (unsigned long long)__double_as_longlong(p.x) : sx)),
                        __longlong_as_double((long long)(lower ? (unsigned long long)__double_as_longlong(p.y) : sy)));
}


// The reference FP64 arithmetic (the exact-sum arithmetic runs in
// emit_h4096x_kernel below).
template <int K, int MODE, int AM>
__global__ void __launch_bounds__(256, 2) emit_h4096_kernel(const __grid_constant__ EmitArgs a) {
    extern __shared__ double2 sl[];  // 4096 slots
    __shared__ unsigned s_cnt[16][8];
    __shared__ unsigned long long s_base;
    __shared__ uint64_t s_mt[64];
    __shared__ double2 s_ma[64];
    __shared__ bool s_fits;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const Field tg = a.target;
    const double s2 = a.sqrt2inv;
    for (uint64_t g = blockIdx.x; g < a.groups; g += gridDim.x) {
        unsigned s0, m;
        group_range<AM>(a, g, s0, m);
        if (m == 0) {  // an emptied cached range
            if (tid == 0) {
                if (MODE == EMIT_COUNT) a.cnt[g] = 0u;
                else if (MODE == EMIT_ATOMIC && a.ocnt) {
                    a.ostart[g] = 0ull;
                    a.ocnt[g] = 0u;
                }
            }
            continue;
        }
        uint64_t gk[K];
        load_key<K>(a.in_keys, group_head<AM>(a, g, s0), gk);
        if (a.mode == GM_HADAMARD_INT && m == 1) {
            uint64_t v0;
            double2 a0;
            member_at<AM>(a, s0, v0, a0);
            const double2 base = cscale(a0, a.extra);
            const bool keep = keep_amp(base, a.eps);
            if (MODE == EMIT_COUNT) {
                if (tid == 0) a.cnt[g] = keep ? 4096u : 0u;
            } else if (MODE == EMIT_ATOMIC && !keep) {
                if (tid == 0 && a.ocnt) {
                    a.ostart[g] = 0ull;
                    a.ocnt[g] = 0u;
                }
            } else if (keep) {
                if (MODE == EMIT_ATOMIC) {
                    if (tid == 0) {
                        s_base = atomicAdd(a.cursor, 4096ull);
                        if (a.ocnt) {
                            a.ostart[g] = s_base;
                            a.ocnt[g] = 4096u;
                        }
                    }
                    __syncthreads();
                }
                const unsigned long long o = MODE == EMIT_WRITE ? a.off[g] : s_base;
                const bool fits = MODE != EMIT_ATOMIC || o + 4096ull <= a.capacity;
                for (unsigned c = tid; fits && c < 4096u; c += 256u) {
                    uint64_t kk[K];
#pragma unroll
                    for (int w = 0; w < K; ++w) kk[w] = gk[w];
                    fset<K>(kk, tg, (uint64_t)c);
                    store_out_sign<K>(a, o + c, kk, base, __popcll((uint64_t)c & v0) & 1);
                }
            }
            __syncthreads();
            continue;
        }
        double2 v[16];
        unsigned rows = 0xffffu;  // rows j that may hold a kept slot (warp-uniform)
        if (a.mode == GM_HADAMARD_FULL && m <= 11u) {
            // sparse bucket: direct product, members in ascending target order (hadamard.cpp:267-304)
            for (unsigned j = tid; j < m; j += 256u) {
                uint64_t tj;
                double2 aj;
                member_at<AM>(a, s0 + j, tj, aj);
                s_mt[j] = tj;
                s_ma[j] = aj;
            }
            __syncthreads();
            if (tid == 0) {
                for (unsigned i = 1; i < m; ++i) {
                    const uint64_t kt = s_mt[i];
                    const double2 ka = s_ma[i];
                    int j = (int)i - 1;
                    while (j >= 0 && s_mt[j] > kt) {
                        s_mt[j + 1] = s_mt[j];
                        s_ma[j + 1] = s_ma[j];
                        --j;
                    }
                    s_mt[j + 1] = kt;
                    s_ma[j + 1] = ka;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const unsigned c = ((unsigned)j << 8) | tid;
                double2 acc = make_double2(0.0, 0.0);
                for (unsigned q = 0; q < m; ++q) {
                    double2 term = cscale(s_ma[q], (__popcll((uint64_t)c & s_mt[q]) & 1) ? -1. : 1.);
                    term = cscale(term, a.extra);
                    acc = cadd(acc, term);
                }
                v[j] = acc;
            }
        } else {
            // A full cached range holds its members in ascending target order
            // (every emit writes a group's outputs in slot order), so member c
            // has target c: the 16 slots of a thread load straight into
            // registers, 16 coalesced loads in flight, no scatter.
            const bool direct = AM == 2 && m == 4096u;
            if (direct) {
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __ldcs(a.in_amp + s0 + (((unsigned)j << 8) | tid));
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) sl[((unsigned)j << 8) | tid] = make_double2(0.0, 0.0);
                __syncthreads();
            }
            // members: 8 independent loads in flight per thread, then scatter
            for (unsigned j0 = 0; !direct && j0 < m; j0 += 8u * 256u) {
                uint64_t tq[8];
                double2 aq[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned j = j0 + (unsigned)q * 256u + tid;
                    if (j < m) member_at<AM>(a, s0 + j, tq[q], aq[q]);
                }
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned j = j0 + (unsigned)q * 256u + tid;
                    if (j < m) sl[tq[q]] = aq[q];
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; !direct && j < 16; ++j) v[j] = sl[((unsigned)j << 8) | tid];
            // stages 0..4: partner lane = lane ^ h
#pragma unroll
            for (int qn = 0; qn < 5; ++qn) {
                const int h = 1 << qn;
                const bool lower = !(lane & (unsigned)h);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const double2 p = shfl_xor_d2(v[j], h);
                    // lower: (v + p) * s2; upper: (p - v) * s2 = (p + (-v)) * s2, the
                    // same rounding; operands picked as bits so that one add is issued
                    v[j] = cscale(cadd(lower ? v[j] : p, sel_neg(lower, p, v[j])), s2);
                }
            }
            // transpose A -> B
#pragma unroll
            for (int j = 0; j < 16; ++j) sl[((unsigned)j << 8) | tid] = v[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = sl[(warp << 9) | ((unsigned)j << 5) | lane];
            // stages 5..8: slot bit qn = bit (qn - 5) of j
#pragma unroll
            for (int b = 0; b < 4; ++b) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (j & (1 << b)) continue;
                    const double2 x0 = v[j], x1 = v[j | (1 << b)];
                    v[j] = cscale(cadd(x0, x1), s2);
                    v[j | (1 << b)] = cscale(csub(x0, x1), s2);
                }
            }
            // transpose B -> A (each thread rewrites the slots it read)
#pragma unroll
            for (int j = 0; j < 16; ++j) sl[(warp << 9) | ((unsigned)j << 5) | lane] = v[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = sl[((unsigned)j << 8) | tid];
            // stages 9..11: slot bit qn = bit (qn - 8) of j
#pragma unroll
            for (int b = 1; b < 4; ++b) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (j & (1 << b)) continue;
                    const double2 x0 = v[j], x1 = v[j | (1 << b)];
                    v[j] = cscale(cadd(x0, x1), s2);
                    v[j | (1 << b)] = cscale(csub(x0, x1), s2);
                }
            }
        }
        // kept slots in ascending slot order: row j (slot bits 8..11), then warp, then lane
        unsigned ball[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            ball[j] = ((rows >> j) & 1u) ? __ballot_sync(0xffffffffu, keep_amp(v[j], a.eps)) : 0u;
            if (lane == 0) s_cnt[j][warp] = __popc(ball[j]);
        }
        __syncthreads();
        if (warp == 0) {
            unsigned c4[4], sum = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned idx = lane * 4 + q;
                c4[q] = s_cnt[idx >> 3][idx & 7];
                sum += c4[q];
            }
            unsigned inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= (unsigned)o) inc += t;
            }
            unsigned run = inc - sum;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned idx = lane * 4 + q;
                s_cnt[idx >> 3][idx & 7] = run;
                run += c4[q];
            }
            const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
            if (lane == 0) {
                if (MODE == EMIT_COUNT) a.cnt[g] = total;
                else if (MODE == EMIT_ATOMIC) {
                    s_base = total ? atomicAdd(a.cursor, (unsigned long long)total) : 0ull;
                    s_fits = s_base + total <= a.capacity;
                    if (a.ocnt) {
                        a.ostart[g] = s_base;
                        a.ocnt[g] = total;
                    }
                }
            }
        }
        __syncthreads();
        if (MODE != EMIT_COUNT) {
            const unsigned long long o = MODE == EMIT_WRITE ? a.off[g] : s_base;
            const unsigned lt = (1u << lane) - 1u;
            // past the output capacity (uniform over the CTA): nothing is written, the host reruns exactly
            const bool fits = MODE != EMIT_ATOMIC || s_fits;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                if (!fits || !((ball[j] >> lane) & 1u)) continue;
                uint64_t kk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) kk[w] = gk[w];
                fset<K>(kk, tg, (uint64_t)(((unsigned)j << 8) | tid));
                store_out<K>(a, o + s_cnt[j][warp] + __popc(ball[j] & lt), kk, v[j]);
            }
        }
        __syncthreads();
    }
}

// The 12-bit Hadamard in the exact-sum arithmetic, one CTA of 512 threads
// per group, two CTAs per SM (32 warps). A thread holds 8 slots; the integer
// stages run in registers in four phases, each with 3 slot bits in the
// thread's index j: layout A (slot = j << 9 | tid: bits 9-11), P0 (tid << 3 | j:
// bits 0-2), P1 (tid_hi << 6 | j << 3 | tid_lo: bits 3-5), P2 (tid_hi << 9 |
// j << 6 | tid_lo: bits 6-8), then back to A for coalesced output. Integer sums
// are exact, so the stage order does not change the result. Slots are stored
// at s ^ ((s >> 3) & 7) (16-byte units): conflict-free in all four layouts.
__device__ __forceinline__ void fwht8(longlong2 (&x)[8]) {
#pragma unroll
    for (int b = 0; b < 3; ++b) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j & (1 << b)) continue;
            const longlong2 x0 = x[j], x1 = x[j | (1 << b)];
            x[j] = ladd(x0, x1);
            x[j | (1 << b)] = lsub(x0, x1);
        }
    }
}
__device__ __forceinline__ unsigned swz8(unsigned q) { return q ^ ((q >> 3) & 7u); }

// SHAPE narrows the kernel to the groups the host knows it has, so that only
// that path is compiled in and the other paths' registers do not count
// against it: H_FULL, every group a cached range of 4096 members (the state
// holds exactly 4096 entries per range); H_SINGLE, every group one entry of
// an integer Hadamard (as many groups as entries); H_ANY, any groups.
enum { H_ANY = 0, H_FULL = 1, H_SINGLE = 2 };
template <int K, int MODE, int AM, int SHAPE>
__global__ void __launch_bounds__(512, 2) emit_h4096x_kernel(const __grid_constant__ EmitArgs a) {
    constexpr bool FULL = SHAPE == H_FULL;
    extern __shared__ double2 sl[];  // 4096 slots
    __shared__ unsigned s_cnt[8][16];
    __shared__ unsigned long long s_base;
    __shared__ uint64_t s_mt[64];
    __shared__ double2 s_ma[64];
    __shared__ unsigned s_emax[16];
    __shared__ bool s_fits;
    __shared__ unsigned long long s_g[2];
    __shared__ unsigned s_ball[8][16];  // keep masks per (row, warp): not held in registers
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const Field tg = a.target;
    longlong2* ls = reinterpret_cast<longlong2*>(sl);
    unsigned it = 0;
    for (uint64_t g = ticket_first(a.ticket, s_g); g < a.groups; g = ticket_next(s_g, it)) {
        ticket_prefetch(a.ticket, s_g, it);
        unsigned s0, m;
        group_range<AM>(a, g, s0, m);
        if ((FULL && m != 4096u) || (SHAPE == H_SINGLE && m != 1u)) {
            // cannot happen for the sizes the host checked; a replayed graph
            // whose groups differ from the recorded ones is reported instead
            if (tid == 0) atomicOr(a.err, 32u);
            continue;
        }
        if (!FULL && m == 0) {  // an emptied cached range
            if (tid == 0) {
                if (MODE == EMIT_COUNT) a.cnt[g] = 0u;
                else if (MODE == EMIT_ATOMIC && a.ocnt) {
                    a.ostart[g] = 0ull;
                    a.ocnt[g] = 0u;
                }
            }
            continue;
        }
        if (SHAPE == H_SINGLE || (!FULL && a.mode == GM_HADAMARD_INT && m == 1)) {
            uint64_t gk[K];
            load_key<K>(a.in_keys, group_head<AM>(a, g, s0), gk);
            // singleton: a * 2^-6, sign (-1)^popcount(t & v) (hadamard.cpp:27-42)
            uint64_t v0;
            double2 a0;
            member_at<AM>(a, s0, v0, a0);
            const double2 base = cscale(a0, a.extra);
            const bool keep = keep_amp(base, a.eps);
            if (MODE == EMIT_COUNT) {
                if (tid == 0) a.cnt[g] = keep ? 4096u : 0u;
            } else if (MODE == EMIT_ATOMIC && !keep) {
                if (tid == 0 && a.ocnt) {
                    a.ostart[g] = 0ull;
                    a.ocnt[g] = 0u;
                }
            } else if (keep) {
                if (MODE == EMIT_ATOMIC) {
                    if (tid == 0) {
                        s_base = atomicAdd(a.cursor, 4096ull);
                        if (a.ocnt) {
                            a.ostart[g] = s_base;
                            a.ocnt[g] = 4096u;
                        }
                    }
                    __syncthreads();
                }
                const unsigned long long o = MODE == EMIT_WRITE ? a.off[g] : s_base;
                const bool fits = MODE != EMIT_ATOMIC || o + 4096ull <= a.capacity;
                for (unsigned c = tid; fits && c < 4096u; c += 512u) {
                    uint64_t kk[K];
#pragma unroll
                    for (int w = 0; w < K; ++w) kk[w] = gk[w];
                    fset<K>(kk, tg, (uint64_t)c);
                    store_out_sign<K>(a, o + c, kk, base, __popcll((uint64_t)c & v0) & 1);
                }
            }
            __syncthreads();
            continue;
        }
        if (SHAPE == H_SINGLE) continue;  // not reached: every group took the path above
        double2 v[8];
        unsigned rows = 0xffu;  // rows j that may hold a kept slot (warp-uniform)
        // the slot of v[j]: layout A (j << 9 | tid) after the sparse-bucket
        // product, layout P2 (tid_hi << 9 | j << 6 | tid_lo) after the FWHT;
        // either way a warp's 32 lanes hold 32 consecutive slots of row j
        bool p2 = FULL;
#define SQ_B2 (((tid >> 6) << 9) | (tid & 63u))
        if (!FULL && a.mode == GM_HADAMARD_FULL && m <= 11u) {
            // sparse bucket: direct product, members in ascending target order (hadamard.cpp:267-304)
            for (unsigned j = tid; j < m; j += 512u) {
                uint64_t tj;
                double2 aj;
                member_at<AM>(a, s0 + j, tj, aj);
                s_mt[j] = tj;
                s_ma[j] = aj;
            }
            __syncthreads();
            if (tid == 0) {
                for (unsigned i = 1; i < m; ++i) {
                    const uint64_t kt = s_mt[i];
                    const double2 ka = s_ma[i];
                    int j = (int)i - 1;
                    while (j >= 0 && s_mt[j] > kt) {
                        s_mt[j + 1] = s_mt[j];
                        s_ma[j + 1] = s_ma[j];
                        --j;
                    }
                    s_mt[j + 1] = kt;
                    s_ma[j + 1] = ka;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const unsigned c = ((unsigned)j << 9) | tid;
                double2 acc = make_double2(0.0, 0.0);
                for (unsigned q = 0; q < m; ++q) {
                    double2 term = cscale(s_ma[q], (__popcll((uint64_t)c & s_mt[q]) & 1) ? -1. : 1.);
                    term = cscale(term, a.extra);
                    acc = cadd(acc, term);
                }
                v[j] = acc;
            }
        } else {
            const bool direct = FULL || (AM == 2 && m == 4096u);  // a full cached range: member c has target c
            int emax = 1;
            if (direct) {
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] = __ldcs(a.in_amp + s0 + (((unsigned)j << 9) | tid));
#pragma unroll
                for (int j = 0; j < 8; ++j) emax = max(emax, amp_exp(v[j]));
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) sl[((unsigned)j << 9) | tid] = make_double2(0.0, 0.0);
                __syncthreads();
                for (unsigned j0 = 0; j0 < m; j0 += 8u * 512u) {
                    uint64_t tq[8];
                    double2 aq[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const unsigned j = j0 + (unsigned)q * 512u + tid;
                        if (j < m) member_at<AM>(a, s0 + j, tq[q], aq[q]);
                    }
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const unsigned j = j0 + (unsigned)q * 512u + tid;
                        if (j < m) {
                            sl[tq[q]] = aq[q];
                            emax = max(emax, amp_exp(aq[q]));
                        }
                    }
                }
            }
            emax = (int)__reduce_max_sync(0xffffffffu, (unsigned)emax);
            if (lane == 0) s_emax[warp] = (unsigned)emax;
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 16; ++i) emax = max(emax, (int)s_emax[i]);
            longlong2 x[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const double2 d = direct ? v[j] : sl[((unsigned)j << 9) | tid];
                x[j] = make_longlong2(to_fixed_right(d.x, emax, 50), to_fixed_right(d.y, emax, 50));
            }
            fwht8(x);  // layout A: slot bits 9-11
            // every thread has read its slots as doubles before they are overwritten; a
            // direct range was read from global memory, and the barrier after the
            // exponent exchange already orders this group's writes after every
            // use of the slots by the previous group
            if (!direct) __syncthreads();
#pragma unroll
            for (int j = 0; j < 8; ++j) ls[swz8(((unsigned)j << 9) | tid)] = x[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = ls[swz8((tid << 3) | (unsigned)j)];
            fwht8(x);  // P0: bits 0-2
#pragma unroll
            for (int j = 0; j < 8; ++j) ls[swz8((tid << 3) | (unsigned)j)] = x[j];
            __syncthreads();
            const unsigned b1 = ((tid >> 3) << 6) | (tid & 7u);
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = ls[swz8(b1 | ((unsigned)j << 3))];
            fwht8(x);  // P1: bits 3-5
#pragma unroll
            for (int j = 0; j < 8; ++j) ls[swz8(b1 | ((unsigned)j << 3))] = x[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = ls[swz8(SQ_B2 | ((unsigned)j << 6))];
            fwht8(x);  // P2: bits 6-8; the outputs are taken from this layout
            p2 = true;
            const int e2 = fix_out_exp(emax, 12);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                // merges leave most slots exactly zero: skip the conversion and the prune test row by row
                const bool nz = (x[j].x | x[j].y) != 0;
                if (__any_sync(0xffffffffu, nz)) {
                    v[j] = from_fixed2(x[j], e2, false, a.sqrt2inv);
                } else {
                    v[j] = make_double2(0.0, 0.0);
                    rows &= ~(1u << j);
                }
            }
        }
        // kept slots in ascending slot order: the 128 runs of 32 consecutive
        // slots (run = slot >> 5), counted and ranked in run order
        unsigned* const s_cnt_run = &s_cnt[0][0];
        unsigned* const s_ball_run = &s_ball[0][0];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned ball = ((rows >> j) & 1u) ? __ballot_sync(0xffffffffu, keep_amp(v[j], a.eps)) : 0u;
            if (lane == 0) {
                const unsigned run = (p2 ? (SQ_B2 | ((unsigned)j << 6)) : (((unsigned)j << 9) | tid)) >> 5;
                s_cnt_run[run] = __popc(ball);
                s_ball_run[run] = ball;
            }
        }
        __syncthreads();
        if (warp == 0) {
            unsigned c4[4], sum = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned idx = lane * 4 + q;  // (row, warp) in row-major order
                c4[q] = s_cnt[idx >> 4][idx & 15];
                sum += c4[q];
            }
            unsigned inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= (unsigned)o) inc += t;
            }
            unsigned run = inc - sum;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned idx = lane * 4 + q;
                s_cnt[idx >> 4][idx & 15] = run;
                run += c4[q];
            }
            const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
            if (lane == 0) {
                if (MODE == EMIT_COUNT) a.cnt[g] = total;
                else if (MODE == EMIT_ATOMIC) {
                    s_base = total ? atomicAdd(a.cursor, (unsigned long long)total) : 0ull;
                    s_fits = s_base + total <= a.capacity;
                    if (a.ocnt) {
                        a.ostart[g] = s_base;
                        a.ocnt[g] = total;
                    }
                }
            }
        }
        __syncthreads();
        if (MODE != EMIT_COUNT && (MODE != EMIT_ATOMIC || s_fits)) {
            const unsigned long long o = MODE == EMIT_WRITE ? a.off[g] : s_base;
            const unsigned lt = (1u << lane) - 1u;
            uint64_t gk[K];  // the group's key, read here rather than held through the transform
            load_key<K>(a.in_keys, group_head<AM>(a, g, s0), gk);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const unsigned slot = p2 ? (SQ_B2 | ((unsigned)j << 6)) : (((unsigned)j << 9) | tid);
                const unsigned ball = s_ball_run[slot >> 5];
                if (!((ball >> lane) & 1u)) continue;
                uint64_t kk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) kk[w] = gk[w];
                fset<K>(kk, tg, (uint64_t)slot);
                store_out<K>(a, o + s_cnt_run[slot >> 5] + __popc(ball & lt), kk, v[j]);
            }
        }
        __syncthreads();
#undef SQ_B2
    }
    ticket_exit(a.ticket);
}

// Entries that fail the control conditions: copied through unchanged.
template <int K>
__global__ void passthrough_kernel(ConstKeyPtrs ik, const double2* __restrict__ ia, const unsigned* __restrict__ idx,
                                   uint64_t count, KeyPtrs ok, double2* __restrict__ oa, uint64_t out_base) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += stride) {
        const unsigned e = idx[j];
        uint64_t k[K];
        load_key<K>(ik, e, k);
        store_entry<K>(ok, oa, out_base + j, k, ia[e]);
    }
}

// ------------------------------------------------------------------ hash grouping
// Group by an open-addressing hash table keyed on the masked group key. A slot
// holds 0 (empty), kSlotLocked (being claimed) or ((gid + 1) << 32 | head + 1)
// where `head` is the first entry that claimed it; keys are compared against
// the head entry's key words. Group ids are dense, in claim order. Every wait
// on a locked slot is bounded.
constexpr unsigned long long kSlotLocked = ~0ull;

// atomicAdd(ctr, 1) for each calling lane, one atomic per group of lanes that
// execute the call together (new group ids: every lane of a warp of
// singleton groups would otherwise hit the same counter)
__device__ __forceinline__ unsigned warp_aggregated_add(unsigned* ctr) {
    const unsigned am = __activemask();
    const unsigned lane = threadIdx.x & 31u;
    const int leader = __ffs(am) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(ctr, (unsigned)__popc(am));
    base = __shfl_sync(am, base, leader);
    return base + (unsigned)__popc(am & ((1u << lane) - 1u));
}

struct HashWs {
    unsigned long long* slots;
    unsigned long long cap_mask;
    unsigned* gcount;     // [0]: groups, [1]: entries failing the conditions, [2]: table overflow
    unsigned* cnt;        // members per group
    unsigned* head;       // one entry per group
    unsigned* gid;        // group of each entry (~0u: fails the conditions)
    unsigned* pass_list;  // entries failing the conditions
};

// The overflow flag is read coherently (another SM sets it while this lane
// may be waiting on a slot that the setter locked and will never fill).
__device__ __forceinline__ bool overflowed(const HashWs& h) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> f(h.gcount[2]);
    return f.load(cuda::memory_order_relaxed) != 0u;
}


__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

template <int K>
__global__ void __launch_bounds__(256) hash_insert_kernel(ConstKeyPtrs keys, const uint64_t* __restrict__ gmask,
                                                          DCondSet cond, uint64_t n, HashWs h, unsigned gmax,
                                                          Field tgt, Field varw, unsigned max_digits, unsigned* err) {
    __shared__ unsigned s_fail[32];
    __shared__ unsigned s_fail_base;
    uint64_t gm[K];
#pragma unroll
    for (int w = 0; w < K; ++w) gm[w] = gmask[w];
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x; b < n; b += stride) {  // block-uniform trip count
        const uint64_t i = b + threadIdx.x;
        const bool valid = i < n;
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = valid ? (keys.w[w][i] & gm[w]) : 0ull;
        bool pass = false;
        if (valid) {
            uint64_t full[K];
#pragma unroll
            for (int w = 0; w < K; ++w) full[w] = keys.w[w][i];
            pass = cond_ok<K>(full, cond);
            if (pass && varw.width) {  // batched Hadamard: drop this entry's own n low target bits
                const unsigned nd = (unsigned)fget<K>(full, varw);
                if (nd > max_digits) {
                    atomicOr(err, 4u);
                    pass = false;
                } else {
                    kword_set<K>(k, tgt.word, kword<K>(k, tgt.word) & ~(wmask(nd) << tgt.shift));
                }
            }
            if (!pass) h.gid[i] = ~0u;
        }
        {   // entries failing the conditions: one atomic per block and round
            const bool fail = valid && !pass;
            const unsigned fb = __ballot_sync(0xffffffffu, fail);
            const unsigned warp = threadIdx.x >> 5;
            if (lane == 0) s_fail[warp] = (unsigned)__popc(fb);
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned run = 0;
                for (unsigned w = 0; w < (blockDim.x >> 5); ++w) {
                    const unsigned c = s_fail[w];
                    s_fail[w] = run;
                    run += c;
                }
                s_fail_base = run ? atomicAdd(&h.gcount[1], run) : 0u;
            }
            __syncthreads();
            if (fail) h.pass_list[s_fail_base + s_fail[warp] + __popc(fb & ((1u << lane) - 1u))] = (unsigned)i;
            __syncthreads();
        }
        unsigned long long hv = 0x9e3779b97f4a7c15ull;
#pragma unroll
        for (int w = 0; w < K; ++w) hv = mix64(hv ^ k[w] ^ (0x632be59bd9b4e019ull * (w + 1)));
        // lanes whose group key hashes equal share one table probe (entries of
        // a group usually arrive together); a lane whose key differs from its
        // leader's despite the equal hash probes on its own
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        const unsigned peers = __match_any_sync(0xffffffffu, hv) & pm;
        const int leader = pass ? __ffs(peers) - 1 : (int)lane;
        bool same = true;
#pragma unroll
        for (int w = 0; w < K; ++w) same = same && (__shfl_sync(0xffffffffu, k[w], leader) == k[w]);
        const unsigned same_mask = __ballot_sync(0xffffffffu, pass && same);
        const bool probe = pass && (!same || (int)lane == leader);
        unsigned mygid = ~0u;
        if (probe) {
            unsigned long long slot = hv & h.cap_mask;
            unsigned spins = 0;
            for (unsigned long long probes = 0; probes <= h.cap_mask;) {
                if (overflowed(h)) break;  // table overflowed: the host retries with a larger one
                cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> ref(h.slots[slot]);
                unsigned long long v = ref.load(cuda::memory_order_relaxed);
                if (v == 0ull) {
                    unsigned long long expected = 0ull;
                    if (ref.compare_exchange_strong(expected, kSlotLocked, cuda::memory_order_relaxed)) {
                        const unsigned g = warp_aggregated_add(&h.gcount[0]);
                        if (g >= gmax) {
                            atomicExch(&h.gcount[2], 1u);
                            break;
                        }
                        h.head[g] = (unsigned)i;
                        ref.store(((unsigned long long)(g + 1) << 32) | (unsigned long long)(i + 1),
                                  cuda::memory_order_relaxed);
                        mygid = g;
                        break;
                    }
                    continue;  // lost the race: re-read this slot
                }
                if (v == kSlotLocked) {
                    if (++spins > spin_limit(err)) {
                        atomicOr(err, 2u);
                        break;
                    }
                    __nanosleep(20);
                    continue;
                }
                const unsigned hidx = (unsigned)(v & 0xffffffffull) - 1u;
                uint64_t hk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) hk[w] = keys.w[w][hidx] & gm[w];
                if (varw.width) {
                    const unsigned hn = (unsigned)fget<K>(hk, varw);
                    kword_set<K>(hk, tgt.word, kword<K>(hk, tgt.word) & ~(wmask(hn) << tgt.shift));
                }
                bool eq = true;
#pragma unroll
                for (int w = 0; w < K; ++w) eq = eq && ((hk[w] ^ k[w]) == 0);
                if (eq) {
                    mygid = (unsigned)(v >> 32) - 1u;
                    break;
                }
                slot = (slot + 1) & h.cap_mask;
                ++probes;
            }
            if (mygid != ~0u) {
                const unsigned c = (int)lane == leader ? __popc(peers & same_mask) : 1u;
                atomicAdd(&h.cnt[mygid], c);
            }
        }
        const unsigned lg = __shfl_sync(0xffffffffu, mygid, leader);
        if (pass) {
            if (!probe) mygid = lg;
            h.gid[i] = mygid;
            if (mygid == ~0u && !overflowed(h)) atomicOr(err, 2u);  // probe gave up: reported
        }
    }
}

// Sketch of the group keys for the size model: 32 registers, each the largest
// leading-zero rank (+1) of the hashed keys falling in its bucket (the
// HyperLogLog register update), over `samples` entries taken at a stride.
template <int K>
__global__ void __launch_bounds__(256) sketch_kernel(ConstKeyPtrs keys, const uint64_t* __restrict__ gmask,
                                                     uint64_t stride, unsigned samples, unsigned* __restrict__ regs) {
    __shared__ unsigned sr[32];
    if (threadIdx.x < 32) sr[threadIdx.x] = 0;
    __syncthreads();
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < samples; s += gridDim.x * blockDim.x) {
        const uint64_t i = (uint64_t)s * stride;
        unsigned long long hv = 0x9e3779b97f4a7c15ull;
#pragma unroll
        for (int w = 0; w < K; ++w) hv = mix64(hv ^ (keys.w[w][i] & gmask[w]) ^ (0x632be59bd9b4e019ull * (w + 1)));
        const unsigned bucket = (unsigned)(hv >> 59);
        const unsigned rank = (unsigned)__clzll((long long)((hv << 5) | 1ull)) + 1u;
        atomicMax(&sr[bucket], rank);
    }
    __syncthreads();
    if (threadIdx.x < 32) atomicMax(&regs[threadIdx.x], sr[threadIdx.x]);
}

// Grouping of a small state in one CTA: the hash table, the member counts and
// the group starts live in shared memory, so grouping is one launch instead of
// the table clear, insert, scan and bucket launches. A slot holds its head
// entry + 1 (claimed by one compare-and-swap, never locked); later entries
// compare their masked key with the head's. Outputs match the multi-CTA hash
// path: group starts, one head per group, members' (target, amplitude)
// contiguous per group, and the entries that fail the conditions.
constexpr unsigned kSmallGroupMax = 8192;  // entries
constexpr unsigned kSmallPer = kSmallGroupMax / 1024;

template <int K>
__device__ __forceinline__ void group_key_of(const uint64_t (&full)[K], const uint64_t (&gm)[K], Field tgt, Field varw,
                                             uint64_t (&k)[K]) {
#pragma unroll
    for (int w = 0; w < K; ++w) k[w] = full[w] & gm[w];
    if (varw.width) {
        const unsigned nd = (unsigned)fget<K>(full, varw);
        kword_set<K>(k, tgt.word, kword<K>(k, tgt.word) & ~(wmask(nd) << tgt.shift));
    }
}
template <int K>
__device__ __forceinline__ void group_key(const ConstKeyPtrs& keys, unsigned e, const uint64_t (&gm)[K], Field tgt,
                                          Field varw, uint64_t (&k)[K]) {
    uint64_t full[K];
#pragma unroll
    for (int w = 0; w < K; ++w) full[w] = keys.w[w][e];
    group_key_of<K>(full, gm, tgt, varw, k);
}

// an entry's target digits (its own width when the width is per entry) and amplitude
__device__ __forceinline__ void small_member(const ConstKeyPtrs& keys, const double2* __restrict__ amp, unsigned e,
                                             Field tgt, Field varw, unsigned& t, double2& a) {
    const unsigned nd = varw.width ? (unsigned)((keys.w[varw.word][e] >> varw.shift) & wmask(varw.width)) : tgt.width;
    t = (unsigned)((keys.w[tgt.word][e] >> tgt.shift) & wmask(nd));
    a = amp[e];
}
template <int K>
__host__ __device__ constexpr unsigned small_batch() { return K <= 2 ? 4u : K <= 4 ? 2u : 1u; }  // no spills

// A thread's entries are handled in batches of small_batch<K>(), whose key words
// (and, when written out, amplitudes) are loaded before any of them is used,
// so that a batch costs one memory round trip instead of one per entry.
// When every entry passes the conditions and no two entries share a group key
// (the split that follows a merge, as a rule), every group is a singleton: the
// groups are the entries in entry order, written without the scan over the
// table and the bucket pass.
template <int K>
__global__ void __launch_bounds__(1024) group_small_kernel(const __grid_constant__ ConstKeyPtrs keys,
                                                           const uint64_t* __restrict__ gmask,
                                                           const __grid_constant__ DCondSet cond,
                                                           const double2* __restrict__ amp,
                                                           unsigned n, unsigned cap, Field tgt, Field varw,
                                                           unsigned max_digits, unsigned* __restrict__ counts,
                                                           unsigned* __restrict__ seg, unsigned* __restrict__ ghead,
                                                           unsigned* __restrict__ btgt, double2* __restrict__ bamp,
                                                           unsigned* __restrict__ pass_list, unsigned* err) {
    constexpr unsigned kSmallBatch = small_batch<K>();
    extern __shared__ unsigned s_tab[];  // cap slots | cap counts
    unsigned* table = s_tab;
    unsigned* cnt = s_tab + cap;
    __shared__ unsigned s_F, s_dup, s_scan[32][2];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (unsigned i = tid; i < 2 * cap; i += 1024u) s_tab[i] = 0u;
    if (tid == 0) {
        s_F = 0u;
        s_dup = 0u;
    }
    uint64_t gm[K];
#pragma unroll
    for (int w = 0; w < K; ++w) gm[w] = gmask[w];
    __syncthreads();
    unsigned myslot[kSmallPer];
#pragma unroll
    for (unsigned qb = 0; qb < kSmallPer; qb += kSmallBatch) {
        uint64_t full[kSmallBatch][K];
#pragma unroll
        for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
            const unsigned e = tid + (qb + qi) * 1024u;
#pragma unroll
            for (int w = 0; w < K; ++w) full[qi][w] = e < n ? keys.w[w][e] : 0ull;
        }
#pragma unroll
        for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
            const unsigned q = qb + qi, e = tid + q * 1024u;
            myslot[q] = ~0u;
            if (e >= n) continue;
            bool pass = cond_ok<K>(full[qi], cond);
            if (pass && varw.width && (unsigned)fget<K>(full[qi], varw) > max_digits) {
                atomicOr(err, 4u);
                pass = false;
            }
            if (!pass) {
                pass_list[atomicAdd(&s_F, 1u)] = e;
                continue;
            }
            uint64_t k[K];
            group_key_of<K>(full[qi], gm, tgt, varw, k);
            unsigned long long hv = 0x9e3779b97f4a7c15ull;
#pragma unroll
            for (int w = 0; w < K; ++w) hv = mix64(hv ^ k[w] ^ (0x632be59bd9b4e019ull * (w + 1)));
            unsigned slot = (unsigned)hv & (cap - 1u);
            for (unsigned probes = 0; probes < cap; ++probes) {  // the table holds 2x the entries: always ends
                const unsigned old = atomicCAS(&table[slot], 0u, e + 1u);
                if (old == 0u) break;
                uint64_t hk[K];
                group_key<K>(keys, old - 1u, gm, tgt, varw, hk);
                bool eq = true;
#pragma unroll
                for (int w = 0; w < K; ++w) eq = eq && hk[w] == k[w];
                if (eq) {
                    s_dup = 1u;  // a group of two or more members
                    break;
                }
                slot = (slot + 1u) & (cap - 1u);
            }
            myslot[q] = slot;
            atomicAdd(&cnt[slot], 1u);
        }
    }
    __syncthreads();
    if (s_F == 0u && s_dup == 0u) {  // uniform over the CTA
#pragma unroll
        for (unsigned qb = 0; qb < kSmallPer; qb += kSmallBatch) {
            double2 av[kSmallBatch];
            unsigned tv[kSmallBatch];
#pragma unroll
            for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
                const unsigned e = tid + (qb + qi) * 1024u;
                if (e < n) small_member(keys, amp, e, tgt, varw, tv[qi], av[qi]);
            }
#pragma unroll
            for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
                const unsigned e = tid + (qb + qi) * 1024u;
                if (e >= n) continue;
                seg[e] = e;
                ghead[e] = e;
                btgt[e] = tv[qi];
                bamp[e] = av[qi];
            }
        }
        if (tid == 0) {
            counts[0] = n;
            counts[1] = 0u;
            seg[n] = n;
        }
        return;
    }
    // dense group ids and member offsets: one block-wide scan over the slots in order
    const unsigned per = cap / 1024u;  // cap >= 1024
    const unsigned s0 = tid * per;
    unsigned occ = 0, mem = 0;
    for (unsigned i = 0; i < per; ++i) {
        occ += table[s0 + i] ? 1u : 0u;
        mem += cnt[s0 + i];
    }
    unsigned io = occ, im = mem;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned a = __shfl_up_sync(0xffffffffu, io, o), b = __shfl_up_sync(0xffffffffu, im, o);
        if (lane >= (unsigned)o) {
            io += a;
            im += b;
        }
    }
    if (lane == 31) {
        s_scan[warp][0] = io;
        s_scan[warp][1] = im;
    }
    __syncthreads();
    if (warp == 0) {
        unsigned a = s_scan[lane][0], b = s_scan[lane][1];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned x = __shfl_up_sync(0xffffffffu, a, o), y = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= (unsigned)o) {
                a += x;
                b += y;
            }
        }
        s_scan[lane][0] = a;
        s_scan[lane][1] = b;
    }
    __syncthreads();
    unsigned gid = io - occ + (warp ? s_scan[warp - 1][0] : 0u);
    unsigned off = im - mem + (warp ? s_scan[warp - 1][1] : 0u);
    for (unsigned i = 0; i < per; ++i) {
        const unsigned h = table[s0 + i];
        if (!h) continue;
        seg[gid] = off;
        ghead[gid] = h - 1u;
        off += cnt[s0 + i];
        cnt[s0 + i] = seg[gid];  // fill cursor of the slot's group
        ++gid;
    }
    if (tid == 1023) {
        counts[0] = s_scan[31][0];
        counts[1] = s_F;
        seg[s_scan[31][0]] = s_scan[31][1];
    }
    __syncthreads();
    // members, contiguous per group
#pragma unroll
    for (unsigned qb = 0; qb < kSmallPer; qb += kSmallBatch) {
        double2 av[kSmallBatch];
        unsigned tv[kSmallBatch];
#pragma unroll
        for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
            const unsigned e = tid + (qb + qi) * 1024u;
            if (myslot[qb + qi] != ~0u) small_member(keys, amp, e, tgt, varw, tv[qi], av[qi]);
        }
#pragma unroll
        for (unsigned qi = 0; qi < kSmallBatch; ++qi) {
            const unsigned q = qb + qi;
            if (myslot[q] == ~0u) continue;
            const unsigned pos = atomicAdd(&cnt[myslot[q]], 1u);
            btgt[pos] = tv[qi];
            bamp[pos] = av[qi];
        }
    }
}

// Partition the condition-passing entries by group: each entry's target value
// and amplitude land in its group's range [seg[g], seg[g+1]); lanes of a warp
// with the same group reserve consecutive slots with one atomic.
__global__ void __launch_bounds__(256) bucket_kernel(const unsigned* __restrict__ gid, const uint64_t* __restrict__ tword,
                                                     Field target, const double2* __restrict__ amp, uint64_t n,
                                                     const unsigned* __restrict__ seg, unsigned* __restrict__ cnt,
                                                     unsigned* __restrict__ btgt, double2* __restrict__ bamp,
                                                     const uint64_t* __restrict__ wword, Field varw) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t base0 = (uint64_t)blockIdx.x * blockDim.x;
    for (uint64_t b = base0; b < n; b += stride) {  // warp-uniform trip count
        const uint64_t i = b + threadIdx.x;
        const unsigned g = i < n ? gid[i] : ~0u;
        const bool valid = g != ~0u;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        const unsigned peers = __match_any_sync(0xffffffffu, g) & vmask;
        if (valid) {
            const int leader = __ffs(peers) - 1;
            const unsigned rank = __popc(peers & ((1u << lane) - 1u));
            unsigned old = 0;
            if ((int)lane == leader) old = atomicSub(&cnt[g], (unsigned)__popc(peers));
            old = __shfl_sync(peers, old, leader);
            const unsigned pos = seg[g] + old - 1u - rank;
            const unsigned nd = varw.width ? (unsigned)((wword[i] >> varw.shift) & wmask(varw.width)) : target.width;
            btgt[pos] = (unsigned)((tword[i] >> target.shift) & wmask(nd));
            bamp[pos] = amp[i];
        }
    }
}

// Exclusive scan of u32 counts into u32 group starts (seg[G] is written by the host).
__global__ void __launch_bounds__(kSelBlock) scan_seg_kernel(const unsigned* __restrict__ cnt, unsigned* __restrict__ seg,
                                                             uint64_t n, LbWs lb, long long ntiles, unsigned* err) {
    __shared__ unsigned s_tile;
    __shared__ unsigned long long s_w[kSelBlock / 32];
    __shared__ unsigned long long s_prefix;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(lb.counter, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const uint64_t base = (uint64_t)tile * kSelTile + (uint64_t)tid * kSelItems;
    unsigned long long v[kSelItems];
    unsigned long long sum = 0;
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        const uint64_t i = base + j;
        v[j] = i < n ? cnt[i] : 0ull;
        sum += v[j];
    }
    unsigned long long inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned long long wv = lane < kSelBlock / 32 ? s_w[lane] : 0ull;
        unsigned long long wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (unsigned)o) wi += t;
        }
        const unsigned long long total = __shfl_sync(0xffffffffu, wi, kSelBlock / 32 - 1);
        if (lane < kSelBlock / 32) s_w[lane] = wi - wv;
        unsigned long long pre = lb_warp_exclusive(lb.status, tile, total, err);
        if (lane == 0) {
            s_prefix = pre;
            if (tile == ntiles - 1) *lb.total = pre + total;
        }
    }
    __syncthreads();
    unsigned long long run = s_prefix + s_w[warp] + inc - sum;
#pragma unroll
    for (int j = 0; j < kSelItems; ++j) {
        const uint64_t i = base + j;
        if (i < n) seg[i] = (unsigned)run;
        run += v[j];
    }
}

}  // namespace

#ifndef SQ_GROUP_K
static int g_strategy = 3;  // 0 heuristic (hash from 4096 entries), 1 sort, 2 hash, 3 autotuned
static int g_sizing = 0;    // 0 auto (single pass when the output bound fits), 1 exact count-then-scan
void set_output_sizing(int m) {
    if (m < 0 || m > 1) fail(SQ_ERR_INVALID, "output sizing must be 0 (auto) or 1 (count then scan)");
    g_sizing = m;
}
int get_output_sizing() { return g_sizing; }
static int g_arith = SQ_ARITH_EXACT_SUM;
void set_fwht_arithmetic(int m) {
    if (m != SQ_ARITH_REFERENCE && m != SQ_ARITH_EXACT_SUM)
        fail(SQ_ERR_INVALID, "FWHT arithmetic must be 0 (reference FP64) or 1 (exact sum)");
    g_arith = m;
}
int get_fwht_arithmetic() { return g_arith; }
void set_group_strategy(int s) {
    if (s < 0 || s > 3)
        fail(SQ_ERR_INVALID, "group strategy must be 0 (auto), 1 (sort), 2 (hash) or 3 (autotuned)");
    g_strategy = s;
}
int get_group_strategy() { return g_strategy; }

// The autotuner of the grouping: per shape class (operator kind, conditions,
// key words, log2 N) the first split of the class runs the sort grouping, the
// second the hash grouping, each timed on the host around the whole operator
// (both synchronise); later splits of the class use the faster. Results are
// the same either way; only the order of the output entries differs.
namespace {
struct TuneEntry {
    double ms[2] = {0.0, 0.0};
    bool tried[2] = {false, false};
};
std::map<uint64_t, TuneEntry> g_tune;
}  // namespace
int autotune_pick(uint64_t key) {
    TuneEntry& e = g_tune[key];
    int pick = !e.tried[0] ? 1 : !e.tried[1] ? 2 : (e.ms[1] <= e.ms[0] ? 2 : 1);
    host_decision(&pick, sizeof(pick));  // a capture repeats the recorded choice
    return pick;
}
void autotune_record(uint64_t key, int strategy, double ms) {
    if (capturing()) return;  // nothing ran: no time to learn from
    TuneEntry& e = g_tune[key];
    const int i = strategy == 2 ? 1 : 0;
    if (!e.tried[i]) {
        e.tried[i] = true;
        e.ms[i] = ms;
    } else {
        e.ms[i] = 0.75 * e.ms[i] + 0.25 * ms;  // keeps following the class
    }
}
void autotune_reset() { g_tune.clear(); }
uint64_t autotune_classes(uint64_t* decided) {
    uint64_t d = 0;
    for (const auto& kv : g_tune) d += (kv.second.tried[0] && kv.second.tried[1]) ? 1 : 0;
    if (decided) *decided = d;
    return g_tune.size();
}
static uint64_t g_hash_groups_hint = 1ull << 20;
void set_hash_groups_hint(uint64_t g) { g_hash_groups_hint = g ? g : (1ull << 20); }
uint64_t hash_groups_hint() { return g_hash_groups_hint; }
static uint64_t g_out_hint = 0;
void hint_output_size(uint64_t outputs) { g_out_hint = outputs; }
uint64_t take_output_size_hint() {
    const uint64_t h = g_out_hint;
    g_out_hint = 0;
    return h;
}
static uint64_t g_single_limit = 0;  // 0: max(4 N, 2^27)
void set_single_pass_limit(uint64_t entries) { g_single_limit = entries; }
uint64_t single_pass_limit() { return g_single_limit; }
static uint64_t g_overflows = 0;
void note_single_pass_overflow() { ++g_overflows; }
uint64_t single_pass_overflows() { return g_overflows; }
void note_output_size(int, uint64_t, uint64_t, uint64_t) {}
#else

// ------------------------------------------------------------------ host pipeline
struct Grouping {
    uint64_t G = 0;      // groups among the condition-passing entries
    uint64_t F = 0;      // entries failing the conditions
    unsigned* seg = nullptr;
    const unsigned* idx = nullptr;        // sort path
    const unsigned* btgt = nullptr;       // hash path
    const double2* bamp = nullptr;
    const unsigned* ghead = nullptr;
    const unsigned* pass = nullptr;       // failing entries (indices)
    bool bucket = false;
};

template <int K>
static Grouping group_by_sort(State& s, const GroupSpec& gs, const uint64_t* gmask, uint64_t* dg) {
    const uint64_t N = s.n;
    cudaStream_t st = stream();
    ConstKeyPtrs ik;
    for (int w = 0; w < SQ_KMAX; ++w) ik.w[w] = s.live.keys[w];
    unsigned long long* stats = (unsigned long long*)(dg + 16);
    std::vector<unsigned long long> init(2 * K + 1, 0);
    for (int w = 0; w < K; ++w) init[K + w] = ~0ull;
    h2d_small(stats, init.data(), init.size() * 8);
    prof_begin("group_stats");
    stats_kernel<K><<<grid_for(N, 256, 4), 256, 0, st>>>(ik, N, gs.cond, dg, stats);
    prof_end((double)N * 8 * K);
    SQ_CUDA(cudaGetLastError());
    std::vector<unsigned long long> res(2 * K + 1);
    host_read(res.data(), stats, res.size() * 8);
    const uint64_t F = res[2 * K];
    const uint64_t P = N - F;

    // varying group-key bits -> extraction runs (least significant first)
    std::vector<Run> runs;
    int V = 0;
    for (int w = 0; w < K; ++w) {
        uint64_t vm = (res[w] ^ res[K + w]) & gmask[w];
        int b = 0;
        while (b < 64) {
            if (!((vm >> b) & 1ull)) { ++b; continue; }
            int e = b;
            while (e < 64 && ((vm >> e) & 1ull)) ++e;
            runs.push_back(Run{(uint8_t)w, (uint8_t)b, (uint8_t)(e - b), 0});
            V += e - b;
            b = e;
        }
    }
    const int total_bits = V + (F ? 1 : 0);

    unsigned* vbuf[2] = {(unsigned*)ws().get(WS_SORT_VAL0, N * 4 + 16), (unsigned*)ws().get(WS_SORT_VAL1, N * 4 + 16)};
    unsigned* idx = vbuf[0];
    const void* sorted_keys = nullptr;
    int key_bytes = 0;

    if (total_bits == 0) {
        prof_begin("iota");
        iota_kernel<<<grid_for(N, 256), 256, 0, st>>>(idx, N);
        prof_end((double)N * 4);
    } else {
        // split the (V + flag) bits into chunks of <= 64, sort least significant chunk first
        struct Chunk {
            Extract ex;
            int bits;
        };
        std::vector<Chunk> chunks;
        {
            Chunk cur;
            memset(&cur, 0, sizeof(cur));
            cur.ex.flag_bit = 0xff;
            int used = 0;
            for (Run r : runs) {
                int len = r.len;
                int sh = r.shift;
                while (len > 0) {
                    if (used == 64 || cur.ex.nruns == kMaxRuns) {
                        cur.bits = used;
                        chunks.push_back(cur);
                        memset(&cur, 0, sizeof(cur));
                        cur.ex.flag_bit = 0xff;
                        used = 0;
                    }
                    int take = std::min(len, 64 - used);
                    cur.ex.runs[cur.ex.nruns++] = Run{r.word, (uint8_t)sh, (uint8_t)take, (uint8_t)used};
                    used += take;
                    sh += take;
                    len -= take;
                }
            }
            if (F) {
                if (used == 64) {
                    cur.bits = used;
                    chunks.push_back(cur);
                    memset(&cur, 0, sizeof(cur));
                    used = 0;
                }
                cur.ex.flag_bit = (uint32_t)used;
                used += 1;
            } else {
                cur.ex.flag_bit = 0xff;
            }
            cur.bits = used;
            if (used > 0) chunks.push_back(cur);
        }
        const bool small = chunks.size() == 1 && chunks[0].bits <= 32;
        if (small) {
            uint32_t* kb[2] = {(uint32_t*)ws().get(WS_SORT_KEY0, N * 4 + 16), (uint32_t*)ws().get(WS_SORT_KEY1, N * 4 + 16)};
            prof_begin("extract_sort_key");
            extract_kernel<K, uint32_t, false><<<grid_for(N, 256), 256, 0, st>>>(ik, N, chunks[0].ex, gs.cond, kb[0], vbuf[0]);
            prof_end((double)N * (8 * K + 8));
            int r = radix_sort_pairs<uint32_t>(kb, vbuf, N, chunks[0].bits);
            idx = vbuf[r];
            sorted_keys = kb[r];
            key_bytes = 4;
        } else {
            uint64_t* kb[2] = {(uint64_t*)ws().get(WS_SORT_KEY0, N * 8 + 16), (uint64_t*)ws().get(WS_SORT_KEY1, N * 8 + 16)};
            int cur = 0;  // buffer pair holding the current (keys, indices)
            for (size_t c = 0; c < chunks.size(); ++c) {
                prof_begin("extract_sort_key");
                if (c == 0)
                    extract_kernel<K, uint64_t, false><<<grid_for(N, 256), 256, 0, st>>>(ik, N, chunks[c].ex, gs.cond, kb[0], vbuf[0]);
                else  // later chunks: key bits of the entry now at position i
                    extract_kernel<K, uint64_t, true><<<grid_for(N, 256), 256, 0, st>>>(ik, N, chunks[c].ex, gs.cond, kb[cur], vbuf[cur]);
                prof_end((double)N * (8 * K + 12));
                SQ_CUDA(cudaGetLastError());
                uint64_t* kk[2] = {kb[cur], kb[cur ^ 1]};
                unsigned* vv[2] = {vbuf[cur], vbuf[cur ^ 1]};
                const int r = radix_sort_pairs<uint64_t>(kk, vv, N, chunks[c].bits);
                if (r) cur ^= 1;
            }
            idx = vbuf[cur];
            sorted_keys = kb[cur];
            key_bytes = chunks.size() == 1 ? 8 : 0;
        }
    }
    SQ_CUDA(cudaGetLastError());

    // group starts over the first P (condition-passing) entries
    Grouping out;
    out.F = F;
    out.idx = idx;
    out.pass = idx + P;
    unsigned* seg = (unsigned*)ws().get(WS_SEG, (P + 2) * 4);
    out.seg = seg;
    if (P > 0) {
        if (total_bits == 0 || V == 0) {
            unsigned hh[2] = {0u, (unsigned)P};
            h2d_small(seg, hh, 8);
            out.G = 1;
        } else {
            const long long nt = (long long)((P + kSelTile - 1) / kSelTile);
            LbWs lb = make_lb(nt);
            const unsigned grid = (unsigned)nt;
            prof_begin("group_heads");
            if (key_bytes == 4)
                heads_kernel<K, uint32_t, true><<<grid, kSelBlock, 0, st>>>((const uint32_t*)sorted_keys, idx, ik, dg, P, seg, lb, nt, device_error_word());
            else if (key_bytes == 8)
                heads_kernel<K, uint64_t, true><<<grid, kSelBlock, 0, st>>>((const uint64_t*)sorted_keys, idx, ik, dg, P, seg, lb, nt, device_error_word());
            else
                heads_kernel<K, uint64_t, false><<<grid, kSelBlock, 0, st>>>(nullptr, idx, ik, dg, P, seg, lb, nt, device_error_word());
            prof_end((double)P * (key_bytes ? key_bytes : 4 + 8 * K));
            SQ_CUDA(cudaGetLastError());
            unsigned long long g = 0;
            host_read(&g, lb.total, 8);
            check_device_error();
            out.G = g;
            prof_add_bytes_last((double)out.G * 4);
            unsigned endv = (unsigned)P;
            h2d_small(seg + out.G, &endv, 4);
        }
    }
    return out;
}

template <int K>
static Grouping group_by_hash(State& s, const GroupSpec& gs, uint64_t* dg, uint64_t want_groups) {
    const uint64_t N = s.n;
    cudaStream_t st = stream();
    ConstKeyPtrs ik;
    for (int w = 0; w < SQ_KMAX; ++w) ik.w[w] = s.live.keys[w];
    // states up to this many entries are grouped by one CTA (SPARQ_SMALL_GROUP_MAX lowers it)
    static const uint64_t small_max = [] {
        const char* e = getenv("SPARQ_SMALL_GROUP_MAX");
        const long v = e ? atol(e) : -1;
        return v >= 0 && v <= (long)kSmallGroupMax ? (uint64_t)v : (uint64_t)kSmallGroupMax;
    }();
    if (N <= small_max) {
        unsigned cap = 1024;
        while (cap < 2 * N) cap <<= 1;
        // one allocation: counts | seg | head | pass | bucket target | bucket amp
        const size_t o_seg = 64, o_head = o_seg + (N + 2) * 4, o_pass = o_head + N * 4, o_btgt = o_pass + N * 4;
        const size_t o_bamp = (o_btgt + N * 4 + 15) & ~size_t(15), total = o_bamp + N * 16;
        char* base = (char*)ws().get(WS_MERGE_KEYS, total);
        static bool smem_set = false;
        if (!smem_set) {
            SQ_CUDA(cudaFuncSetAttribute(group_small_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * 2 * kSmallGroupMax * 4)));
            smem_set = true;
        }
        prof_begin("group_small");
        group_small_kernel<K><<<1, 1024, 2 * cap * 4, st>>>(
            ik, dg, gs.cond, s.live.amp, (unsigned)N, cap, gs.target, gs.varw, gs.target.width, (unsigned*)base,
            (unsigned*)(base + o_seg), (unsigned*)(base + o_head), (unsigned*)(base + o_btgt),
            (double2*)(base + o_bamp), (unsigned*)(base + o_pass), device_error_word());
        prof_end((double)N * (8.0 * K + 16) * 2);
        SQ_CUDA(cudaGetLastError());
        unsigned gc[2] = {0, 0};
        host_read(gc, base, 8);
        check_device_error();  // synchronizes
        Grouping out;
        out.G = gc[0];
        out.F = gc[1];
        out.seg = (unsigned*)(base + o_seg);
        out.ghead = (unsigned*)(base + o_head);
        out.btgt = (unsigned*)(base + o_btgt);
        out.bamp = (double2*)(base + o_bamp);
        out.pass = (unsigned*)(base + o_pass);
        out.bucket = true;
        return out;
    }
    // Table sized for the expected number of groups (load factor <= 1/2);
    // if more groups show up the kernel flags overflow and we retry with a
    // table that fits every entry.
    uint64_t want = std::min<uint64_t>(N, want_groups ? want_groups : hash_groups_hint());
    HashWs h;
    char* base = nullptr;
    size_t off_btgt = 0, off_bamp = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        uint64_t cap = 1024;
        while (cap < 2 * want) cap <<= 1;
        const uint64_t gmax = cap / 2;
        // one allocation: slots | counters | cnt | head | gid | pass_list | bucket target | bucket amp
        const size_t off_cnt = cap * 8 + 256;
        const size_t off_head = off_cnt + gmax * 4;
        const size_t off_gid = off_head + gmax * 4;
        const size_t off_pass = off_gid + N * 4;
        off_btgt = off_pass + N * 4;
        off_bamp = (off_btgt + N * 4 + 15) & ~size_t(15);
        const size_t total = off_bamp + N * 16;
        base = (char*)ws().get(WS_MERGE_KEYS, total);
        h.slots = (unsigned long long*)base;
        h.cap_mask = cap - 1;
        h.gcount = (unsigned*)(base + cap * 8);
        h.cnt = (unsigned*)(base + off_cnt);
        h.head = (unsigned*)(base + off_head);
        h.gid = (unsigned*)(base + off_gid);
        h.pass_list = (unsigned*)(base + off_pass);
        SQ_CUDA(cudaMemsetAsync(base, 0, off_head, st));  // slots, counters, cnt
        prof_begin("hash_insert");
        hash_insert_kernel<K><<<grid_for(N, 256, 8), 256, 0, st>>>(ik, dg, gs.cond, N, h, (unsigned)gmax, gs.target,
                                                                   gs.varw, gs.target.width, device_error_word());
        prof_end((double)N * (8.0 * K + 4));
        SQ_CUDA(cudaGetLastError());
        unsigned gc[3] = {0, 0, 0};
        host_read(gc, h.gcount, 12);
        check_device_error();
        if (!gc[2]) break;
        if (attempt == 1) fail(SQ_ERR_DEVICE_TIMEOUT, "hash grouping overflowed a table sized for every entry");
        want = N;
    }
    unsigned gc[2] = {0, 0};
    host_read(gc, h.gcount, 8);
    Grouping out;
    out.G = gc[0];
    out.F = gc[1];
    out.pass = h.pass_list;
    out.ghead = h.head;
    out.bucket = true;
    const uint64_t P = N - out.F;
    unsigned* seg = (unsigned*)ws().get(WS_SEG, (out.G + 2) * 4);
    out.seg = seg;
    if (out.G > 0) {
        const long long nt = (long long)((out.G + kSelTile - 1) / kSelTile);
        LbWs lb = make_lb(nt);
        prof_begin("scan_group_sizes");
        scan_seg_kernel<<<(unsigned)nt, kSelBlock, 0, st>>>(h.cnt, seg, out.G, lb, nt, device_error_word());
        prof_end((double)out.G * 8);
        SQ_CUDA(cudaGetLastError());
        unsigned endv = (unsigned)P;
        h2d_small(seg + out.G, &endv, 4);
        unsigned* btgt = (unsigned*)(base + off_btgt);
        double2* bamp = (double2*)(base + off_bamp);
        prof_begin("bucket_members");
        bucket_kernel<<<grid_for(N, 256, 8), 256, 0, st>>>(h.gid, s.live.keys[gs.target.word], gs.target, s.live.amp,
                                                           N, seg, h.cnt, btgt, bamp,
                                                           s.live.keys[gs.varw.width ? gs.varw.word : 0], gs.varw);
        prof_end((double)N * (4 + 8 + 16) + (double)P * (4 + 16 + 8));
        SQ_CUDA(cudaGetLastError());
        out.btgt = btgt;
        out.bamp = bamp;
    }
    return out;
}

// ------------------------------------------------------------------ pair splits by partner lookup
// A 1-bit split pairs each entry with the entry whose key differs in the
// target bit alone. Instead of grouping (hash buckets or a sort of the keys
// without the bit), the entries that pass the conditions go into an
// open-addressing table by their whole key (keys are unique), and every
// entry looks its partner up: the member with bit 0 of a pair, or a member
// without a partner, writes the pair's outputs (pair_math, the arithmetic of
// the grouped path); the member with bit 1 of a pair writes nothing; entries
// that fail the conditions are copied. A slot is (fingerprint 24 | index + 1),
// zero empty; the table holds at least twice the entries, so every probe
// sequence ends at an empty slot.
struct PairTable {
    unsigned long long* slots;
    unsigned long long mask;  // capacity - 1
};
template <int K>
__device__ __forceinline__ unsigned long long full_key_hash(const uint64_t (&k)[K]) {
    unsigned long long hv = 0x9e3779b97f4a7c15ull;
#pragma unroll
    for (int w = 0; w < K; ++w) hv = mix64(hv ^ k[w] ^ (0x632be59bd9b4e019ull * (w + 1)));
    return hv;
}

template <int K>
__global__ void __launch_bounds__(256) pair_table_build_kernel(ConstKeyPtrs keys, uint64_t n, DCondSet cond,
                                                               PairTable t) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k[K];
        load_key<K>(keys, i, k);
        if (!cond_ok<K>(k, cond)) continue;
        const unsigned long long hv = full_key_hash<K>(k);
        const unsigned long long tag = ((hv >> 40) << 32) | (unsigned long long)(i + 1);
        unsigned long long slot = hv & t.mask;
        // at most capacity probes; a lost race re-reads the slot it lost
        // (filled now), so the loop moves on after at most one retry per slot
        for (unsigned long long probes = 0; probes <= t.mask;) {
            const unsigned long long v = t.slots[slot];
            if (v == 0ull) {
                if (atomicCAS(&t.slots[slot], 0ull, tag) == 0ull) break;
                continue;
            }
            slot = (slot + 1) & t.mask;
            ++probes;
        }
    }
}

// The entry index holding key pk, or -1.
template <int K>
__device__ __forceinline__ long long pair_find(const PairTable& t, const ConstKeyPtrs& keys, const uint64_t (&pk)[K]) {
    const unsigned long long hv = full_key_hash<K>(pk);
    const unsigned long long fp = hv >> 40;
    unsigned long long slot = hv & t.mask;
    for (unsigned long long probes = 0; probes <= t.mask; ++probes) {
        const unsigned long long v = __ldg(t.slots + slot);
        if (v == 0ull) return -1;
        if ((v >> 32) == fp) {
            const unsigned long long j = (v & 0xffffffffull) - 1ull;
            bool eq = true;
#pragma unroll
            for (int w = 0; w < K; ++w) eq = eq && (__ldg(keys.w[w] + j) == pk[w]);
            if (eq) return (long long)j;
        }
        slot = (slot + 1) & t.mask;
    }
    return -1;
}

// One thread per entry; the lanes of a warp reserve their outputs with one
// atomic, in lane order. Writes nothing past a.capacity (the bound 2n is
// exact, so that only matters to a graph replayed on other data).
template <int K>
__global__ void __launch_bounds__(256) pair_partner_emit_kernel(const __grid_constant__ EmitArgs a, uint64_t n,
                                                                DCondSet cond, PairTable t) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t bit = 1ull << a.target.shift;
    for (uint64_t gb = (uint64_t)blockIdx.x * blockDim.x; gb < n; gb += stride) {  // warp-uniform trips
        const uint64_t i = gb + threadIdx.x;
        const bool valid = i < n;
        uint64_t k[K];
        double2 rz = make_double2(0.0, 0.0), ro = make_double2(0.0, 0.0);
        bool kz = false, ko = false, copy = false;
        if (valid) {
            load_key<K>(a.in_keys, i, k);
            const double2 ai = a.in_amp[i];
            if (!cond_ok<K>(k, cond)) {
                copy = true;
                rz = ai;
            } else {
                const bool one = (k[a.target.word] & bit) != 0ull;
                uint64_t pk[K];
#pragma unroll
                for (int w = 0; w < K; ++w) pk[w] = k[w];
                pk[a.target.word] ^= bit;
                const long long j = pair_find<K>(t, a.in_keys, pk);
                if (!(one && j >= 0)) {  // the bit-0 member of a pair, or a lone member
                    const double2 aj = j >= 0 ? a.in_amp[j] : make_double2(0.0, 0.0);
                    const double2 az = one ? aj : ai, ao = one ? ai : aj;
                    pair_math<K>(a, k, az, ao, !one || j >= 0, one || j >= 0, rz, ro, kz, ko);
                }
            }
        }
        const unsigned c = copy ? 1u : (unsigned)kz + (unsigned)ko;
        unsigned inc = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= (unsigned)d) inc += v;
        }
        const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
        unsigned long long base = 0;
        if (lane == 31 && total) base = atomicAdd(a.cursor, (unsigned long long)total);
        base = __shfl_sync(0xffffffffu, base, 31);
        if (!valid || c == 0 || base + total > a.capacity) continue;
        unsigned long long o = base + (inc - c);
        if (copy) {
            store_out<K>(a, o, k, rz);
            continue;
        }
        if (kz) {
            fset<K>(k, a.target, 0);
            store_out<K>(a, o++, k, rz);
        }
        if (ko) {
            fset<K>(k, a.target, 1);
            store_out<K>(a, o, k, ro);
        }
    }
}

// Pair split by partner lookup: table build, one emit pass with reserved
// outputs (at most 2N: two per passing entry, one per copied entry).
template <int K>
static void run_pair_partner(State& s, const GroupSpec& gs, EmitArgs& ea) {
    const uint64_t N = s.n;
    cudaStream_t st = stream();
    uint64_t cap = 1024;
    while (cap < 2 * N) cap <<= 1;
    PairTable t;
    t.slots = (unsigned long long*)ws().get(WS_PAIR_TABLE, cap * 8);
    t.mask = cap - 1;
    SQ_CUDA(cudaMemsetAsync(t.slots, 0, cap * 8, st));
    const DCondSet dc = gs.cond;
    prof_begin("pair_table_build");
    pair_table_build_kernel<K><<<grid_for(N, 256, 8), 256, 0, st>>>(ea.in_keys, N, dc, t);
    prof_end((double)N * 8.0 * K + (double)cap * 8);
    SQ_CUDA(cudaGetLastError());
    const uint64_t capT = 2 * N;
    ensure_buffers(s.spare, capT, regtable().k, 0);
    for (int w = 0; w < SQ_KMAX; ++w) ea.out_keys.w[w] = s.spare.keys[w];
    ea.out_amp = s.spare.amp;
    unsigned long long* cur = (unsigned long long*)ws().get(WS_CURSOR, 64);
    ea.cursor = cur;
    ea.capacity = capT;
    SQ_CUDA(cudaMemsetAsync(cur, 0, 8, st));
    prof_begin("emit_pair_partner");
    pair_partner_emit_kernel<K><<<grid_for(N, 256, 8), 256, 0, st>>>(ea, N, dc, t);
    prof_end((double)N * (8.0 * K + 16));
    SQ_CUDA(cudaGetLastError());
    unsigned long long T = 0;
    host_read(&T, cur, 8);
    if (T > capT) fail(SQ_ERR_CAPACITY, "pair split wrote past its bound");
    prof_add_bytes_last((double)T * (8 * K + 16));
    swap_live_spare(s);
    s.n = T;
}

constexpr uint64_t kModelMinEntries = 1ull << 15;  // below this a prediction costs more than it saves

// Features of the size model (layout in sparq_gb300.h).
template <int K>
static void split_features(State& s, const GroupSpec& gs, uint64_t N, const uint64_t* dg, bool cached,
                           uint64_t cached_groups, float* f) {
    const int kind = gs.mode == GM_HADAMARD_INT ? 0 : gs.mode == GM_HADAMARD_FULL ? 1 : gs.mode == GM_HADAMARD_BOOL ? 2
                   : gs.mode == GM_ROT ? 3 : (gs.mode == GM_CONDROT) ? 4 : gs.mode == GM_UNITARY ? 5 : 6;
    f[kind] = 1.f;
    f[7] = gs.varw.width ? 1.f : 0.f;
    f[8] = (float)gs.target.width / 16.f;
    f[9] = (float)K / 8.f;
    f[10] = (float)(std::log2((double)N) / 32.0);
    f[11] = cached ? 1.f : 0.f;
    f[12] = cached ? (float)(std::log2((double)cached_groups + 1.0) / 32.0) : 0.f;
    f[13] = (float)gs.cond.n / 8.f;
    f[15] = 1.f;
    cudaStream_t st = stream();
    unsigned* regs = (unsigned*)ws().get(WS_SKETCH, 32 * 4);
    SQ_CUDA(cudaMemsetAsync(regs, 0, 32 * 4, st));
    const unsigned samples = (unsigned)std::min<uint64_t>(N, 65536);
    ConstKeyPtrs ik;
    for (int w = 0; w < SQ_KMAX; ++w) ik.w[w] = s.live.keys[w];
    prof_begin("size_sketch");
    sketch_kernel<K><<<64, 256, 0, st>>>(ik, dg, N / samples, samples, regs);
    prof_end((double)samples * 8 * K);
    SQ_CUDA(cudaGetLastError());
    unsigned h[32];
    host_read(h, regs, sizeof(h));
    for (int i = 0; i < 32; ++i) f[16 + i] = (float)h[i] / 32.f;
}

// The counters of the dynamic group order (two words, zero between launches).
static unsigned long long* group_ticket(cudaStream_t st) {
    static unsigned long long* p = nullptr;
    if (!p) {
        p = (unsigned long long*)dev_alloc(16);
        SQ_CUDA(cudaMemsetAsync(p, 0, 16, st));
    }
    return p;
}

template <int K, int MODE>
static void launch_h4096_fp64(int am, unsigned grid, size_t sm, cudaStream_t st, const EmitArgs& ea) {
    if (am == 2) emit_h4096_kernel<K, MODE, 2><<<grid, 256, sm, st>>>(ea);
    else if (am == 1) emit_h4096_kernel<K, MODE, 1><<<grid, 256, sm, st>>>(ea);
    else emit_h4096_kernel<K, MODE, 0><<<grid, 256, sm, st>>>(ea);
}
template <int K, int MODE>
static void launch_h4096(int am, unsigned grid, size_t sm, cudaStream_t st, const EmitArgs& ea) {
    if (ea.fix) {  // exact sums: 512 threads, 8 slots each
        // am: 0-2 access mode; 3 full cached ranges; 4 / 5 singletons (access mode 0 / 1)
        if (am == 3) emit_h4096x_kernel<K, MODE, 2, H_FULL><<<grid, 512, sm, st>>>(ea);
        else if (am == 4) emit_h4096x_kernel<K, MODE, 0, H_SINGLE><<<grid, 512, sm, st>>>(ea);
        else if (am == 5) emit_h4096x_kernel<K, MODE, 1, H_SINGLE><<<grid, 512, sm, st>>>(ea);
        else if (am == 2) emit_h4096x_kernel<K, MODE, 2, H_ANY><<<grid, 512, sm, st>>>(ea);
        else if (am == 1) emit_h4096x_kernel<K, MODE, 1, H_ANY><<<grid, 512, sm, st>>>(ea);
        else emit_h4096x_kernel<K, MODE, 0, H_ANY><<<grid, 512, sm, st>>>(ea);
    } else {
        launch_h4096_fp64<K, MODE>(am == 3 ? 2 : am == 4 ? 0 : am == 5 ? 1 : am, grid, sm, st, ea);
    }
}
template <int K, int W, bool WRITE>
static void launch_hadamard(int am, unsigned grid, size_t sm, cudaStream_t st, const EmitArgs& ea) {
    if (am == 2) emit_hadamard_kernel<K, W, WRITE, 2><<<grid, 256, sm, st>>>(ea);
    else if (am == 1) emit_hadamard_kernel<K, W, WRITE, 1><<<grid, 256, sm, st>>>(ea);
    else emit_hadamard_kernel<K, W, WRITE, 0><<<grid, 256, sm, st>>>(ea);
}
template <int K, int NB, bool WRITE, bool UNI>
static void launch_small_am(int am, unsigned grid, cudaStream_t st, const EmitArgs& ea) {
    if (am == 2) emit_small_kernel<K, NB, WRITE, 2, UNI><<<grid, 256, 0, st>>>(ea);
    else if (am == 1) emit_small_kernel<K, NB, WRITE, 1, UNI><<<grid, 256, 0, st>>>(ea);
    else emit_small_kernel<K, NB, WRITE, 0, UNI><<<grid, 256, 0, st>>>(ea);
}
template <int K, int NB, bool WRITE>
static void launch_small_nb(int am, unsigned grid, cudaStream_t st, const EmitArgs& ea) {
    if (ea.mode == GM_UNITARY) launch_small_am<K, NB, WRITE, true>(am, grid, st, ea);
    else launch_small_am<K, NB, WRITE, false>(am, grid, st, ea);
}
template <int K, bool WRITE>
static void launch_small(int am, int nb, unsigned grid, cudaStream_t st, const EmitArgs& ea) {
    if (nb == 1) launch_small_nb<K, 1, WRITE>(am, grid, st, ea);
    else if (nb == 2) launch_small_nb<K, 2, WRITE>(am, grid, st, ea);
    else if (nb == 3) launch_small_nb<K, 3, WRITE>(am, grid, st, ea);
    else launch_small_am<K, 4, WRITE, false>(am, grid, st, ea);  // Hadamards only
}
template <int K>
static void set_emit_smem_limits() {
    const int sm = 4096 * (int)sizeof(double2);
    const int g = 96 * 1024;
#define SQ_SMEM(f, b) SQ_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, b))
#define SQ_SMEM_H(m)                                                                                           \
    SQ_SMEM((emit_h4096_kernel<K, m, 0>), sm); SQ_SMEM((emit_h4096_kernel<K, m, 1>), sm);                     \
    SQ_SMEM((emit_h4096_kernel<K, m, 2>), sm); SQ_SMEM((emit_h4096x_kernel<K, m, 0, H_ANY>), sm);              \
    SQ_SMEM((emit_h4096x_kernel<K, m, 1, H_ANY>), sm); SQ_SMEM((emit_h4096x_kernel<K, m, 2, H_ANY>), sm);     \
    SQ_SMEM((emit_h4096x_kernel<K, m, 2, H_FULL>), sm); SQ_SMEM((emit_h4096x_kernel<K, m, 0, H_SINGLE>), sm); \
    SQ_SMEM((emit_h4096x_kernel<K, m, 1, H_SINGLE>), sm);
    SQ_SMEM_H(EMIT_COUNT)
    SQ_SMEM_H(EMIT_WRITE)
    SQ_SMEM_H(EMIT_ATOMIC)
#undef SQ_SMEM_H
    SQ_SMEM((emit_hadamard_kernel<K, 256, true, 0>), g); SQ_SMEM((emit_hadamard_kernel<K, 256, true, 1>), g);
    SQ_SMEM((emit_hadamard_kernel<K, 256, true, 2>), g); SQ_SMEM((emit_hadamard_kernel<K, 256, false, 0>), g);
    SQ_SMEM((emit_hadamard_kernel<K, 256, false, 1>), g); SQ_SMEM((emit_hadamard_kernel<K, 256, false, 2>), g);
#undef SQ_SMEM
}

static bool same_field(const Field& a, const Field& b) {
    return a.word == b.word && a.shift == b.shift && a.width == b.width;
}
static void ensure_cache_set(GroupCache& c, int i, uint64_t G) {
    if (c.cap[i] >= G) return;
    const uint64_t cap = std::max<uint64_t>(G + G / 4, 1024);
    dev_free(c.start[i]);
    dev_free(c.cnt[i]);
    c.start[i] = nullptr;
    c.cnt[i] = nullptr;
    c.cap[i] = 0;
    c.start[i] = (unsigned long long*)dev_alloc(cap * 8);
    c.cnt[i] = (unsigned*)dev_alloc(cap * 4);
    c.cap[i] = cap;
}

template <int K>
static void run_group(State& s, const GroupSpec& gs) {
    const uint64_t N = s.n;
    cudaStream_t st = stream();
    ConstKeyPtrs ik;
    for (int w = 0; w < SQ_KMAX; ++w) ik.w[w] = s.live.keys[w];

    // 1-bit splits: partner lookup instead of a grouping, under the default
    // strategies with single-pass sizing (the 'sort' and 'hash' strategies
    // and exact sizing keep the grouped path, the same arithmetic)
    {
        const bool pair_mode = gs.mode == GM_HADAMARD_BOOL || gs.mode == GM_ROT || gs.mode == GM_CONDROT;
        const int strat0 = get_group_strategy();
        bool partner = pair_mode && !gs.varw.width && (strat0 == 0 || strat0 == 3) && get_output_sizing() == 0;
        host_decision(&partner, sizeof(partner));
        if (partner) {
            s.groups.valid = false;
            EmitArgs ea;
            memset(&ea, 0, sizeof(ea));
            ea.in_keys = ik;
            ea.in_amp = s.live.amp;
            ea.target = gs.target;
            ea.aux = gs.aux;
            ea.mode = gs.mode;
            ea.nbits = 1;
            ea.sqrt2inv = 1.0 / std::sqrt(2.0);
            ea.eps = gs.eps;
            ea.sign2pi = gs.sign * 2 * 3.14159265358979323846;
            for (int i = 0; i < 4; ++i) ea.m[i] = gs.m[i];
            ea.mtable = gs.mtable;
            ea.err = device_error_word();
            run_pair_partner<K>(s, gs, ea);
            return;
        }
    }

    // group mask: active bits except the target bits
    uint64_t gmask[SQ_KMAX];
    regtable().active_mask(gmask);
    // fixed width: the target bits never belong to the group key; batched
    // width: the hash kernel clears each entry's own low n bits
    if (gs.target.width && !gs.varw.width) gmask[gs.target.word] &= ~(wmask(gs.target.width) << gs.target.shift);
    uint64_t* dg = (uint64_t*)ws().get(WS_REDUCE, 64 * 8);
    h2d_small(dg, gmask, SQ_KMAX * 8);

    // the merge sums runs in order, so it keeps the (stable) sort; the
    // transforms are order-independent and default to the hash grouping
    int strat = get_group_strategy();
    uint64_t tune_key = 0;
    const bool tuned = strat == 3 && gs.mode != GM_MERGE && !gs.varw.width && N >= 4096;
    if (tuned) {
        tune_key = (uint64_t)gs.mode | ((uint64_t)gs.cond.n << 8) | ((uint64_t)K << 16) |
                   ((uint64_t)(63 - __builtin_clzll(N)) << 24);
        strat = autotune_pick(tune_key);
    } else if (strat == 3) {
        strat = 0;
    }
    const bool use_hash = gs.varw.width || (gs.mode != GM_MERGE && (strat == 2 || (strat == 0 && N >= 4096)));
    struct TuneTimer {
        bool on;
        uint64_t key;
        int strategy;
        std::chrono::steady_clock::time_point t0;
        ~TuneTimer() {
            if (on) autotune_record(key, strategy,
                                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        }
    } tune_timer{tuned, tune_key, strat, std::chrono::steady_clock::now()};
    // A Hadamard on the same bits as the split that produced this state (no
    // key change since, no conditions) takes that split's output ranges as
    // its groups: every member is still read and transformed, only the
    // grouping pass is not needed.
    GroupCache& gc = s.groups;
    const bool cache_out = gs.mode == GM_HADAMARD_INT || gs.mode == GM_HADAMARD_FULL;
    const bool reuse = gc.valid && cache_out && gs.cond.n == 0 && same_field(gc.target, gs.target) &&
                       same_field(gc.varw, gs.varw) && std::equal(gmask, gmask + SQ_KMAX, gc.gmask);
    gc.valid = false;
    if (reuse) tune_timer.on = false;  // no grouping to time

    // the size model: features before the operator, sizes after it
    const bool model_on = (predictor_enabled() || predictor_logging()) && N >= kModelMinEntries;
    float feat[SQ_PRED_FEATURES] = {0.f};
    float pred[2] = {0.f, 0.f};
    bool have_pred = false;
    if (model_on) {
        split_features<K>(s, gs, N, dg, reuse, gc.G, feat);
        have_pred = predictor_predict(feat, pred);
    }
    const double g_pred = have_pred ? (double)N * std::exp2(16.0 * pred[0]) : 0.0;
    const double t_pred = have_pred ? (double)N * std::exp2(16.0 * pred[1]) : 0.0;

    Grouping gr;
    if (reuse) gr.G = gc.G;
    else if (use_hash) gr = group_by_hash<K>(s, gs, dg, have_pred ? (uint64_t)(g_pred * 1.5) + 1024 : 0);
    else gr = group_by_sort<K>(s, gs, gmask, dg);
    // logged once the output size is known
    auto log_sizes = [&](uint64_t T_out) {
        if (!model_on || !predictor_logging()) return;
        const float t[2] = {(float)(std::log2((double)std::max<uint64_t>(gr.G, 1) / (double)N) / 16.0),
                            (float)(std::log2((double)(T_out + 1) / (double)N) / 16.0)};
        predictor_log(feat, t);
    };
    const int am = reuse ? 2 : gr.bucket ? 1 : 0;
    const int out_set = 1 - gc.cur;
    const uint64_t G = gr.G, F = gr.F, P = N - F;

    // emit: count pass, scan, write pass
    EmitArgs ea;
    memset(&ea, 0, sizeof(ea));
    ea.in_keys = ik;
    ea.in_amp = s.live.amp;
    ea.idx = gr.idx;
    ea.btgt = gr.btgt;
    ea.bamp = gr.bamp;
    ea.ghead = gr.ghead;
    ea.seg = gr.seg;
    ea.groups = G;
    ea.target = gs.target;
    ea.aux = gs.aux;
    ea.mode = gs.mode;
    ea.nbits = gs.target.width;
    ea.extra = gs.unscaled ? 1.0 : 1.0 / std::sqrt((double)(1ull << gs.target.width));
    ea.sqrt2inv = 1.0 / std::sqrt(2.0);
    ea.eps = gs.eps;
    ea.sign2pi = gs.sign * 2 * 3.14159265358979323846;
    for (int i = 0; i < 4; ++i) ea.m[i] = gs.m[i];
    ea.mtable = gs.mtable;
    ea.umat = gs.umat;
    ea.udag = gs.udag;
    ea.varw = gs.varw;
    ea.fix = get_fwht_arithmetic() == SQ_ARITH_EXACT_SUM ? 1 : 0;
    if (reuse) {
        ea.rstart = gc.start[gc.cur];
        ea.rcnt = gc.cnt[gc.cur];
    }
    if (cache_out && gr.F == 0 && gr.G > 0) {
        ensure_cache_set(gc, out_set, gr.G);
        ea.ostart = gc.start[out_set];
        ea.ocnt = gc.cnt[out_set];
    }
    // the ranges are kept when every entry landed in one (no pass-through)
    auto keep_ranges = [&]() {
        if (!ea.ocnt) return;
        gc.valid = true;
        gc.cur = out_set;
        gc.G = gr.G;
        gc.target = gs.target;
        gc.varw = gs.varw;
        std::copy(gmask, gmask + SQ_KMAX, gc.gmask);
    };
    ea.cnt = (unsigned*)ws().get(WS_COUNT, (G + 1) * 4);
    unsigned long long* off = (unsigned long long*)ws().get(WS_OFFSET, (G + 1) * 8);
    ea.off = off;

    const bool pair = gs.mode == GM_HADAMARD_BOOL || gs.mode == GM_ROT || gs.mode == GM_CONDROT;
    const int nb = gs.target.width;
    const unsigned S = 1u << nb;
    size_t smem = 0;
    int W = 0;
    if (!pair && gs.mode != GM_MERGE) {
        if (nb > 12) fail(SQ_ERR_UNSUPPORTED, "Hadamard on more than 12 bits at once is not provided by this engine");
        if (gs.mode == GM_UNITARY && nb > 8) fail(SQ_ERR_UNSUPPORTED, "Rot_GeneralUnitary on more than 8 bits");
        W = S <= 256 ? 32 : 256;
        smem = (size_t)(W == 32 ? 8 : 1) * S * sizeof(double2);
    }
    const bool bk = gr.bucket;
    // targets of 1 to 3 bits, and Hadamards on 4 bits (not batched): one
    // thread per group (a 16-slot unitary is 256 complex products a thread)
    const bool small = !pair && gs.mode != GM_MERGE && !gs.varw.width && nb >= 1 &&
                       (nb <= 3 || (nb == 4 && gs.mode != GM_UNITARY));
    uint64_t T = 0;
    // Hadamard on 12 bits: register FWHT kernel; single pass when the output
    // bound (every group fully populated) fits a modest multiple of the input
    const bool h4096 = !pair && gs.mode != GM_MERGE && gs.mode != GM_UNITARY && nb == 12;
    // Output sizing. Single pass (each group reserves its outputs with one
    // atomic) when an output capacity is known up front: the bound "every
    // group fully populated" when it fits a modest multiple of the input, else
    // a predicted size when one was given (size_hint_outputs). A single pass
    // whose outputs overflow the capacity writes nothing past it and the
    // exact count-then-scan path runs instead, so results never depend on
    // the capacity.
    const bool generic = !pair && gs.mode != GM_MERGE;
    const bool sizable = gs.mode != GM_MERGE;  // pairs: at most two outputs per group
    const uint64_t boundT = sizable ? G * (uint64_t)S : 0;
    const uint64_t policy = single_pass_limit() ? single_pass_limit() : std::max<uint64_t>(4 * N, 1ull << 27);
    uint64_t capT = 0;
    // a warp per group reserves its outputs with one atomic on one cursor;
    // past about a million groups that serialisation costs more than a count
    // pass (the one-thread-per-group kernels reserve once per 32 groups)
    const uint64_t max_single_groups = 1ull << 20;
    if (sizable && get_output_sizing() == 0 && G > 0 && (pair || small || G <= max_single_groups)) {
        const uint64_t hint = take_output_size_hint();
        if (boundT <= policy) capT = boundT;
        else if (hint) capT = std::min<uint64_t>(hint, boundT);
        else if (have_pred) capT = std::min<uint64_t>((uint64_t)(t_pred * 1.25) + 4096, boundT);
    }
    host_decision(&capT, sizeof(capT));  // a capture sizes the outputs as the recorded pass did
    const bool single_pass = capT > 0;
    {
        static bool limits_set = false;
        if (!limits_set) {
            set_emit_smem_limits<K>();
            limits_set = true;
        }
    }
    // Algorithmic bytes of a split, as the operator is defined: every entry
    // in and every entry out once, E = 8K + 16 bytes each, (P + T) * E, booked
    // on the launch that writes the outputs; a count pass books its re-read
    // of the inputs, P * E. (What the kernels physically move differs by
    // access mode: a full cached range is read as amplitudes only.)
    const double E = 8.0 * K + 16.0;
    auto launch_h4096_mode = [&](int mode) {
        const unsigned grid = (unsigned)std::min<uint64_t>(G, (uint64_t)num_sms() * 2);
        ea.ticket = group_ticket(st);
        ea.err = device_error_word();
        // cached ranges holding N = 4096 G entries are all full (none holds
        // more); G = P groups of an integer Hadamard are all singletons
        const int amx = am == 2 && F == 0 && N == G * 4096ull                  ? 3
                        : am < 2 && gs.mode == GM_HADAMARD_INT && G == P && !gs.varw.width ? 4 + am
                                                                                          : am;
        const size_t sm = 4096 * sizeof(double2);
        // the single-pass forms are named apart: the merge of full cached
        // ranges and the split of singletons bound differently
        prof_begin(mode == EMIT_COUNT   ? "emit_h4096_count"
                   : mode == EMIT_WRITE ? "emit_h4096_write"
                   : amx == 3           ? "emit_h4096_merge"
                   : amx >= 4           ? "emit_h4096_split"
                                        : "emit_h4096_single_pass");
        if (mode == EMIT_COUNT) launch_h4096<K, EMIT_COUNT>(amx, grid, sm, st, ea);
        else if (mode == EMIT_WRITE) launch_h4096<K, EMIT_WRITE>(amx, grid, sm, st, ea);
        else launch_h4096<K, EMIT_ATOMIC>(amx, grid, sm, st, ea);
        prof_end(mode == EMIT_COUNT ? (double)P * E : (double)(P + T) * E);
        SQ_CUDA(cudaGetLastError());
    };
    if (single_pass) {
        ensure_buffers(s.spare, capT + F, regtable().k, 0);
        for (int w = 0; w < SQ_KMAX; ++w) ea.out_keys.w[w] = s.spare.keys[w];
        ea.out_amp = s.spare.amp;
        unsigned long long* cur = (unsigned long long*)ws().get(WS_CURSOR, 64);
        ea.cursor = cur;
        ea.capacity = capT;
        SQ_CUDA(cudaMemsetAsync(cur, 0, 8, st));
        if (h4096) {
            launch_h4096_mode(EMIT_ATOMIC);
        } else if (pair) {  // one atomic per warp of groups
            prof_begin("emit_pair_single_pass");
            if (bk) emit_pair_kernel<K, true, true><<<grid_for(G, 256), 256, 0, st>>>(ea);
            else emit_pair_kernel<K, true, false><<<grid_for(G, 256), 256, 0, st>>>(ea);
            prof_end((double)P * E);
            SQ_CUDA(cudaGetLastError());
        } else if (small) {
            prof_begin("emit_small_single_pass");
            launch_small<K, true>(am, nb, grid_for(G, 256), st, ea);
            prof_end((double)P * E);
            SQ_CUDA(cudaGetLastError());
        } else {
            // a fresh grouping (no empty groups) whose groups are all (G == P) or
            // mostly (2G > P) singletons: the fan-out kernel, which lists the
            // groups of several members for the warp-per-group kernel after it
            const bool fanout = W == 32 && gs.mode == GM_HADAMARD_INT && am < 2 && 2 * G > P;
            // named apart by what the groups mostly are: members of several-member
            // groups (merges) or singletons fanned out
            prof_begin(fanout          ? "emit_fanout_single_pass"
                       : 2 * G <= P    ? "emit_hadamard_merge"
                                       : "emit_hadamard_single_pass");
            const unsigned fgrid = (unsigned)std::min<uint64_t>((G + 7) / 8, (uint64_t)num_sms() * 8);
            if (fanout) {
                ea.err = device_error_word();
                // 256 groups per CTA and round (a group per lane)
                const unsigned ogrid = (unsigned)std::min<uint64_t>((G + 255) / 256, (uint64_t)num_sms() * 8);
                if (G < P) {  // the list's length, then the group ids
                    unsigned* gl = (unsigned*)ws().get(WS_GROUP_LIST, (G + 16) * 4);
                    SQ_CUDA(cudaMemsetAsync(gl, 0, 4, st));
                    ea.glist_n = gl;
                    ea.glist = gl + 16;
                }
                if (am == 1) emit_fanout_kernel<K, 1><<<ogrid, 256, 0, st>>>(ea);
                else emit_fanout_kernel<K, 0><<<ogrid, 256, 0, st>>>(ea);
                if (G < P) {
                    SQ_CUDA(cudaGetLastError());
                    launch_hadamard<K, 32, true>(am, fgrid, smem, st, ea);
                    ea.glist = ea.glist_n = nullptr;
                }
            } else if (W == 32) launch_hadamard<K, 32, true>(am, fgrid, smem, st, ea);
            else launch_hadamard<K, 256, true>(am, (unsigned)std::min<uint64_t>(G, (uint64_t)num_sms() * 2), smem, st, ea);
            prof_end((double)P * E);
            SQ_CUDA(cudaGetLastError());
        }
        unsigned long long t = 0;
        host_read(&t, cur, 8);
        ea.cursor = nullptr;
        ea.capacity = 0;
        note_output_size(gs.mode, N, G, t);
        if (t <= capT) {
            T = t;
            log_sizes(T);
            prof_add_bytes_last((double)T * (8 * K + 16));
            if (F) {
                prof_begin("passthrough");
                passthrough_kernel<K><<<grid_for(F, 256), 256, 0, st>>>(ik, s.live.amp, gr.pass, F, ea.out_keys, ea.out_amp, T);
                prof_end((double)F * (4 + 2.0 * (8 * K + 16)));
                SQ_CUDA(cudaGetLastError());
            }
            swap_live_spare(s);
            s.n = T + F;
            keep_ranges();
            return;
        }
        // the capacity was too small: nothing usable was written, run exactly
        note_single_pass_overflow();
    }
    auto launch_emit = [&](bool write) {
        if (h4096) {
            if (G > 0) launch_h4096_mode(write ? EMIT_WRITE : EMIT_COUNT);
            return;
        }
        if (G == 0) return;
        prof_begin(write ? (pair ? "emit_pair_write" : gs.mode == GM_MERGE ? "emit_merge_write"
                                                    : small ? "emit_small_write" : "emit_hadamard_write")
                         : (pair ? "emit_pair_count" : gs.mode == GM_MERGE ? "emit_merge_count"
                                                    : small ? "emit_small_count" : "emit_hadamard_count"));
        if (small) {
            if (write) launch_small<K, true>(am, nb, grid_for(G, 256), st, ea);
            else launch_small<K, false>(am, nb, grid_for(G, 256), st, ea);
        } else if (pair) {
            const unsigned grid = grid_for(G, 256);
            if (write && bk) emit_pair_kernel<K, true, true><<<grid, 256, 0, st>>>(ea);
            else if (write) emit_pair_kernel<K, true, false><<<grid, 256, 0, st>>>(ea);
            else if (bk) emit_pair_kernel<K, false, true><<<grid, 256, 0, st>>>(ea);
            else emit_pair_kernel<K, false, false><<<grid, 256, 0, st>>>(ea);
        } else if (gs.mode == GM_MERGE) {
            if (write) emit_merge_kernel<K, true><<<grid_for(G, 256), 256, 0, st>>>(ea);
            else emit_merge_kernel<K, false><<<grid_for(G, 256), 256, 0, st>>>(ea);
        } else if (W == 32) {
            const unsigned grid = (unsigned)std::min<uint64_t>((G + 7) / 8, (uint64_t)num_sms() * 8);
            if (write) launch_hadamard<K, 32, true>(am, grid, smem, st, ea);
            else launch_hadamard<K, 32, false>(am, grid, smem, st, ea);
        } else {
            const unsigned grid = (unsigned)std::min<uint64_t>(G, (uint64_t)num_sms() * 2);
            if (write) launch_hadamard<K, 256, true>(am, grid, smem, st, ea);
            else launch_hadamard<K, 256, false>(am, grid, smem, st, ea);
        }
        prof_end(write ? (double)(P + T) * E : (double)P * E);
        SQ_CUDA(cudaGetLastError());
    };
    launch_emit(false);
    if (G > 0) {
        const long long nt = (long long)((G + kSelTile - 1) / kSelTile);
        LbWs lb = make_lb(nt);
        prof_begin("scan_counts");
        scan_counts_kernel<<<(unsigned)nt, kSelBlock, 0, st>>>(ea.cnt, off, G, lb, nt, device_error_word());
        prof_end((double)G * 12);
        SQ_CUDA(cudaGetLastError());
        unsigned long long t = 0;
        host_read(&t, lb.total, 8);
        check_device_error();
        T = t;
    }
    if (generic) note_output_size(gs.mode, N, G, T);
    log_sizes(T);
    const uint64_t out_n = T + F;
    ensure_buffers(s.spare, std::max<uint64_t>(out_n, 1), regtable().k, 0);
    for (int w = 0; w < SQ_KMAX; ++w) ea.out_keys.w[w] = s.spare.keys[w];
    ea.out_amp = s.spare.amp;
    ea.capacity = T;
    launch_emit(true);
    if (F) {
        prof_begin("passthrough");
        passthrough_kernel<K><<<grid_for(F, 256), 256, 0, st>>>(ik, s.live.amp, gr.pass, F, ea.out_keys, ea.out_amp, T);
        prof_end((double)F * (4 + 2.0 * (8 * K + 16)));
        SQ_CUDA(cudaGetLastError());
    }
    if (ea.ocnt) {  // count-then-scan: the counts and offsets are the output ranges
        SQ_CUDA(cudaMemcpyAsync(ea.ocnt, ea.cnt, G * 4, cudaMemcpyDeviceToDevice, st));
        SQ_CUDA(cudaMemcpyAsync(ea.ostart, off, G * 8, cudaMemcpyDeviceToDevice, st));
    }
    swap_live_spare(s);
    s.n = out_n;
    keep_ranges();
}

#define SQ_CAT2(a, b) a##b
#define SQ_CAT(a, b) SQ_CAT2(a, b)
void SQ_CAT(run_group_k, SQ_GROUP_K)(State& s, const GroupSpec& g) { run_group<SQ_GROUP_K>(s, g); }
#endif  // SQ_GROUP_K

#ifndef SQ_GROUP_K
void run_group_k1(State&, const GroupSpec&);
void run_group_k2(State&, const GroupSpec&);
void run_group_k3(State&, const GroupSpec&);
void run_group_k4(State&, const GroupSpec&);
void run_group_k5(State&, const GroupSpec&);
void run_group_k6(State&, const GroupSpec&);
void run_group_k7(State&, const GroupSpec&);
void run_group_k8(State&, const GroupSpec&);

void group_transform(State& s, const GroupSpec& g) {
    sync_words(s);
    if (s.n == 0) return;
    if (s.n >= (1ull << 30)) fail(SQ_ERR_CAPACITY, "split/merge operators are limited to < 2^30 entries");
    switch (regtable().k) {
        case 1: run_group_k1(s, g); break;
        case 2: run_group_k2(s, g); break;
        case 3: run_group_k3(s, g); break;
        case 4: run_group_k4(s, g); break;
        case 5: run_group_k5(s, g); break;
        case 6: run_group_k6(s, g); break;
        case 7: run_group_k7(s, g); break;
        default: run_group_k8(s, g); break;
    }
}

// add_systems: dst = merge(dst ++ coef*src), equal keys summed in (dst, src) order.
__global__ void scale_copy_kernel(const double2* __restrict__ in, double2* __restrict__ out, uint64_t n, double k,
                                  int do_scale) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 v = in[i];
        out[i] = do_scale ? make_double2(v.x * k, v.y * k) : v;
    }
}

void add_systems(State& dst, const State& src, double coef) {
    if (src.n == 0) return;
    sync_words(dst);
    const uint32_t k = regtable().k;
    const uint64_t n0 = dst.n, n1 = src.n;
    ensure_buffers(dst.live, n0 + n1, k, n0);
    cudaStream_t st = stream();
    for (uint32_t w = 0; w < k; ++w) {
        if (w < src.live.kalloc)
            SQ_CUDA(cudaMemcpyAsync(dst.live.keys[w] + n0, src.live.keys[w], n1 * 8, cudaMemcpyDeviceToDevice, st));
        else
            SQ_CUDA(cudaMemsetAsync(dst.live.keys[w] + n0, 0, n1 * 8, st));
    }
    const int do_scale = std::abs(coef - 1.0) > 1e-14 ? 1 : 0;
    prof_begin("scale_copy");
    scale_copy_kernel<<<grid_for(n1, 256), 256, 0, st>>>(src.live.amp, dst.live.amp + n0, n1, coef, do_scale);
    prof_end((double)n1 * 32);
    SQ_CUDA(cudaGetLastError());
    dst.n = n0 + n1;
    if (n0 == 0) return;
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_MERGE;
    g.eps = 1e-14;
    group_transform(dst, g);
}
#endif  // !SQ_GROUP_K

}  // namespace sq
