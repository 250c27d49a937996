// compact.cu — ClearZero (order-preserving single-pass stream compaction),
// Normalize (deterministic FP64 two-level reduction + scale).
//
// ClearZero reads each amplitude once, and the key words of surviving entries
// once, and writes the survivors once: N*16 + N_out*(8K+16) bytes, the
// algorithmic minimum. Tile offsets come from a decoupled look-back, so the
// kernel is a single pass and keeps the reference's remove_if order.
#include <cmath>
#include <cstring>
#include <limits>

#include "lookback.cuh"
#include "sq_internal.cuh"

namespace sq {

constexpr int kCzBlock = 256;
constexpr int kCzItems = 8;
constexpr int kCzTile = kCzBlock * kCzItems;

struct LookbackWs {
    unsigned long long* status;
    unsigned* counter;
    unsigned long long* total;
};

// Layout of the look-back workspace: [counter (u32) | total (u64) | pad to 256 B | status[ntiles]].
static LookbackWs lookback_ws(long long ntiles) {
    size_t bytes = 256 + (size_t)ntiles * 8;
    char* p = (char*)ws().get(WS_LOOKBACK, bytes);
    SQ_CUDA(cudaMemsetAsync(p, 0, bytes, stream()));
    LookbackWs w;
    w.counter = (unsigned*)p;
    w.total = (unsigned long long*)(p + 8);
    w.status = (unsigned long long*)(p + 256);
    return w;
}

// Entries kept by a selection on key values (PartialTraceSelect[Range]): all
// conditions of `sel` hold and, if rf has a width, lo <= value(rf) <= hi.
double norm_sq(const State& s);
void scale_amp(State& s, double k);

struct KeySelect {
    DCondSet sel;
    Field rf;
    uint64_t lo, hi;
};

// SEL = false: ClearZero (keep |a|^2 >= eps); SEL = true: keep the entries the
// key selection accepts. Same single pass either way.
template <int K, bool SEL>
__global__ void __launch_bounds__(kCzBlock) clearzero_kernel(ConstKeyPtrs ik, const double2* __restrict__ ia,
                                                             KeyPtrs ok, double2* __restrict__ oa, uint64_t n,
                                                             double eps, LookbackWs lb, long long ntiles,
                                                             unsigned* err, const __grid_constant__ KeySelect ks) {
    __shared__ unsigned s_tile;
    __shared__ unsigned s_cnt[kCzItems][kCzBlock / 32];
    __shared__ unsigned long long s_prefix;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(lb.counter, 1u);
    __syncthreads();
    const long long tile = s_tile;
    const uint64_t base = (uint64_t)tile * kCzTile;
    double2 a[kCzItems];
    unsigned ball[kCzItems];
#pragma unroll
    for (int j = 0; j < kCzItems; ++j) {
        const uint64_t i = base + (uint64_t)j * kCzBlock + tid;
        bool keep = false;
        if (i < n) {
            a[j] = ia[i];
            if (SEL) {
                uint64_t k[K];
#pragma unroll
                for (int w = 0; w < K; ++w) k[w] = ik.w[w][i];
                keep = cond_ok<K>(k, ks.sel);
                if (ks.rf.width) {
                    const uint64_t v = fget<K>(k, ks.rf);
                    keep = keep && ks.lo <= v && v <= ks.hi;
                }
            } else {
                keep = sq_keep_amp(a[j].x, a[j].y, eps);
            }
        }
        ball[j] = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) s_cnt[j][warp] = __popc(ball[j]);
    }
    __syncthreads();
    // exclusive scan of the 64 (item-row, warp) counts in index order, by warp 0
    if (warp == 0) {
        unsigned v0 = s_cnt[(2 * lane) / (kCzBlock / 32)][(2 * lane) % (kCzBlock / 32)];
        unsigned v1 = s_cnt[(2 * lane + 1) / (kCzBlock / 32)][(2 * lane + 1) % (kCzBlock / 32)];
        unsigned sum = v0 + v1, inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (unsigned)o) inc += t;
        }
        const unsigned excl = inc - sum;
        const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
        s_cnt[(2 * lane) / (kCzBlock / 32)][(2 * lane) % (kCzBlock / 32)] = excl;
        s_cnt[(2 * lane + 1) / (kCzBlock / 32)][(2 * lane + 1) % (kCzBlock / 32)] = excl + v0;
        unsigned long long pre = lb_warp_exclusive(lb.status, tile, total, err);
        if (lane == 0) {
            s_prefix = pre;
            if (tile == ntiles - 1) *lb.total = pre + total;
        }
    }
    __syncthreads();
    const unsigned long long prefix = s_prefix;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kCzItems; ++j) {
        if (!((ball[j] >> lane) & 1u)) continue;
        const uint64_t i = base + (uint64_t)j * kCzBlock + tid;
        const uint64_t o = prefix + s_cnt[j][warp] + __popc(ball[j] & lt);
#pragma unroll
        for (int w = 0; w < K; ++w) ok.w[w][o] = ik.w[w][i];
        oa[o] = a[j];
    }
}

template <int K, bool SEL = false>
static void launch_cz(const Buffers& in, Buffers& out, uint64_t n, double eps, LookbackWs lb, long long nt,
                      const KeySelect* ks = nullptr) {
    ConstKeyPtrs ik;
    KeyPtrs okp;
    for (int w = 0; w < SQ_KMAX; ++w) {
        ik.w[w] = in.keys[w];
        okp.w[w] = out.keys[w];
    }
    KeySelect none;
    memset(&none, 0, sizeof(none));
    prof_begin(SEL ? "select_entries" : "clearzero");
    clearzero_kernel<K, SEL><<<(unsigned)nt, kCzBlock, 0, stream()>>>(ik, in.amp, okp, out.amp, n, eps, lb, nt,
                                                                    device_error_word(), ks ? *ks : none);
    prof_end((double)n * 16);  // every amplitude read; survivors added below
    SQ_CUDA(cudaGetLastError());
}

// Reads (and clears) the device error word. Not logged for replay: under
// capture it is skipped, and the flags raised by a replayed graph are read at
// the next synchronising call.
void check_device_error() {
    if (capturing()) return;
    unsigned v = 0;
    SQ_CUDA(cudaMemcpyAsync(&v, device_error_word(), 4, cudaMemcpyDeviceToHost, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    if (v) {
        SQ_CUDA(cudaMemsetAsync(device_error_word(), 0, 4, stream()));
        if (v & 32u) fail(SQ_ERR_INVALID, "a replayed graph saw other sizes than were recorded; the state is not valid");
        if (v & 64u) fail(SQ_ERR_INVALID, "angle: a register pair has no entry in the angle table");
        if (v & 8u) fail(SQ_ERR_INVALID, "lookup: a register value has no entry in the table");
        if (v & 4u) fail(SQ_ERR_INVALID, "batched Hadamard: an entry's digit count exceeds max_digits");
        if (v & 2u) fail(SQ_ERR_DEVICE_TIMEOUT, "hash grouping gave up (table full or a bounded wait expired)");
        fail(SQ_ERR_DEVICE_TIMEOUT, "a bounded device-side wait gave up (decoupled look-back)");
    }
}

// The poll limit of every bounded device wait (0 = kSpinLimit), word 1 of
// the device error block; stream-ordered, so launches queued before the
// call keep the limit they were queued with.
static unsigned g_wait_limit = 0;
void set_wait_limit(unsigned polls) {
    g_wait_limit = polls;
    SQ_CUDA(cudaMemcpyAsync(device_error_word() + 1, &g_wait_limit, 4, cudaMemcpyHostToDevice, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
}
unsigned wait_limit() { return g_wait_limit; }

// One ClearZero of 2 tiles of zero amplitudes, launched as one block whose
// ticket is preset to tile 1: it publishes its count and waits for tile 0's,
// which no block ever publishes. The wait gives up after `polls` polls,
// raises the error word and the block finishes (no survivors, nothing
// written); the host then reports SQ_ERR_DEVICE_TIMEOUT. Every index stays
// inside the 2-tile buffers.
void selftest_wait_timeout(unsigned polls) {
    if (polls == 0 || polls > (1u << 20)) fail(SQ_ERR_INVALID, "wait self-test: polls must be 1..2^20");
    check_device_error();  // start from a clean error word
    const uint64_t n = 2 * (uint64_t)kCzTile;
    char* buf = (char*)ws().get(WS_SCRATCH_TEST, n * 8 * 2 + n * 16 * 2);
    uint64_t* kin = (uint64_t*)buf;
    uint64_t* kout = kin + n;
    double2* ain = (double2*)(kout + n);
    double2* aout = ain + n;
    SQ_CUDA(cudaMemsetAsync(buf, 0, n * 8 * 2 + n * 16 * 2, stream()));
    LookbackWs lb = lookback_ws(2);
    const unsigned one = 1;
    SQ_CUDA(cudaMemcpyAsync(lb.counter, &one, 4, cudaMemcpyHostToDevice, stream()));
    const unsigned prev = g_wait_limit;
    set_wait_limit(polls);
    ConstKeyPtrs ik;
    KeyPtrs okp;
    memset(&ik, 0, sizeof(ik));
    memset(&okp, 0, sizeof(okp));
    ik.w[0] = kin;
    okp.w[0] = kout;
    KeySelect none;
    memset(&none, 0, sizeof(none));
    clearzero_kernel<1, false><<<1, kCzBlock, 0, stream()>>>(ik, ain, okp, aout, n, 1e-14, lb, 2,
                                                              device_error_word(), none);
    count_launch();
    const cudaError_t le = cudaGetLastError();
    set_wait_limit(prev);  // synchronizes: the block has finished
    SQ_CUDA(le);
    check_device_error();  // fails with SQ_ERR_DEVICE_TIMEOUT when the wait gave up
}

// Compacts `in` (n entries) into `out`, returns the survivor count. `out`
// must already hold n entries of capacity.
uint64_t compact_nonzero(const Buffers& in, Buffers& out, uint64_t n, double eps, uint32_t k) {
    if (n == 0) return 0;
    const long long nt = (long long)((n + kCzTile - 1) / kCzTile);
    LookbackWs lb = lookback_ws(nt);
    switch (k) {
        case 1: launch_cz<1>(in, out, n, eps, lb, nt); break;
        case 2: launch_cz<2>(in, out, n, eps, lb, nt); break;
        case 3: launch_cz<3>(in, out, n, eps, lb, nt); break;
        case 4: launch_cz<4>(in, out, n, eps, lb, nt); break;
        case 5: launch_cz<5>(in, out, n, eps, lb, nt); break;
        case 6: launch_cz<6>(in, out, n, eps, lb, nt); break;
        case 7: launch_cz<7>(in, out, n, eps, lb, nt); break;
        default: launch_cz<8>(in, out, n, eps, lb, nt); break;
    }
    unsigned long long total = 0;
    host_read(&total, lb.total, 8);
    check_device_error();  // synchronizes
    prof_add_bytes_last((double)total * (16.0 * k + 16));  // survivors: keys read + keys and amp written
    return total;
}

// PartialTraceSelect / PartialTraceSelectRange (partial_trace.cpp:148-225):
// keep the entries whose selected registers hold the selected values (or
// whose register lies in [lo, hi]), in order; then scale them by 1/sqrt(p), p
// their total probability. Returns that factor, or +inf when nothing is left.
double select_entries(State& s, const DCondSet& sel, Field rf, uint64_t lo, uint64_t hi) {
    drop_groups(s);
    sync_words(s);
    if (s.n == 0) return 0.0;
    const uint32_t k = regtable().k;
    ensure_buffers(s.spare, s.n, k, 0);
    KeySelect ks;
    memset(&ks, 0, sizeof(ks));
    ks.sel = sel;
    ks.rf = rf;
    ks.lo = lo;
    ks.hi = hi;
    const uint64_t n = s.n;
    const long long nt = (long long)((n + kCzTile - 1) / kCzTile);
    LookbackWs lb = lookback_ws(nt);
    switch (k) {
        case 1: launch_cz<1, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 2: launch_cz<2, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 3: launch_cz<3, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 4: launch_cz<4, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 5: launch_cz<5, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 6: launch_cz<6, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        case 7: launch_cz<7, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
        default: launch_cz<8, true>(s.live, s.spare, n, 0.0, lb, nt, &ks); break;
    }
    unsigned long long total = 0;
    host_read(&total, lb.total, 8);
    check_device_error();  // synchronizes
    prof_add_bytes_last((double)total * (16.0 * k + 16) - (double)n * 16 + (double)n * (8.0 * k + 16));
    swap_live_spare(s);
    s.n = total;
    if (total == 0) return std::numeric_limits<double>::infinity();
    const double p = norm_sq(s);
    if (p == 0.0) return std::numeric_limits<double>::infinity();
    const double f = 1.0 / std::sqrt(p);
    scale_amp(s, f);
    return f;
}

// ------------------------------------------------------------------ GetOutput
constexpr int kRedBlock = 256;
__global__ void __launch_bounds__(kRedBlock) norm_final_kernel(const double* __restrict__ partial, int m,
                                                               double* __restrict__ out);
__global__ void scale_kernel(double2* __restrict__ a, uint64_t n, double k);

// The dense index of a selected entry: its index fields concatenated, the
// first field in the lowest bits.
struct OutIndex {
    uint32_t n;
    uint32_t off[SQ_MAX_OUTPUT_FIELDS];
    Field f[SQ_MAX_OUTPUT_FIELDS];
};

// Scatter + partial probability sums in one pass. Dense indices are distinct
// because the selected registers and the index fields together cover every
// active register (checked on the host) and keys are unique.
template <int K>
__global__ void __launch_bounds__(kRedBlock) get_output_kernel(ConstKeyPtrs ik, const double2* __restrict__ ia,
                                                               uint64_t n, const __grid_constant__ DCondSet sel,
                                                               const __grid_constant__ OutIndex ix,
                                                               double2* __restrict__ out,
                                                               double* __restrict__ partial) {
    __shared__ double s[kRedBlock];
    double acc = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k[K];
#pragma unroll
        for (int w = 0; w < K; ++w) k[w] = ik.w[w][i];
        if (!cond_ok<K>(k, sel)) continue;
        uint64_t id = 0;
        for (uint32_t j = 0; j < ix.n; ++j) id |= fget<K>(k, ix.f[j]) << ix.off[j];
        const double2 v = ia[i];
        out[id] = v;
        acc += v.x * v.x + v.y * v.y;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kRedBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

template <int K>
static void launch_get_output(const State& s, const DCondSet& sel, const OutIndex& ix, double2* out,
                              double* part, int g) {
    ConstKeyPtrs ik;
    for (int w = 0; w < SQ_KMAX; ++w) ik.w[w] = s.live.keys[w];
    get_output_kernel<K><<<g, kRedBlock, 0, stream()>>>(ik, s.live.amp, s.n, sel, ix, out, part);
}

// GetOutput (qda_fundamental.cpp:123-166): the entries whose `sel` registers
// all hold 0 are placed in a dense vector of 2^(sum of index widths)
// amplitudes, at the concatenation of their index fields (main + anc_1 * 2^n +
// anc_4 * 2^(n+1) for the QDA read-out, qda_fundamental.h:640-645); every other
// slot is 0. p = the placed entries' total probability; the vector is scaled
// by 1/sqrt(p) unless |p - 1| < 1e-14 (the reference's epsilon) or p == 0.
// The state is left as it is. Returns p; the vector is copied into `host_out`
// (2 doubles per slot).
double get_output(State& s, const DCondSet& sel, const Field* fields, uint32_t nf, double* host_out) {
    sync_words(s);
    OutIndex ix;
    memset(&ix, 0, sizeof(ix));
    ix.n = nf;
    uint32_t bits = 0;
    for (uint32_t j = 0; j < nf; ++j) {
        ix.f[j] = fields[j];
        ix.off[j] = bits;
        bits += fields[j].width;
    }
    const uint64_t len = 1ull << bits;
    double2* out = (double2*)ws().get(WS_OUTPUT, len * 16);
    SQ_CUDA(cudaMemsetAsync(out, 0, len * 16, stream()));
    const int g = num_sms() * 4;
    double* part = (double*)ws().get(WS_REDUCE, (size_t)(g + 1) * 8);
    if (s.n == 0) {
        SQ_CUDA(cudaMemsetAsync(part + g, 0, 8, stream()));
    } else {
        const uint32_t k = regtable().k;
        prof_begin("get_output");
        switch (k) {
            case 1: launch_get_output<1>(s, sel, ix, out, part, g); break;
            case 2: launch_get_output<2>(s, sel, ix, out, part, g); break;
            case 3: launch_get_output<3>(s, sel, ix, out, part, g); break;
            case 4: launch_get_output<4>(s, sel, ix, out, part, g); break;
            case 5: launch_get_output<5>(s, sel, ix, out, part, g); break;
            case 6: launch_get_output<6>(s, sel, ix, out, part, g); break;
            case 7: launch_get_output<7>(s, sel, ix, out, part, g); break;
            default: launch_get_output<8>(s, sel, ix, out, part, g); break;
        }
        prof_end((double)s.n * (8.0 * k + 16));
        SQ_CUDA(cudaGetLastError());
        norm_final_kernel<<<1, kRedBlock, 0, stream()>>>(part, g, part + g);
        SQ_CUDA(cudaGetLastError());
    }
    double p = 0.0;
    host_read(&p, part + g, 8);
    if (!(std::fabs(p - 1.0) < 1e-14) && p != 0.0) {
        prof_begin("scale");
        scale_kernel<<<grid_for(len, 256), 256, 0, stream()>>>(out, len, 1.0 / std::sqrt(p));
        prof_end((double)len * 32);
        SQ_CUDA(cudaGetLastError());
    }
    host_read(host_out, out, len * 16);
    return p;
}

void clear_zero(State& s, double eps) {
    drop_groups(s);
    sync_words(s);
    if (s.n == 0) return;
    const uint32_t k = regtable().k;
    ensure_buffers(s.spare, s.n, k, 0);
    uint64_t m = compact_nonzero(s.live, s.spare, s.n, eps, k);
    swap_live_spare(s);
    s.n = m;
}

// ------------------------------------------------------------------ norm

__global__ void __launch_bounds__(kRedBlock) norm_partial_kernel(const double2* __restrict__ a, uint64_t n,
                                                                 double* __restrict__ partial) {
    __shared__ double s[kRedBlock];
    double acc = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double2 v = a[i];
        acc += v.x * v.x + v.y * v.y;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kRedBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void __launch_bounds__(kRedBlock) norm_final_kernel(const double* __restrict__ partial, int m,
                                                               double* __restrict__ out) {
    __shared__ double s[kRedBlock];
    double acc = 0.0;
    for (int i = threadIdx.x; i < m; i += kRedBlock) acc += partial[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kRedBlock / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

double norm_sq(const State& s) {
    if (s.n == 0) return 0.0;
    const int g = num_sms() * 4;
    double* part = (double*)ws().get(WS_REDUCE, (size_t)(g + 1) * 8);
    prof_begin("norm_partial");
    norm_partial_kernel<<<g, kRedBlock, 0, stream()>>>(s.live.amp, s.n, part);
    prof_end((double)s.n * 16);
    prof_begin("norm_final");
    norm_final_kernel<<<1, kRedBlock, 0, stream()>>>(part, g, part + g);
    prof_end((double)g * 8);
    SQ_CUDA(cudaGetLastError());
    double r = 0;
    host_read(&r, part + g, 8);
    return r;
}

__global__ void scale_kernel(double2* __restrict__ a, uint64_t n, double k) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 v = a[i];
        a[i] = make_double2(v.x * k, v.y * k);
    }
}

void scale_amp(State& s, double k) {
    if (s.n == 0) return;
    prof_begin("scale");
    scale_kernel<<<grid_for(s.n, 256), 256, 0, stream()>>>(s.live.amp, s.n, k);
    prof_end((double)s.n * 32);
    SQ_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------ ClearZero without allocation
// Some callers may not let a library allocate device memory on their behalf:
// programs that hand out all GPU memory from their own pre-planned pool or
// framework allocator, and latency-critical loops where a hidden cudaMalloc
// (which can synchronize the device) is not acceptable. For them this entry
// point compacts caller-owned arrays into caller-owned arrays and takes its
// only scratch, the decoupled look-back status, from one fixed device array
// declared below: 8 * (32 + 32768) bytes, enough for up to 2^26 entries.
// That array lives in every GPU that loads this library until the process
// exits, and all calls share it, so two calls whose work overlaps on the GPU
// (different streams, different host threads) race on it.
constexpr uint64_t kNoAllocMaxEntries = 1ull << 26;
constexpr uint64_t kNoAllocTiles = kNoAllocMaxEntries / kCzTile;
constexpr uint64_t kNoAllocHeaderWords = 32;  // [0] tile counter, [1] survivor total, [2] error word
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocHeaderWords + kNoAllocTiles];

constexpr int kNoAllocMaxDevices = 64;
static unsigned long long* g_noalloc_dev_ptr[kNoAllocMaxDevices] = {nullptr};

template <int K>
static void launch_cz_noalloc(const uint64_t* const* keys_in, const double* amps_in, uint64_t* const* keys_out,
                              double* amps_out, uint64_t n, double eps, unsigned long long* scratch, long long nt,
                              cudaStream_t s) {
    ConstKeyPtrs ik;
    KeyPtrs okp;
    for (int w = 0; w < SQ_KMAX; ++w) {
        ik.w[w] = w < K ? keys_in[w] : nullptr;
        okp.w[w] = w < K ? keys_out[w] : nullptr;
    }
    LookbackWs lb;
    lb.counter = (unsigned*)scratch;
    lb.total = scratch + 1;
    lb.status = scratch + kNoAllocHeaderWords;
    KeySelect none;
    memset(&none, 0, sizeof(none));
    clearzero_kernel<K, false><<<(unsigned)nt, kCzBlock, 0, s>>>(ik, (const double2*)amps_in, okp,
                                                                 (double2*)amps_out, n, eps, lb, nt,
                                                                 (unsigned*)(scratch + 2), none);
    count_launch();
}

}  // namespace sq

extern "C" int sq_clear_zero_noalloc(const uint64_t* const* keys_in, const double* amps_in, uint32_t k, uint64_t n,
                                     double eps, uint64_t* const* keys_out, double* amps_out, uint64_t* n_out,
                                     void* stream_handle) {
    using namespace sq;
    auto bad = [&](int code, const char* msg) {
        set_last_error(std::string("sq_clear_zero_noalloc: ") + msg);
        return code;
    };
    if (!n_out) return bad(SQ_ERR_INVALID, "null n_out");
    if (k < 1 || k > SQ_KMAX) return bad(SQ_ERR_INVALID, "k must be 1..SQ_MAX_KEY_WORDS");
    if (n > kNoAllocMaxEntries) return bad(SQ_ERR_CAPACITY, "n exceeds SQ_NOALLOC_MAX_ENTRIES (2^26)");
    if (n > 0 && (!keys_in || !amps_in || !keys_out || !amps_out)) return bad(SQ_ERR_INVALID, "null array");
    for (uint32_t w = 0; n > 0 && w < k; ++w)
        if (!keys_in[w] || !keys_out[w]) return bad(SQ_ERR_INVALID, "null key-word array");
    // outputs are written while other blocks still read inputs: no output
    // array may overlap an input array
    if (n > 0) {
        auto overlap = [](const void* a, uint64_t abytes, const void* b, uint64_t bbytes) {
            const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
            return x < y + bbytes && y < x + abytes;
        };
        for (uint32_t w = 0; w < k; ++w) {
            if (overlap(keys_out[w], n * 8, amps_in, n * 16)) return bad(SQ_ERR_INVALID, "an output overlaps an input");
            for (uint32_t v = 0; v < k; ++v)
                if (overlap(keys_out[w], n * 8, keys_in[v], n * 8)) return bad(SQ_ERR_INVALID, "an output overlaps an input");
        }
        if (overlap(amps_out, n * 16, amps_in, n * 16)) return bad(SQ_ERR_INVALID, "an output overlaps an input");
        for (uint32_t v = 0; v < k; ++v)
            if (overlap(amps_out, n * 16, keys_in[v], n * 8)) return bad(SQ_ERR_INVALID, "an output overlaps an input");
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return bad(SQ_ERR_CUDA, "no current CUDA device");
    // One-time set-up per device, with that device current: the host-side name
    // of a __device__ array is not its device address, so ask the runtime.
    if (!g_noalloc_dev_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return bad(SQ_ERR_CUDA, cudaGetErrorString(e));
        g_noalloc_dev_ptr[dev] = (unsigned long long*)p;
    }
    if (n == 0) {
        *n_out = 0;
        return SQ_OK;
    }
    cudaStream_t s = (cudaStream_t)stream_handle;
    unsigned long long* scratch = g_noalloc_dev_ptr[dev];
    const long long nt = (long long)((n + kCzTile - 1) / kCzTile);
    // the look-back status, tile counter, total and error word must start at zero
    if (cudaMemsetAsync(scratch, 0, (size_t)(kNoAllocHeaderWords + nt) * 8, s) != cudaSuccess)
        return bad(SQ_ERR_CUDA, "cudaMemsetAsync failed");
    switch (k) {
        case 1: launch_cz_noalloc<1>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 2: launch_cz_noalloc<2>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 3: launch_cz_noalloc<3>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 4: launch_cz_noalloc<4>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 5: launch_cz_noalloc<5>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 6: launch_cz_noalloc<6>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        case 7: launch_cz_noalloc<7>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
        default: launch_cz_noalloc<8>(keys_in, amps_in, keys_out, amps_out, n, eps, scratch, nt, s); break;
    }
    if (cudaGetLastError() != cudaSuccess) return bad(SQ_ERR_CUDA, "kernel launch failed");
    unsigned long long hdr[3] = {0, 0, 0};
    if (cudaMemcpyAsync(hdr, scratch, sizeof(hdr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return bad(SQ_ERR_CUDA, "reading the survivor count failed");
    if (hdr[2] & 0xffffffffull) return bad(SQ_ERR_DEVICE_TIMEOUT, "a bounded look-back wait gave up");
    *n_out = hdr[1];
    return SQ_OK;
}
