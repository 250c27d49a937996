// sq_core.cu — host runtime of the engine: errors, the process-global register
// table and its bit packing, the library stream, state buffers and the
// grow-only workspace.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

#include "sq_internal.cuh"

namespace sq {

[[noreturn]] void fail(int code, const std::string& msg) { throw Error{code, msg}; }

void cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        fail(SQ_ERR_OOM, std::string("device allocation failed: ") + what);
    }
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        fail(SQ_ERR_NO_DEVICE, std::string(cudaGetErrorString(e)) + " in " + what);
    fail(SQ_ERR_CUDA, std::string(cudaGetErrorString(e)) + " in " + what);
}

// ------------------------------------------------------------------ register table
static RegTable g_table;
RegTable& regtable() { return g_table; }

const RegEntry& RegTable::at(uint32_t id) const {
    if (id >= regs.size() || !regs[id].active) fail(SQ_ERR_INVALID, "register id " + std::to_string(id) + " is not active");
    return regs[id];
}

Field RegTable::field(uint32_t id) const {
    const RegEntry& r = at(id);
    Field f;
    f.word = (uint8_t)r.word;
    f.shift = (uint8_t)r.shift;
    f.width = (uint8_t)r.width;
    f.type = (uint8_t)r.type;
    return f;
}

// First fit over the existing words, lowest shift first; opens a new word
// when none has room. A register never straddles two words.
bool RegTable::alloc_bits(uint32_t width, uint32_t* word, uint32_t* shift) {
    if (width == 0) {
        *word = 0;
        *shift = 0;
        return true;
    }
    const uint64_t m = wmask(width);
    for (uint32_t w = 0; w < SQ_KMAX; ++w) {
        for (uint32_t s = 0; s + width <= 64; ++s) {
            if (((used[w] >> s) & m) == 0) {
                used[w] |= m << s;
                *word = w;
                *shift = s;
                if (w + 1 > k) k = w + 1;
                return true;
            }
        }
    }
    return false;
}

void RegTable::free_bits(uint32_t word, uint32_t shift, uint32_t width) {
    if (width == 0) return;
    used[word] &= ~(wmask(width) << shift);
}

uint32_t RegTable::add(uint32_t type, uint32_t width) {
    if (width > 64) fail(SQ_ERR_INVALID, "register width > 64");
    if (type > SQ_RATIONAL) fail(SQ_ERR_INVALID, "bad register type");
    uint32_t word, shift;
    if (!alloc_bits(width, &word, &shift))
        fail(SQ_ERR_CAPACITY, "packed key space exhausted (" + std::to_string(SQ_KMAX * 64) + " bits)");
    uint32_t id;
    if (!reusable.empty()) {
        id = reusable.back();
        reusable.pop_back();
    } else {
        if (regs.size() >= SQ_MAX_REGISTERS) {
            free_bits(word, shift, width);
            fail(SQ_ERR_CAPACITY, "more than SQ_MAX_REGISTERS registers");
        }
        regs.emplace_back();
        id = (uint32_t)regs.size() - 1;
    }
    RegEntry& e = regs[id];
    e.active = true;
    e.type = type;
    e.width = width;
    e.word = word;
    e.shift = shift;
    return id;
}

void RegTable::remove(uint32_t id) {
    if (id >= regs.size()) fail(SQ_ERR_INVALID, "register not found");
    if (!regs[id].active) fail(SQ_ERR_INVALID, "register is not activated");
    RegEntry& e = regs[id];
    free_bits(e.word, e.shift, e.width);
    e.active = false;
    reusable.push_back(id);
}

void RegTable::active_mask(uint64_t out[SQ_KMAX]) const {
    for (int w = 0; w < SQ_KMAX; ++w) out[w] = 0;
    for (const auto& r : regs)
        if (r.active && r.width) out[r.word] |= wmask(r.width) << r.shift;
}

DCondSet resolve_cond(const sq_cond* c) {
    DCondSet d;
    memset(&d, 0, sizeof(d));
    if (!c) return d;
    if (c->count > SQ_MAX_CONDITIONS) fail(SQ_ERR_INVALID, "too many conditions");
    d.n = c->count;
    for (uint32_t i = 0; i < c->count; ++i) {
        const sq_condition& q = c->c[i];
        if (q.kind > SQ_COND_VALUE) fail(SQ_ERR_INVALID, "bad condition kind");
        Field f = regtable().field(q.reg);
        d.c[i].kind = (uint8_t)q.kind;
        d.c[i].word = f.word;
        d.c[i].shift = f.shift;
        d.c[i].width = f.width;
        d.c[i].mask = wmask(f.width);
        d.c[i].param = q.param;
        if (q.kind == SQ_COND_BIT && q.param >= 64) fail(SQ_ERR_INVALID, "condition bit >= 64");
    }
    return d;
}

// ------------------------------------------------------------------ device / stream
static cudaStream_t g_stream = nullptr;
static int g_sms = 0;
static int g_device = -1;
static std::atomic<uint64_t> g_launches{0};

cudaStream_t stream() {
    if (!g_stream) {
        int dev = g_device < 0 ? 0 : g_device;
        SQ_CUDA(cudaSetDevice(dev));
        g_device = dev;
        SQ_CUDA(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
        cudaDeviceProp p;
        SQ_CUDA(cudaGetDeviceProperties(&p, dev));
        g_sms = p.multiProcessorCount;
        // Keep freed stream-ordered memory in the pool instead of returning it.
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    return g_stream;
}

void init_device(int device) {
    int n = 0;
    SQ_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) fail(SQ_ERR_INVALID, "device index out of range");
    if (g_stream && device != g_device) fail(SQ_ERR_INVALID, "library already bound to another device");
    g_device = device;
    (void)stream();
}

int num_sms() {
    if (!g_sms) (void)stream();
    return g_sms;
}

// Device allocations made by this library (cudaMalloc and cudaMallocAsync).
static std::atomic<uint64_t> g_dev_allocs{0};
uint64_t device_allocations() { return g_dev_allocs.load(); }

static unsigned int* g_err_word = nullptr;
unsigned int* device_error_word() {
    if (!g_err_word) {
        (void)stream();
        ++g_dev_allocs;
        SQ_CUDA(cudaMalloc(&g_err_word, 256));
        SQ_CUDA(cudaMemset(g_err_word, 0, 256));
    }
    return g_err_word;
}

void count_launch(int n) { g_launches += (uint64_t)n; }
uint64_t launches() { return g_launches.load(); }

// ------------------------------------------------------------------ per-kernel timing
// When enabled, every launch is bracketed by two CUDA events recorded on the
// library stream; collect() turns the pairs into per-kernel totals.
struct ProfRec {
    const char* name;
    cudaEvent_t a, b;
    double bytes;
};
static bool g_prof = false;
static std::vector<ProfRec> g_pending;
static std::vector<cudaEvent_t> g_event_pool;
static const char* g_open_name = nullptr;
static cudaEvent_t g_open_event = nullptr;
struct ProfStat {
    uint64_t count = 0;
    double ms = 0.0;
    double bytes = 0.0;
};
static std::vector<std::pair<std::string, ProfStat>> g_stats;

static cudaEvent_t take_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    SQ_CUDA(cudaEventCreate(&e));
    return e;
}

// ------------------------------------------------------------------ record / replay
// A sequence of operators is turned into a CUDA graph in two passes. The
// record pass runs it eagerly and logs every value the host reads back (group
// and output counts, histograms, flags). The capture pass issues the same
// calls under stream capture: each read returns the logged value instead of
// waiting for the device, and a one-block check compares it on the device with
// what the replayed kernels actually produced (error bit 5: the replay is
// invalid). Allocation, freeing and synchronisation are refused or skipped
// while capturing; the record pass has grown every buffer the sequence needs.
static ReplayState g_replay;
ReplayState& replay() { return g_replay; }
bool capturing() { return g_replay.mode == RP_CAPTURE; }

struct ReplayBytes {
    unsigned n;
    unsigned char b[kReplayReadMax];
};
__global__ void replay_check_kernel(const unsigned char* __restrict__ src, const __grid_constant__ ReplayBytes want,
                                    unsigned* err) {
    for (unsigned i = threadIdx.x; i < want.n; i += blockDim.x)
        if (src[i] != want.b[i]) atomicOr(err, 32u);
}

void host_read(void* dst, const void* src, size_t bytes) {
    ReplayState& r = g_replay;
    if (r.mode == RP_CAPTURE) {
        if (bytes > kReplayReadMax) fail(SQ_ERR_UNSUPPORTED, "capture: a read-back larger than a replay check holds");
        if (r.pos + bytes > r.log.size()) fail(SQ_ERR_INVALID, "capture: the operators differ from the recorded ones");
        memcpy(dst, r.log.data() + r.pos, bytes);
        r.pos += bytes;
        ReplayBytes w;
        w.n = (unsigned)bytes;
        memcpy(w.b, dst, bytes);
        replay_check_kernel<<<1, 128, 0, stream()>>>(static_cast<const unsigned char*>(src), w, device_error_word());
        SQ_CUDA(cudaGetLastError());
        count_launch();
        return;
    }
    SQ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    if (r.mode == RP_RECORD) {
        const unsigned char* b = static_cast<const unsigned char*>(dst);
        r.log.insert(r.log.end(), b, b + bytes);
    }
}

void host_decision(void* v, size_t bytes) {
    ReplayState& r = g_replay;
    if (r.mode == RP_CAPTURE) {
        if (r.pos + bytes > r.log.size()) fail(SQ_ERR_INVALID, "capture: the operators differ from the recorded ones");
        memcpy(v, r.log.data() + r.pos, bytes);
        r.pos += bytes;
    } else if (r.mode == RP_RECORD) {
        const unsigned char* b = static_cast<const unsigned char*>(v);
        r.log.insert(r.log.end(), b, b + bytes);
    }
}

__global__ void param_copy_kernel(unsigned char* __restrict__ dst, const __grid_constant__ ReplayBytes src) {
    for (unsigned i = threadIdx.x; i < src.n; i += blockDim.x) dst[i] = src.b[i];
}

void h2d_small(void* dst, const void* src, size_t bytes) {
    if (!capturing()) {
        SQ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream()));
        return;
    }
    // a captured copy from host memory would read it at every replay: the
    // bytes travel as a kernel parameter instead, baked into the graph
    if (bytes > kReplayReadMax) fail(SQ_ERR_UNSUPPORTED, "capture: a host-to-device copy larger than a parameter block");
    ReplayBytes b;
    b.n = (unsigned)bytes;
    memcpy(b.b, src, bytes);
    param_copy_kernel<<<1, 128, 0, stream()>>>(static_cast<unsigned char*>(dst), b);
    SQ_CUDA(cudaGetLastError());
    count_launch();
}

void replay_note_input(const void* p, size_t bytes) {
    ReplayState& r = g_replay;
    if (r.mode == RP_OFF || !p || !bytes) return;
    for (const auto& s : r.inputs)
        if (s.first == p) return;
    r.inputs.emplace_back(p, bytes);
}

__device__ __forceinline__ unsigned long long cs_mix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
// Sum over the span's 8-byte words (and its tail bytes) of a mix of the word,
// its position and the span's salt: independent of the summation order.
__global__ void checksum_kernel(const unsigned char* __restrict__ p, uint64_t bytes, unsigned long long salt,
                                unsigned long long* acc) {
    const uint64_t n8 = bytes / 8;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    const unsigned long long* w = reinterpret_cast<const unsigned long long*>(p);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += stride)
        local += cs_mix(w[i] ^ (i * 0x9e3779b97f4a7c15ull) ^ salt);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (uint64_t b = n8 * 8; b < bytes; ++b) local += cs_mix((unsigned long long)p[b] ^ (b << 8) ^ ~salt);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31u) == 0 && local) atomicAdd(acc, local);
}

// One device word read back through a mapped pinned word that a single
// thread stores, not by a device-to-host copy: a copy would wait in the copy
// engine's queue behind a bulk download of another state in flight (these
// reads come before every graph launch and table write, while the previous
// step's result is being downloaded). Synchronises the library stream.
__global__ void store_word_kernel(const unsigned long long* __restrict__ src, unsigned long long* dst) {
    *reinterpret_cast<volatile unsigned long long*>(dst) = *src;
}

uint64_t read_word_mapped(const unsigned long long* dev_word) {
    static unsigned long long* word_host = nullptr;
    static unsigned long long* word_dev = nullptr;
    if (capturing()) fail(SQ_ERR_UNSUPPORTED, "capture: a value would be read back");
    if (!word_host) {
        SQ_CUDA(cudaHostAlloc((void**)&word_host, 64, cudaHostAllocMapped));
        SQ_CUDA(cudaHostGetDevicePointer((void**)&word_dev, word_host, 0));
    }
    cudaStream_t st = stream();
    store_word_kernel<<<1, 1, 0, st>>>(dev_word, word_dev);
    SQ_CUDA(cudaGetLastError());
    SQ_CUDA(cudaStreamSynchronize(st));
    return *reinterpret_cast<volatile unsigned long long*>(word_host);
}

uint64_t device_checksum(const std::vector<std::pair<const void*, size_t>>& spans) {
    cudaStream_t st = stream();
    unsigned long long* acc = (unsigned long long*)dev_alloc(8);
    SQ_CUDA(cudaMemsetAsync(acc, 0, 8, st));
    unsigned long long salt = 0x2545f4914f6cdd1dull;
    for (const auto& s : spans) {
        salt = salt * 6364136223846793005ull + 1442695040888963407ull;
        if (!s.first || !s.second) continue;
        if (reinterpret_cast<uintptr_t>(s.first) & 7) fail(SQ_ERR_INVALID, "checksum: unaligned span");
        checksum_kernel<<<grid_for(s.second / 8 + 1, 256), 256, 0, st>>>(static_cast<const unsigned char*>(s.first),
                                                                        s.second, salt, acc);
        SQ_CUDA(cudaGetLastError());
    }
    const uint64_t h = read_word_mapped(acc);
    dev_free(acc);
    return h;
}

void sync_library_stream() {
    if (!capturing()) SQ_CUDA(cudaStreamSynchronize(stream()));
}

void prof_begin(const char* name) {
    if (!g_prof || capturing()) return;
    g_open_name = name;
    g_open_event = take_event();
    SQ_CUDA(cudaEventRecord(g_open_event, stream()));
}

void prof_end(double alg_bytes) {
    count_launch();
    if (!g_prof || !g_open_event || capturing()) return;
    cudaEvent_t b = take_event();
    SQ_CUDA(cudaEventRecord(b, stream()));
    g_pending.push_back(ProfRec{g_open_name, g_open_event, b, alg_bytes});
    g_open_event = nullptr;
}

void prof_add_bytes_last(double alg_bytes) {
    if (g_prof && !g_pending.empty()) g_pending.back().bytes += alg_bytes;
}

void prof_collect() {
    if (g_pending.empty()) return;
    SQ_CUDA(cudaStreamSynchronize(stream()));
    for (auto& r : g_pending) {
        float ms = 0.f;
        SQ_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto it = std::find_if(g_stats.begin(), g_stats.end(), [&](const auto& kv) { return kv.first == r.name; });
        if (it == g_stats.end()) {
            g_stats.emplace_back(r.name, ProfStat{});
            it = g_stats.end() - 1;
        }
        it->second.count += 1;
        it->second.ms += ms;
        it->second.bytes += r.bytes;
        g_event_pool.push_back(r.a);
        g_event_pool.push_back(r.b);
    }
    g_pending.clear();
}

void prof_enable(bool on) {
    prof_collect();
    g_prof = on;
}
void prof_reset() {
    prof_collect();
    g_stats.clear();
}
size_t prof_count() { return g_stats.size(); }
const char* prof_name(size_t i) { return g_stats[i].first.c_str(); }
uint64_t prof_launches(size_t i) { return g_stats[i].second.count; }
double prof_ms(size_t i) { return g_stats[i].second.ms; }
double prof_bytes(size_t i) { return g_stats[i].second.bytes; }

void* dev_alloc(size_t bytes) {
    if (capturing()) fail(SQ_ERR_UNSUPPORTED, "capture: a buffer would grow; the record pass must run the same operators");
    if (bytes == 0) bytes = 16;
    void* p = nullptr;
    ++g_dev_allocs;
    cudaError_t e = cudaMallocAsync(&p, bytes, stream());
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        fail(SQ_ERR_OOM, "cudaMallocAsync of " + std::to_string(bytes) + " bytes failed");
    }
    return p;
}

void dev_free(void* p) {
    if (p && capturing()) fail(SQ_ERR_UNSUPPORTED, "capture: a buffer would be freed");
    if (p) SQ_CUDA(cudaFreeAsync(p, stream()));
}

// ------------------------------------------------------------------ buffers
void free_buffers(Buffers& b) {
    for (int w = 0; w < SQ_KMAX; ++w) {
        dev_free(b.keys[w]);
        b.keys[w] = nullptr;
    }
    dev_free(b.amp);
    b.amp = nullptr;
    b.cap = 0;
    b.kalloc = 0;
}

// Copies by the SMs over the host link, between device memory and mapped
// pinned host memory (either side): a few blocks storing into host memory
// (asynchronous downloads) or a full grid loading from it (uploads). A bulk
// copy-engine transfer delays every small device-to-host read queued after it
// (the count reads of the split operators wait behind it: 155 us instead of
// 20 us each), and on some systems an upload waits behind a download in
// flight; so downloads into pinned memory default to 12 blocks storing (about
// 150 GB/s of the link's 190, leaving the SMs and the small reads to the work
// they overlap), and uploads from pinned memory are loaded by the SMs, which
// leaves the copy engine to a download that overlaps later work.
constexpr int kD2HSegs = SQ_KMAX + 2;
constexpr int kD2HBlocks = 12;
struct D2HJobs {
    const uint2* src[kD2HSegs];
    uint2* dst[kD2HSegs];
    uint64_t n8[kD2HSegs];  // 8-byte units
    int n;
};

__global__ void __launch_bounds__(512) link_copy_kernel(const __grid_constant__ D2HJobs j) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (int s = 0; s < j.n; ++s) {
        const uint64_t n8 = j.n8[s];
        const bool v16 = ((reinterpret_cast<uintptr_t>(j.src[s]) | reinterpret_cast<uintptr_t>(j.dst[s])) & 15) == 0;
        if (v16) {
            const uint4* src = reinterpret_cast<const uint4*>(j.src[s]);
            uint4* dst = reinterpret_cast<uint4*>(j.dst[s]);
            const uint64_t n16 = n8 >> 1;
            for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
            if ((n8 & 1) && blockIdx.x == 0 && threadIdx.x == 0) j.dst[s][n8 - 1] = j.src[s][n8 - 1];
        } else {
            for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += stride)
                j.dst[s][i] = j.src[s][i];
        }
    }
}

// The device alias of mapped pinned host memory (8-byte aligned start and
// size), or null for any other memory.
static void* mapped_alias(const void* host, size_t bytes) {
    cudaPointerAttributes at;
    const cudaError_t pe = cudaPointerGetAttributes(&at, host);
    if (pe != cudaSuccess) {
        (void)cudaGetLastError();  // that query's own error only
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
    if ((reinterpret_cast<uintptr_t>(host) & 7) != 0 || bytes % 8 != 0) return nullptr;
    return at.devicePointer;
}

void copy_h2d_async(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    cudaStream_t st = stream();
    const void* alias = (reinterpret_cast<uintptr_t>(dst) & 7) == 0 ? mapped_alias(src, bytes) : nullptr;
    if (!alias) {
        SQ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
        return;
    }
    D2HJobs j;
    memset(&j, 0, sizeof(j));
    j.src[0] = static_cast<const uint2*>(alias);
    j.dst[0] = static_cast<uint2*>(dst);
    j.n8[0] = bytes / 8;
    j.n = 1;
    const uint64_t blocks = std::min<uint64_t>((bytes / 16 + 511) / 512, (uint64_t)num_sms() * 2);
    link_copy_kernel<<<(unsigned)std::max<uint64_t>(blocks, 1), 512, 0, st>>>(j);
    SQ_CUDA(cudaGetLastError());
}

namespace {
constexpr int kCopyStreams = 4;
cudaStream_t g_copy[kCopyStreams] = {nullptr};
cudaEvent_t g_copy_ev[kCopyStreams + 1] = {nullptr};
}  // namespace

void parallel_copy(const CopyJob* jobs, int n, cudaMemcpyKind kind) {
    cudaStream_t st = stream();
    if (!g_copy[0]) {
        for (int i = 0; i < kCopyStreams; ++i) {
            SQ_CUDA(cudaStreamCreateWithFlags(&g_copy[i], cudaStreamNonBlocking));
            SQ_CUDA(cudaEventCreateWithFlags(&g_copy_ev[i], cudaEventDisableTiming));
        }
        SQ_CUDA(cudaEventCreateWithFlags(&g_copy_ev[kCopyStreams], cudaEventDisableTiming));
    }
    std::vector<CopyJob> rest;
    if (kind == cudaMemcpyHostToDevice) {  // uploads from mapped pinned memory: by the SMs
        for (int j = 0; j < n; ++j) {
            if (jobs[j].bytes && mapped_alias(jobs[j].src, jobs[j].bytes) &&
                (reinterpret_cast<uintptr_t>(jobs[j].dst) & 7) == 0)
                copy_h2d_async(jobs[j].dst, jobs[j].src, jobs[j].bytes);
            else
                rest.push_back(jobs[j]);
        }
        jobs = rest.data();
        n = (int)rest.size();
    }
    size_t total = 0;
    for (int j = 0; j < n; ++j) total += jobs[j].bytes;
    if (total < (8u << 20)) {  // small: one stream is as fast
        for (int j = 0; j < n; ++j)
            if (jobs[j].bytes) SQ_CUDA(cudaMemcpyAsync(jobs[j].dst, jobs[j].src, jobs[j].bytes, kind, st));
        SQ_CUDA(cudaStreamSynchronize(st));
        return;
    }
    // every copy stream starts after the library stream's queued work
    SQ_CUDA(cudaEventRecord(g_copy_ev[kCopyStreams], st));
    for (int i = 0; i < kCopyStreams; ++i) SQ_CUDA(cudaStreamWaitEvent(g_copy[i], g_copy_ev[kCopyStreams], 0));
    // chunks of about total / (2 * streams) bytes, round-robin over the streams
    const size_t chunk = std::max<size_t>((total / (2 * kCopyStreams) + 4095) & ~size_t(4095), 1u << 20);
    int next = 0;
    for (int j = 0; j < n; ++j) {
        for (size_t off = 0; off < jobs[j].bytes; off += chunk) {
            const size_t b = std::min(chunk, jobs[j].bytes - off);
            SQ_CUDA(cudaMemcpyAsync((char*)jobs[j].dst + off, (const char*)jobs[j].src + off, b, kind,
                                    g_copy[next]));
            next = (next + 1) % kCopyStreams;
        }
    }
    // the library stream waits for the copies too (later work may reuse the buffers)
    for (int i = 0; i < kCopyStreams; ++i) {
        SQ_CUDA(cudaEventRecord(g_copy_ev[i], g_copy[i]));
        SQ_CUDA(cudaStreamWaitEvent(st, g_copy_ev[i], 0));
    }
    SQ_CUDA(cudaStreamSynchronize(st));
}

// Low-priority download streams: copy-engine downloads are cut into chunks
// spread over these, so that several copy engines share a large transfer.
constexpr int kAsyncStreams = 4;
static cudaStream_t g_async[kAsyncStreams] = {nullptr};
static cudaEvent_t g_async_ev[kAsyncStreams + 1] = {nullptr};
static int g_d2h_engine = SQ_DOWNLOAD_SM_STORES;

void set_d2h_engine(int engine) {
    if (engine != SQ_DOWNLOAD_SM_STORES && engine != SQ_DOWNLOAD_COPY_ENGINE && engine != SQ_DOWNLOAD_SPLIT)
        fail(SQ_ERR_INVALID, "download engine must be SQ_DOWNLOAD_SM_STORES, SQ_DOWNLOAD_COPY_ENGINE or SQ_DOWNLOAD_SPLIT");
    g_d2h_engine = engine;
}

static int env_int(const char* name, int lo, int hi, int dflt) {
    const char* e = getenv(name);
    const int v = e ? atoi(e) : 0;
    return e && v >= lo && v <= hi ? v : dflt;
}

void async_copy_d2h(const CopyJob* jobs, int n, cudaEvent_t done) {
    cudaStream_t st = stream();
    static const int nstreams = env_int("SPARQ_D2H_STREAMS", 1, kAsyncStreams - 1, 1);
    static const int blocks = env_int("SPARQ_D2H_BLOCKS", 1, 1024, kD2HBlocks);
    if (!g_async[0]) {
        int least = 0, greatest = 0;
        SQ_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        for (int i = 0; i < kAsyncStreams; ++i)
            SQ_CUDA(cudaStreamCreateWithPriority(&g_async[i], cudaStreamNonBlocking, least));
        for (int i = 0; i <= kAsyncStreams; ++i)
            SQ_CUDA(cudaEventCreateWithFlags(&g_async_ev[i], cudaEventDisableTiming));
    }
    if (n > kD2HSegs) fail(SQ_ERR_INVALID, "asynchronous download: too many arrays");
    // stream 0 runs the store kernel, streams 1..nstreams the copy-engine chunks
    const int used = 1 + nstreams;
    // after the library stream's queued work (the state's last writer)
    SQ_CUDA(cudaEventRecord(g_async_ev[kAsyncStreams], st));
    for (int i = 0; i < used; ++i) SQ_CUDA(cudaStreamWaitEvent(g_async[i], g_async_ev[kAsyncStreams], 0));
    D2HJobs kj;
    memset(&kj, 0, sizeof(kj));
    size_t total = 0;
    for (int i = 0; i < n; ++i) total += jobs[i].bytes;
    const size_t chunk = std::max<size_t>((total / (2 * nstreams) + 4095) & ~size_t(4095), 1u << 20);
    int next = 0;
    auto by_copy_engine = [&](char* dst, const char* src, size_t bytes) {
        for (size_t off = 0; off < bytes; off += chunk) {
            const size_t b = std::min(chunk, bytes - off);
            SQ_CUDA(cudaMemcpyAsync(dst + off, src + off, b, cudaMemcpyDeviceToHost, g_async[1 + next]));
            next = (next + 1) % nstreams;
        }
    };
    for (int i = 0; i < n; ++i) {
        if (jobs[i].bytes == 0) continue;
        void* alias = g_d2h_engine != SQ_DOWNLOAD_COPY_ENGINE ? mapped_alias(jobs[i].dst, jobs[i].bytes) : nullptr;
        // split mode: the first half (a multiple of 16 bytes) by the SMs, the rest by the copy engine
        const size_t sm_bytes = !alias ? 0
                                : g_d2h_engine == SQ_DOWNLOAD_SPLIT ? (jobs[i].bytes / 2) & ~size_t(15)
                                                                    : jobs[i].bytes;
        if (sm_bytes) {
            kj.src[kj.n] = static_cast<const uint2*>(jobs[i].src);
            kj.dst[kj.n] = static_cast<uint2*>(alias);
            kj.n8[kj.n] = sm_bytes / 8;
            ++kj.n;
        }
        if (sm_bytes < jobs[i].bytes)
            by_copy_engine((char*)jobs[i].dst + sm_bytes, (const char*)jobs[i].src + sm_bytes,
                           jobs[i].bytes - sm_bytes);
    }
    if (kj.n) {
        link_copy_kernel<<<blocks, 512, 0, g_async[0]>>>(kj);
        SQ_CUDA(cudaGetLastError());
    }
    // join the copy streams into the first, whose event marks the end
    for (int i = 1; i < used; ++i) {
        SQ_CUDA(cudaEventRecord(g_async_ev[i], g_async[i]));
        SQ_CUDA(cudaStreamWaitEvent(g_async[0], g_async_ev[i], 0));
    }
    SQ_CUDA(cudaEventRecord(done, g_async[0]));
}

void sync_async_copies() {
    for (int i = 0; i < kAsyncStreams; ++i)
        if (g_async[i]) SQ_CUDA(cudaStreamSynchronize(g_async[i]));
}

void free_group_cache(GroupCache& c) {
    for (int i = 0; i < 2; ++i) {
        dev_free(c.start[i]);
        dev_free(c.cnt[i]);
        c.start[i] = nullptr;
        c.cnt[i] = nullptr;
        c.cap[i] = 0;
    }
    c.valid = false;
}

void ensure_buffers(Buffers& b, uint64_t cap, uint32_t k, uint64_t keep) {
    if (k > SQ_KMAX) fail(SQ_ERR_CAPACITY, "too many key words");
    if (keep > b.cap) keep = b.cap;
    if (cap <= b.cap) {
        // capacity fine; maybe add words
        for (uint32_t w = b.kalloc; w < k; ++w) {
            b.keys[w] = (uint64_t*)dev_alloc(b.cap * 8);
            SQ_CUDA(cudaMemsetAsync(b.keys[w], 0, b.cap * 8, stream()));
        }
        if (k > b.kalloc) b.kalloc = k;
        return;
    }
    uint64_t newcap = std::max<uint64_t>(cap, b.cap + b.cap / 2);
    newcap = std::max<uint64_t>(newcap, 1024);
    uint32_t kk = std::max(k, b.kalloc);
    Buffers nb;
    nb.cap = newcap;
    nb.kalloc = kk;
    for (uint32_t w = 0; w < kk; ++w) {
        nb.keys[w] = (uint64_t*)dev_alloc(newcap * 8);
        if (w < b.kalloc && keep) {
            SQ_CUDA(cudaMemcpyAsync(nb.keys[w], b.keys[w], keep * 8, cudaMemcpyDeviceToDevice, stream()));
            SQ_CUDA(cudaMemsetAsync(nb.keys[w] + keep, 0, (newcap - keep) * 8, stream()));
        } else {
            SQ_CUDA(cudaMemsetAsync(nb.keys[w], 0, newcap * 8, stream()));
        }
    }
    nb.amp = (double2*)dev_alloc(newcap * 16);
    if (keep && b.amp) SQ_CUDA(cudaMemcpyAsync(nb.amp, b.amp, keep * 16, cudaMemcpyDeviceToDevice, stream()));
    free_buffers(b);
    b = nb;
}

void sync_words(State& s) {
    uint32_t k = regtable().k;
    if (s.live.kalloc < k) ensure_buffers(s.live, s.live.cap, k, s.n);
}

void swap_live_spare(State& s) {
    std::swap(s.live, s.spare);
    ++s.swaps;
}

// ------------------------------------------------------------------ workspace
static Workspace g_ws;
Workspace& ws() { return g_ws; }

void* Workspace::get(int slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (sz[slot] < bytes) {
        dev_free(p[slot]);
        size_t n = std::max(bytes, sz[slot] + sz[slot] / 2);
        n = (n + 255) & ~size_t(255);
        p[slot] = dev_alloc(n);
        sz[slot] = n;
    }
    return p[slot];
}

}  // namespace sq
