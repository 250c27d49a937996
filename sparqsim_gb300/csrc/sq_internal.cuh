// sq_internal.cuh — shared device/host internals of the GB300 sparse-state engine.
//
// Data layout in HBM (per state):
//   keys[w][i]  uint64, w < K: word-major arrays; each active register is a bit
//               field (word, shift, width) inside one word.
//   amp[i]      double2 (re, im), 16-byte aligned.
// A state owns two such buffer sets (live + spare) so split/merge operators
// write their output out of place and swap.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "sparq_gb300.h"

#define SQ_KMAX SQ_MAX_KEY_WORDS

namespace sq {

// ------------------------------------------------------------------ errors
struct Error {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const std::string& msg);
// Message returned by sq_last_error() on this thread.
void set_last_error(const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define SQ_CUDA(x) ::sq::cuda_check((x), #x)

// Device word raised by bounded device-side waits (bit 0: a look-back gave
// up). Allocated once per process; kernels that wait receive its address.
unsigned int* device_error_word();

// ------------------------------------------------------------------ registers
// Prune predicate of ClearZero and of every split: keep unless
// x*x + y*y < eps, evaluated in FP64 with that exact rounding. The result is
// first decided from the exponent fields where they settle it (FP64 runs at a
// small fraction of the integer rate on this part, and most amplitudes are far
// from the threshold): with M = max(|x|,|y|) of biased exponent e,
// M >= 2^(e-1023) gives fl(x*x + y*y) >= 2^(2e-2046), and M < 2^(e-1022) gives
// fl(x*x + y*y) <= 2^(2e-2043); eps lies in [2^(ee-1023), 2^(ee-1022)).
#ifdef __CUDACC__
// The FP64 evaluation sits in a function of its own so that the compiler
// branches around it instead of issuing it, predicated off, for every entry.
static __device__ __noinline__ bool sq_keep_amp_fp64(double x, double y, double eps) {
    return !(x * x + y * y < eps);
}
__device__ __forceinline__ bool sq_keep_amp(double x, double y, double eps) {
    const int ex = (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
    const int ey = (int)((unsigned long long)__double_as_longlong(y) >> 52) & 0x7ff;
    const int e = ex > ey ? ex : ey;
    const long long eb = __double_as_longlong(eps);
    const int ee = (int)(eb >> 52) & 0x7ff;
    if (2 * e >= ee + 1024) return true;              // also inf/NaN amplitudes, as the formula does
    if (eb > 0 && ee > 0 && 2 * e < ee + 1020) return false;  // eps positive and normal
    return sq_keep_amp_fp64(x, y, eps);
}
#endif

struct Field {
    uint8_t word;
    uint8_t shift;
    uint8_t width;
    uint8_t type;
};

__host__ __device__ __forceinline__ uint64_t wmask(unsigned w) {
    return w >= 64 ? ~0ull : ((1ull << w) - 1ull);
}

struct RegEntry {
    bool active = false;
    uint32_t type = 0;
    uint32_t width = 0;
    uint32_t word = 0;
    uint32_t shift = 0;
};

// Process-global register table (mirrors System::name_register_map plus the
// packing of each register into a key word).
struct RegTable {
    std::vector<RegEntry> regs;
    std::vector<uint32_t> reusable;   // ids freed by remove, reused LIFO
    uint64_t used[SQ_KMAX] = {0};     // allocated bits per word
    uint32_t k = 1;                   // key words in use (>= 1)
    double clearzero_eps = 1e-14;

    Field field(uint32_t id) const;
    const RegEntry& at(uint32_t id) const;
    uint32_t add(uint32_t type, uint32_t width);
    void remove(uint32_t id);
    bool alloc_bits(uint32_t width, uint32_t* word, uint32_t* shift);
    void free_bits(uint32_t word, uint32_t shift, uint32_t width);
    void active_mask(uint64_t out[SQ_KMAX]) const;
};
RegTable& regtable();

// ------------------------------------------------------------------ conditions
struct DCond {
    uint8_t kind;
    uint8_t word;
    uint8_t shift;
    uint8_t width;
    uint32_t pad;
    uint64_t param;
    uint64_t mask;  // wmask(width), computed on the host
};
struct DCondSet {
    uint32_t n;
    uint32_t pad;
    DCond c[SQ_MAX_CONDITIONS];
};

template <int K>
__device__ __forceinline__ uint64_t kword(const uint64_t (&k)[K], unsigned w) {
    uint64_t r = 0;
#pragma unroll
    for (int i = 0; i < K; ++i)
        if ((unsigned)i == w) r = k[i];
    return r;
}
template <int K>
__device__ __forceinline__ void kword_set(uint64_t (&k)[K], unsigned w, uint64_t v) {
#pragma unroll
    for (int i = 0; i < K; ++i)
        if ((unsigned)i == w) k[i] = v;
}
template <int K>
__device__ __forceinline__ uint64_t fget(const uint64_t (&k)[K], Field f) {
    return (kword<K>(k, f.word) >> f.shift) & wmask(f.width);
}
template <int K>
__device__ __forceinline__ void fset(uint64_t (&k)[K], Field f, uint64_t v) {
    const uint64_t m = wmask(f.width) << f.shift;
    const uint64_t w = kword<K>(k, f.word);
    kword_set<K>(k, f.word, (w & ~m) | ((v << f.shift) & m));
}

template <int K>
__device__ __forceinline__ bool cond_ok(const uint64_t (&k)[K], const DCondSet& cs) {
    bool ok = true;
    for (uint32_t i = 0; i < cs.n; ++i) {
        const DCond& c = cs.c[i];
        const uint64_t v = (kword<K>(k, c.word) >> c.shift) & c.mask;
        switch (c.kind) {
            case SQ_COND_NONZERO: ok = ok && (v != 0); break;
            case SQ_COND_ALL_ONES: ok = ok && (v == c.mask); break;
            case SQ_COND_BIT: ok = ok && (c.param < 64) && ((v >> c.param) & 1ull); break;
            default: ok = ok && (v == c.param); break;
        }
    }
    return ok;
}

DCondSet resolve_cond(const sq_cond* c);

// ------------------------------------------------------------------ QRAM
struct QramTable {
    void* dev = nullptr;
    uint32_t elem_bytes = 8;
    uint32_t address_size = 0;
    uint32_t data_size = 0;
    uint64_t n_words = 0;
    uint64_t max_word = 0;  // OR of every word: the highest bit any word uses
    // a lookup table (SQ_OP_LOOKUP_XOR): u64 words [dense (dense_len) |
    // sparse keys (n_sparse) | sparse words (n_sparse)]
    bool lookup = false;
    uint64_t dense_len = 0;
    uint64_t n_sparse = 0;
    // an angle table (SQ_OP_ANGLE_XOR): slots of 3 u64 words (lhs, rhs,
    // word), both keys ~0 when empty; slot count pair_mask + 1
    int pair_kind = -1;
    uint32_t pair_w[3] = {0, 0, 0};
    uint64_t pair_mask = 0;
    uint32_t pair_probe = 0;  // longest insertion probe: lookups stop after it
};

// The slot of an angle table's (lhs, rhs) pair, the same on host and device.
__host__ __device__ __forceinline__ uint64_t pair_slot_hash(uint64_t a, uint64_t b) {
    uint64_t z = a * 0x9e3779b97f4a7c15ull ^ (b + 0x632be59bd9b4e019ull + (a << 6) + (a >> 2));
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// ------------------------------------------------------------------ state
struct Buffers {
    uint64_t* keys[SQ_KMAX] = {nullptr};
    double2* amp = nullptr;
    uint64_t cap = 0;
    uint32_t kalloc = 0;
};

// Group ranges left by the last Hadamard split: the entries of each group of
// that operation's output (equal keys outside the low `target.width` bits of
// `target`) sit in one contiguous range [start[g], start[g] + cnt[g]). A
// following split on the same bits takes its groups from here instead of
// grouping again. Anything that changes key values or entry positions drops
// the ranges (drop_groups).
struct GroupCache {
    bool valid = false;
    Field target{};
    Field varw{};                              // batched width register (width 0: none)
    uint64_t gmask[SQ_KMAX] = {0};
    uint64_t G = 0;
    int cur = 0;                               // the valid set; the other one is written next
    unsigned long long* start[2] = {nullptr, nullptr};
    unsigned* cnt[2] = {nullptr, nullptr};
    uint64_t cap[2] = {0, 0};
};

struct State {
    Buffers live;
    Buffers spare;
    uint64_t n = 0;
    GroupCache groups;
    uint64_t swaps = 0;              // live/spare exchanges so far (graphs need an even number per sequence)
    cudaEvent_t d2h_done = nullptr;  // recorded when the last asynchronous download finished reading
    bool d2h_pending = false;        // the library stream has not been made to wait for it yet
};
inline void drop_groups(State& s) { s.groups.valid = false; }
void free_group_cache(GroupCache& c);
double select_entries(State& s, const DCondSet& sel, Field rf, uint64_t lo, uint64_t hi);
double get_output(State& s, const DCondSet& sel, const Field* fields, uint32_t nf, double* host_out);
// Host <-> device copies of several arrays, split into chunks spread over a
// few copy streams (one copy engine does not reach the host link's rate);
// ordered after all work queued on the library stream, and complete on
// return. `dirs` gives cudaMemcpyDeviceToHost or HostToDevice per copy.
struct CopyJob {
    void* dst;
    const void* src;
    size_t bytes;
};
void parallel_copy(const CopyJob* jobs, int n, cudaMemcpyKind kind);
// The same device-to-host copies on their own streams, returning at once;
// `done` is recorded when every copy has finished. The host memory must stay
// valid, and the device memory unwritten, until then.
void async_copy_d2h(const CopyJob* jobs, int n, cudaEvent_t done);
// Blocks until every asynchronous download has finished.
void sync_async_copies();
uint64_t read_word_mapped(const unsigned long long* dev_word);
// Host-to-device copy on the library stream, by the SMs from mapped pinned
// memory, else by the copy engine.
void copy_h2d_async(void* dst, const void* src, size_t bytes);
void set_d2h_engine(int engine);
// Copy a host table of 64-bit words to the device at the narrowest width (2,
// 4 or 8 bytes) that holds every word; eb_guess is tried first.
void* qram_upload(const uint64_t* host_words, uint64_t n, uint32_t eb_guess, uint32_t* eb_out, uint64_t* all_out);
// New words for an existing table (same size), written in place at its stored
// width; returns the OR of the new words.
uint64_t qram_rewrite(QramTable& t, const uint64_t* host_words);

struct KeyPtrs {
    uint64_t* w[SQ_KMAX];
};
struct ConstKeyPtrs {
    const uint64_t* w[SQ_KMAX];
};

cudaStream_t stream();
int num_sms();
void count_launch(int n = 1);
// Bracket one kernel launch: prof_begin(name); kernel<<<...>>>(...); prof_end(bytes);
// prof_end() also counts the launch; `bytes` is the launch's algorithmic
// (compulsory) HBM traffic, used for the roofline.
// Record / replay of host decisions (graph capture of operator sequences).
enum ReplayMode { RP_OFF = 0, RP_RECORD = 1, RP_CAPTURE = 2 };
constexpr size_t kReplayReadMax = 8192;
struct ReplayState {
    int mode = RP_OFF;
    std::vector<unsigned char> log;
    size_t pos = 0;
    std::vector<std::pair<const void*, size_t>> inputs;  // device tables the recorded operators read
};
ReplayState& replay();
bool capturing();
// `bytes` device bytes into host memory, after the work queued before them:
// a read-back (logged when recording); under capture the logged bytes, with a
// device-side check that the replay produces the same.
void host_read(void* dst, const void* src, size_t bytes);
// A host-side choice (autotuning, timing-dependent paths): logged when
// recording, taken from the log under capture.
void host_decision(void* v, size_t bytes);
// A small host-to-device copy (parameters, counters' initial values) on the
// library stream; under capture the bytes go into the graph as a kernel
// parameter (at most kReplayReadMax bytes).
void h2d_small(void* dst, const void* src, size_t bytes);
// Notes a device table read by an operator being recorded or captured (a
// replay is only allowed when its content is unchanged).
void replay_note_input(const void* p, size_t bytes);
// Order-independent 64-bit checksum of device byte spans (synchronises).
uint64_t device_checksum(const std::vector<std::pair<const void*, size_t>>& spans);
// cudaStreamSynchronize on the library stream; nothing under capture.
void sync_library_stream();
void prof_begin(const char* name);
void prof_end(double alg_bytes = 0.0);
void prof_add_bytes_last(double alg_bytes);
void prof_collect();
void prof_enable(bool on);
void prof_reset();
size_t prof_count();
const char* prof_name(size_t i);
uint64_t prof_launches(size_t i);
double prof_ms(size_t i);
double prof_bytes(size_t i);
void* dev_alloc(size_t bytes);
void dev_free(void* p);

// Make sure `b` has at least `cap` entries and `k` key words; existing
// contents (first `keep` entries) are preserved; new words are zero-filled.
void ensure_buffers(Buffers& b, uint64_t cap, uint32_t k, uint64_t keep);
// Make the state's live buffers hold K = regtable().k words.
void sync_words(State& s);
void free_buffers(Buffers& b);
void swap_live_spare(State& s);

// Workspace (grow-only device scratch shared by all operators).
enum WsSlot {
    WS_SORT_KEY0 = 0,
    WS_SORT_KEY1,
    WS_SORT_VAL0,
    WS_SORT_VAL1,
    WS_LOOKBACK,
    WS_HIST,
    WS_SEG,
    WS_COUNT,
    WS_OFFSET,
    WS_MISC,
    WS_REDUCE,
    WS_MERGE_KEYS,
    WS_MATRIX,
    WS_CURSOR,
    WS_SKETCH,
    WS_OUTPUT,
    WS_PAIR_TABLE,    // partner table of the 1-bit splits
    WS_GROUP_LIST,    // groups a singleton fan-out leaves to the warp-per-group emit
    WS_SCRATCH_TEST,  // buffers of the bounded-wait self-test
    WS_COUNT_MAX
};
struct Workspace {
    void* p[WS_COUNT_MAX] = {nullptr};
    size_t sz[WS_COUNT_MAX] = {0};
    void* get(int slot, size_t bytes);
};
Workspace& ws();


// ------------------------------------------------------------------ launch helpers
inline unsigned grid_for(uint64_t n, int block, int per_sm = 8) {
    uint64_t g = (n + block - 1) / block;
    uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (g > cap) g = cap;
    if (g == 0) g = 1;
    return (unsigned)g;
}

// ------------------------------------------------------------------ operators (host entry, in .cu files)
struct DInstr;
void run_program(State& s, const sq_instr* prog, uint32_t n);
void clear_zero(State& s, double eps);
double norm_sq(const State& s);
void scale_amp(State& s, double k);
void add_systems(State& dst, const State& src, double coef);

enum GroupMode {
    GM_HADAMARD_INT = 0,   // Hadamard_Int: singleton formula, FWHT otherwise
    GM_HADAMARD_FULL = 1,  // Hadamard_Int_Full: sparse product below threshold, FWHT otherwise
    GM_HADAMARD_BOOL = 2,  // Hadamard_Bool pair rules
    GM_ROT = 3,            // Rot_Bool general 2x2
    GM_CONDROT = 4,        // CondRot_Rational_Bool
    GM_MERGE = 5,          // sum equal keys (add_systems)
    GM_UNITARY = 6         // Rot_GeneralUnitary: dense 2^k x 2^k per group
};
struct GroupSpec {
    int mode;
    Field target;        // varying bits (word, shift, n)
    Field aux;           // CondRot input register
    double2 m[4];        // Rot_Bool matrix
    double sign;         // CondRot: +1 / -1 (dag)
    DCondSet cond;
    double eps;          // prune threshold for outputs
    bool prune;
    const double2* mtable;  // device: CondRot_General_Bool matrices (4 per input value)
    const double2* umat;    // device: Rot_GeneralUnitary matrix
    int udag;
    Field varw;             // batched Hadamard: register holding each entry's digit count (width 0: unused)
    int unscaled;           // Hadamard singleton fan-out without the 2^(-n/2) factor (AddRegisterWithHadamard)
};
void group_transform(State& s, const GroupSpec& g);
void set_group_strategy(int s);
int get_group_strategy();
void set_output_sizing(int m);
int get_output_sizing();
void set_fwht_arithmetic(int m);
int get_fwht_arithmetic();
void set_hash_groups_hint(uint64_t groups);
uint64_t hash_groups_hint();
// Output-size hints for the next split (0: none); taken once.
void hint_output_size(uint64_t outputs);
uint64_t take_output_size_hint();
// Split outcomes, for the size predictor's training log and its overflow rate.
void note_output_size(int mode, uint64_t n_in, uint64_t groups, uint64_t n_out);
void note_single_pass_overflow();
uint64_t single_pass_overflows();
void set_single_pass_limit(uint64_t entries);
int autotune_pick(uint64_t key);
void autotune_record(uint64_t key, int strategy, double ms);
void autotune_reset();
uint64_t autotune_classes(uint64_t* decided);
uint64_t single_pass_limit();
// The learned size model (predictor.cu).
bool predictor_enabled();
bool predictor_logging();
bool predictor_predict(const float* features, float* out);
void predictor_log(const float* features, const float* sizes);
void zero_field(State& s, Field f);
void move_field(State& s, Field first, Field second, Field dst);

uint64_t* device_u64_scratch();

}  // namespace sq
