// api.cu — the extern "C" boundary (include/sparq_gb300.h). Validates
// arguments the way the reference operator constructors do, translates
// register ids into packed fields and forwards to the device pipelines.
// Exceptions never cross the boundary: every entry returns an sq_status and
// records a message for sq_last_error().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "sq_internal.cuh"

namespace sq {
void init_device(int device);
uint64_t launches();
void check_device_error();
void set_wait_limit(unsigned polls);
unsigned wait_limit();
void selftest_wait_timeout(unsigned polls);
uint64_t device_allocations();
}  // namespace sq

struct sq_state {
    sq::State s;
};
struct sq_qram {
    sq::QramTable t;
};

using namespace sq;

static thread_local std::string t_err;

namespace sq {
void set_last_error(const std::string& msg) { t_err = msg; }
}  // namespace sq

#define SQ_API_BEGIN try {
#define SQ_API_END                                   \
    return SQ_OK;                                    \
    }                                                \
    catch (const sq::Error& e) {                     \
        t_err = e.msg;                               \
        return e.code;                               \
    }                                                \
    catch (const std::bad_alloc&) {                  \
        t_err = "host allocation failed";            \
        return SQ_ERR_OOM;                           \
    }                                                \
    catch (const std::exception& e) {                \
        t_err = e.what();                            \
        return SQ_ERR_INVALID;                       \
    }

static void need(bool ok, const char* msg) {
    if (!ok) fail(SQ_ERR_INVALID, msg);
}
static sq_state* g_capture_state = nullptr;  // the state a capture runs on

// Every entry point that may write or free a state's buffers gets it here:
// the library stream first waits for an asynchronous download still reading
// them. While a capture runs, only its state may be used.
static State& S(sq_state* st) {
    need(st != nullptr, "null state");
    if (capturing() && st != g_capture_state) fail(SQ_ERR_INVALID, "capture: operators on another state");
    State& s = st->s;
    if (s.d2h_pending) {
        SQ_CUDA(cudaStreamWaitEvent(stream(), s.d2h_done, 0));
        s.d2h_pending = false;
    }
    return s;
}
static const State& S(const sq_state* st) {
    need(st != nullptr, "null state");
    return st->s;
}

static sq_instr make_instr(uint32_t op, const sq_cond* cond) {
    sq_instr in;
    memset(&in, 0, sizeof(in));
    in.op = op;
    if (cond) in.cond = *cond;
    return in;
}
static int run1(sq_state* st, const sq_instr& in) {
    SQ_API_BEGIN
    run_program(S(st), &in, 1);
    SQ_API_END
}

extern "C" {

int sq_abi_version(void) { return SQ_ABI_VERSION; }
const char* sq_last_error(void) { return t_err.c_str(); }

int sq_init(int device) {
    SQ_API_BEGIN
    init_device(device);
    SQ_API_END
}

int sq_synchronize(void) {
    SQ_API_BEGIN
    SQ_CUDA(cudaStreamSynchronize(stream()));
    sync_async_copies();
    check_device_error();
    SQ_API_END
}

int sq_launch_count(uint64_t* count) {
    SQ_API_BEGIN
    need(count != nullptr, "null pointer");
    *count = launches();
    SQ_API_END
}

int sq_profile_enable(int on) {
    SQ_API_BEGIN
    prof_enable(on != 0);
    SQ_API_END
}

int sq_profile_reset(void) {
    SQ_API_BEGIN
    prof_reset();
    SQ_API_END
}

int sq_profile_read(char* names_buf, size_t buf_len, uint64_t* counts, double* total_ms, double* total_bytes,
                    uint32_t max, uint32_t* n_out) {
    SQ_API_BEGIN
    prof_collect();
    const size_t n = std::min<size_t>(prof_count(), max);
    size_t off = 0;
    for (size_t i = 0; i < n; ++i) {
        const char* nm = prof_name(i);
        const size_t l = strlen(nm) + 1;
        if (names_buf && off + l <= buf_len) {
            memcpy(names_buf + off, nm, l);
            off += l;
        }
        if (counts) counts[i] = prof_launches(i);
        if (total_ms) total_ms[i] = prof_ms(i);
        if (total_bytes) total_bytes[i] = prof_bytes(i);
    }
    if (n_out) *n_out = (uint32_t)n;
    SQ_API_END
}

int sq_get_stream(void** s) {
    SQ_API_BEGIN
    need(s != nullptr, "null pointer");
    *s = (void*)stream();
    SQ_API_END
}

// ------------------------------------------------------------------ registers
int sq_system_clear(void) {
    SQ_API_BEGIN
    // the default prune threshold is a setting of its own, kept across a
    // clear as the reference's global clearzero_default_eps
    // (system_operations.h:577) is
    RegTable& t = regtable();
    const double eps = t.clearzero_eps;
    t = RegTable();
    t.clearzero_eps = eps;
    SQ_API_END
}

int sq_system_add_register(uint32_t type, uint32_t width, uint32_t* id_out) {
    SQ_API_BEGIN
    need(id_out != nullptr, "null pointer");
    *id_out = regtable().add(type, width);
    SQ_API_END
}

int sq_system_remove_register(uint32_t id) {
    SQ_API_BEGIN
    regtable().remove(id);
    SQ_API_END
}

int sq_system_register_info(uint32_t id, uint32_t* type, uint32_t* width, uint32_t* active, uint32_t* word,
                            uint32_t* shift) {
    SQ_API_BEGIN
    const RegTable& t = regtable();
    need(id < t.regs.size(), "register not found");
    const RegEntry& r = t.regs[id];
    if (type) *type = r.type;
    if (width) *width = r.width;
    if (active) *active = r.active ? 1 : 0;
    if (word) *word = r.word;
    if (shift) *shift = r.shift;
    SQ_API_END
}

int sq_system_register_count(uint32_t* n) {
    SQ_API_BEGIN
    need(n != nullptr, "null pointer");
    *n = (uint32_t)regtable().regs.size();
    SQ_API_END
}

int sq_system_key_words(uint32_t* k) {
    SQ_API_BEGIN
    need(k != nullptr, "null pointer");
    *k = regtable().k;
    SQ_API_END
}

int sq_system_set_register_type(uint32_t id, uint32_t type) {
    SQ_API_BEGIN
    need(type <= SQ_RATIONAL, "bad register type");
    (void)regtable().at(id);
    regtable().regs[id].type = type;
    SQ_API_END
}

// Live objects a graph may read: device tables by address with a generation
// number (an address the pool hands out again gets a new one), states by
// handle. Destroying one removes it, so that a graph launch refuses on the
// host, before any device read, when something it reads is gone.
static std::unordered_map<const void*, uint64_t> g_live_tables;
static std::unordered_set<const sq_state*> g_live_states;
static uint64_t g_table_gen = 0;
static void table_born(const void* dev) { g_live_tables[dev] = ++g_table_gen; }
static void table_dead(const void* dev) { g_live_tables.erase(dev); }
static uint64_t table_generation(const void* dev) {
    auto it = g_live_tables.find(dev);
    return it == g_live_tables.end() ? 0 : it->second;
}

// ------------------------------------------------------------------ state
int sq_state_create(uint64_t capacity, sq_state** out) {
    SQ_API_BEGIN
    need(out != nullptr, "null pointer");
    sq_state* st = new sq_state();
    try {
        ensure_buffers(st->s.live, capacity ? capacity : 1, regtable().k, 0);
        // one entry |0...0>, amplitude 1
        double2 one = make_double2(1.0, 0.0);
        SQ_CUDA(cudaMemcpyAsync(st->s.live.amp, &one, sizeof(one), cudaMemcpyHostToDevice, stream()));
        for (uint32_t w = 0; w < st->s.live.kalloc; ++w)
            SQ_CUDA(cudaMemsetAsync(st->s.live.keys[w], 0, 8, stream()));
        SQ_CUDA(cudaStreamSynchronize(stream()));
        st->s.n = 1;
    } catch (...) {
        free_buffers(st->s.live);
        delete st;
        throw;
    }
    g_live_states.insert(st);
    *out = st;
    SQ_API_END
}

int sq_state_destroy(sq_state* st) {
    SQ_API_BEGIN
    if (!st) return SQ_OK;
    g_live_states.erase(st);
    if (st->s.d2h_done) {  // an asynchronous download may still read the buffers
        SQ_CUDA(cudaEventSynchronize(st->s.d2h_done));
        SQ_CUDA(cudaEventDestroy(st->s.d2h_done));
    }
    free_buffers(st->s.live);
    free_buffers(st->s.spare);
    free_group_cache(st->s.groups);
    delete st;
    SQ_API_END
}

int sq_state_size(const sq_state* st, uint64_t* n) {
    SQ_API_BEGIN
    need(n != nullptr, "null pointer");
    *n = S(st).n;
    SQ_API_END
}

int sq_state_capacity(const sq_state* st, uint64_t* cap) {
    SQ_API_BEGIN
    need(cap != nullptr, "null pointer");
    *cap = S(st).live.cap;
    SQ_API_END
}

int sq_state_reserve(sq_state* st, uint64_t capacity) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    ensure_buffers(s.live, capacity, regtable().k, s.n);
    SQ_API_END
}

int sq_state_reset(sq_state* st) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    sync_words(s);
    ensure_buffers(s.live, 1, regtable().k, 0);
    double2 one = make_double2(1.0, 0.0);
    SQ_CUDA(cudaMemcpyAsync(s.live.amp, &one, sizeof(one), cudaMemcpyHostToDevice, stream()));
    for (uint32_t w = 0; w < s.live.kalloc; ++w) SQ_CUDA(cudaMemsetAsync(s.live.keys[w], 0, 8, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    s.n = 1;
    SQ_API_END
}

int sq_state_copy(sq_state* dst, const sq_state* src) {
    SQ_API_BEGIN
    State& d = S(dst);
    const State& s = S(src);
    drop_groups(d);
    const uint32_t k = regtable().k;
    ensure_buffers(d.live, std::max<uint64_t>(s.n, 1), k, 0);
    for (uint32_t w = 0; w < k; ++w) {
        if (w < s.live.kalloc)
            SQ_CUDA(cudaMemcpyAsync(d.live.keys[w], s.live.keys[w], s.n * 8, cudaMemcpyDeviceToDevice, stream()));
        else
            SQ_CUDA(cudaMemsetAsync(d.live.keys[w], 0, s.n * 8, stream()));
    }
    SQ_CUDA(cudaMemcpyAsync(d.live.amp, s.live.amp, s.n * 16, cudaMemcpyDeviceToDevice, stream()));
    d.n = s.n;
    SQ_API_END
}

// Host packing: one uint64 per register id per entry -> K packed words.
int sq_state_upload(sq_state* st, uint64_t n, const uint64_t* regs, uint32_t nregs, const double* amps) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    need(n == 0 || (regs != nullptr || nregs == 0) , "null regs");
    need(n == 0 || amps != nullptr, "null amps");
    const RegTable& t = regtable();
    const uint32_t k = t.k;
    std::vector<uint64_t> packed((size_t)k * n, 0);
    for (uint32_t id = 0; id < nregs && id < t.regs.size(); ++id) {
        const RegEntry& r = t.regs[id];
        if (!r.active || r.width == 0) continue;
        const uint64_t m = wmask(r.width);
        uint64_t* dst = packed.data() + (size_t)r.word * n;
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t v = regs[i * nregs + id];
            if (v & ~m) fail(SQ_ERR_INVALID, "register value wider than its register");
            dst[i] |= v << r.shift;
        }
    }
    ensure_buffers(s.live, std::max<uint64_t>(n, 1), k, 0);
    for (uint32_t w = 0; w < k; ++w)
        SQ_CUDA(cudaMemcpyAsync(s.live.keys[w], packed.data() + (size_t)w * n, n * 8, cudaMemcpyHostToDevice, stream()));
    SQ_CUDA(cudaMemcpyAsync(s.live.amp, amps, n * 16, cudaMemcpyHostToDevice, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    s.n = n;
    SQ_API_END
}

int sq_state_download(const sq_state* st, uint64_t* regs, uint32_t nregs, double* amps) {
    SQ_API_BEGIN
    const State& s = S(st);
    const RegTable& t = regtable();
    const uint64_t n = s.n;
    const uint32_t k = std::min<uint32_t>(t.k, s.live.kalloc);
    std::vector<uint64_t> packed((size_t)k * n);
    for (uint32_t w = 0; w < k; ++w)
        SQ_CUDA(cudaMemcpyAsync(packed.data() + (size_t)w * n, s.live.keys[w], n * 8, cudaMemcpyDeviceToHost, stream()));
    if (amps) SQ_CUDA(cudaMemcpyAsync(amps, s.live.amp, n * 16, cudaMemcpyDeviceToHost, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    if (regs) {
        for (uint64_t i = 0; i < n; ++i)
            for (uint32_t id = 0; id < nregs; ++id) {
                uint64_t v = 0;
                if (id < t.regs.size() && t.regs[id].active && t.regs[id].word < k) {
                    const RegEntry& r = t.regs[id];
                    v = (packed[(size_t)r.word * n + i] >> r.shift) & wmask(r.width);
                }
                regs[i * nregs + id] = v;
            }
    }
    SQ_API_END
}

int sq_state_upload_packed(sq_state* st, uint64_t n, const uint64_t* keys, const double* amps) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    need(n == 0 || (keys != nullptr && amps != nullptr), "null pointer");
    const uint32_t k = regtable().k;
    ensure_buffers(s.live, std::max<uint64_t>(n, 1), k, 0);
    std::vector<CopyJob> jobs;
    for (uint32_t w = 0; w < k; ++w) jobs.push_back({s.live.keys[w], keys + (size_t)w * n, (size_t)n * 8});
    jobs.push_back({s.live.amp, amps, (size_t)n * 16});
    parallel_copy(jobs.data(), (int)jobs.size(), cudaMemcpyHostToDevice);
    s.n = n;
    SQ_API_END
}

int sq_state_download_packed(const sq_state* st, uint64_t* keys, double* amps) {
    SQ_API_BEGIN
    const State& s = S(st);
    const uint32_t k = regtable().k;
    const uint64_t n = s.n;
    std::vector<CopyJob> jobs;
    for (uint32_t w = 0; w < k; ++w) {
        if (!keys) break;
        if (w < s.live.kalloc) jobs.push_back({keys + (size_t)w * n, s.live.keys[w], (size_t)n * 8});
        else memset(keys + (size_t)w * n, 0, n * 8);
    }
    if (amps) jobs.push_back({amps, s.live.amp, (size_t)n * 16});
    parallel_copy(jobs.data(), (int)jobs.size(), cudaMemcpyDeviceToHost);
    SQ_API_END
}

int sq_state_download_packed_async(sq_state* st, uint64_t* keys, double* amps) {
    SQ_API_BEGIN
    State& s = S(st);
    const uint32_t k = regtable().k;
    const uint64_t n = s.n;
    std::vector<CopyJob> jobs;
    for (uint32_t w = 0; w < k; ++w) {
        if (!keys) break;
        if (w < s.live.kalloc) jobs.push_back({keys + (size_t)w * n, s.live.keys[w], (size_t)n * 8});
        else memset(keys + (size_t)w * n, 0, n * 8);
    }
    if (amps) jobs.push_back({amps, s.live.amp, (size_t)n * 16});
    if (!s.d2h_done) SQ_CUDA(cudaEventCreateWithFlags(&s.d2h_done, cudaEventDisableTiming));
    async_copy_d2h(jobs.data(), (int)jobs.size(), s.d2h_done);
    s.d2h_pending = true;
    SQ_API_END
}

int sq_set_download_engine(int engine) {
    SQ_API_BEGIN
    set_d2h_engine(engine);
    SQ_API_END
}

int sq_state_wait(sq_state* st) {
    SQ_API_BEGIN
    need(st != nullptr, "null state");
    if (st->s.d2h_done) SQ_CUDA(cudaEventSynchronize(st->s.d2h_done));
    SQ_API_END
}

// ------------------------------------------------------------------ graphs
struct sq_graph {
    cudaGraph_t graph = nullptr;  // kept for inspection (sq_graph_debug_dot)
    cudaGraphExec_t exec = nullptr;
    uint64_t input_sum = 0, table_sum = 0;  // the recorded input state and tables
    std::vector<std::pair<const void*, size_t>> tables;
    std::vector<uint64_t> table_gens;  // generation of each table when recorded
    sq_state* st = nullptr;
    State pre, post;  // the state's host-side fields before and after the captured operators
    void* ws_p[WS_COUNT_MAX] = {nullptr};
    uint64_t launches = 0;
};

static State g_capture_pre;
static void* g_capture_ws[WS_COUNT_MAX];
static uint64_t g_capture_launch0 = 0;

static bool same_buffers(const Buffers& a, const Buffers& b) {
    if (a.amp != b.amp || a.cap != b.cap || a.kalloc != b.kalloc) return false;
    for (int w = 0; w < SQ_KMAX; ++w)
        if (a.keys[w] != b.keys[w]) return false;
    return true;
}
static bool same_layout(const State& a, const State& b) {
    if (!same_buffers(a.live, b.live) || !same_buffers(a.spare, b.spare)) return false;
    const GroupCache &x = a.groups, &y = b.groups;
    for (int i = 0; i < 2; ++i)
        if (x.start[i] != y.start[i] || x.cnt[i] != y.cnt[i] || x.cap[i] != y.cap[i]) return false;
    return x.valid == y.valid && x.cur == y.cur && a.n == b.n;
}

static sq_state* g_record_state = nullptr;
static uint64_t g_record_swaps = 0;
static int g_record_cur = 0;
static uint64_t g_record_input_sum = 0;   // the state the recording started from
static uint64_t g_record_table_sum = 0;   // the tables its operators read
static std::vector<std::pair<const void*, size_t>> g_record_tables;
static std::vector<uint64_t> g_record_table_gens;

// Checksum of a state's entries (key words and amplitudes): a replay runs only
// on the input it was recorded with, so that every recorded count holds.
static uint64_t state_checksum(const State& s) {
    std::vector<std::pair<const void*, size_t>> spans;
    for (uint32_t w = 0; w < s.live.kalloc; ++w) spans.emplace_back(s.live.keys[w], (size_t)s.n * 8);
    spans.emplace_back(s.live.amp, (size_t)s.n * 16);
    return device_checksum(spans);
}

int sq_graph_record_begin(sq_state* st) {
    SQ_API_BEGIN
    need(replay().mode == RP_OFF, "graph: a record or capture is already open");
    const State& s = S(st);
    g_record_state = st;
    g_record_swaps = s.swaps;
    g_record_cur = s.groups.cur;
    g_record_input_sum = state_checksum(s);
    replay().log.clear();
    replay().inputs.clear();
    replay().pos = 0;
    replay().mode = RP_RECORD;
    SQ_API_END
}

int sq_graph_record_end(void) {
    SQ_API_BEGIN
    need(replay().mode == RP_RECORD, "graph: no record is open");
    replay().mode = RP_OFF;
    const State& s = g_record_state->s;
    g_record_state = nullptr;
    // a replay starts where the previous one ended: the buffers must be back in their roles
    need((s.swaps - g_record_swaps) % 2 == 0 && s.groups.cur == g_record_cur,
         "graph: the operators leave the state's buffers in other roles (an odd number of splits)");
    g_record_tables = replay().inputs;
    g_record_table_gens.clear();
    for (const auto& t : g_record_tables) g_record_table_gens.push_back(table_generation(t.first));
    g_record_table_sum = device_checksum(g_record_tables);
    SQ_API_END
}

int sq_graph_capture_begin(sq_state* st) {
    SQ_API_BEGIN
    need(replay().mode == RP_OFF, "graph: a record or capture is already open");
    State& s = S(st);
    SQ_CUDA(cudaStreamSynchronize(stream()));
    need(state_checksum(s) == g_record_input_sum, "graph: the capture does not start from the recorded input");
    g_capture_pre = s;
    for (int i = 0; i < WS_COUNT_MAX; ++i) g_capture_ws[i] = ws().p[i];
    g_capture_launch0 = launches();
    g_capture_state = st;
    replay().pos = 0;
    SQ_CUDA(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal));
    replay().mode = RP_CAPTURE;
    SQ_API_END
}

int sq_graph_capture_end(sq_graph** out) {
    SQ_API_BEGIN
    need(replay().mode == RP_CAPTURE, "graph: no capture is open");
    replay().mode = RP_OFF;
    sq_state* st = g_capture_state;
    g_capture_state = nullptr;
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(stream(), &g);
    // nothing ran: the state is as it was, and the captured launches are not counted
    State post = st->s;
    const cudaEvent_t ev = st->s.d2h_done;
    st->s = g_capture_pre;
    st->s.d2h_done = ev;
    const uint64_t captured = launches() - g_capture_launch0;
    count_launch(-(int)captured);
    if (ce != cudaSuccess || !g) {
        (void)cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        fail(SQ_ERR_CUDA, std::string("graph: capture failed: ") + cudaGetErrorString(ce));
    }
    bool ws_same = true;
    for (int i = 0; i < WS_COUNT_MAX; ++i) ws_same = ws_same && ws().p[i] == g_capture_ws[i];
    if (replay().pos != replay().log.size() || !ws_same) {
        cudaGraphDestroy(g);
        fail(SQ_ERR_INVALID, "graph: the captured operators differ from the recorded ones");
    }
    sq_graph* gr = new sq_graph();
    const cudaError_t ie = cudaGraphInstantiate(&gr->exec, g, 0);
    gr->graph = g;
    if (ie != cudaSuccess) {
        cudaGraphDestroy(g);
        delete gr;
        fail(SQ_ERR_CUDA, std::string("graph: instantiate failed: ") + cudaGetErrorString(ie));
    }
    gr->st = st;
    gr->input_sum = g_record_input_sum;
    gr->table_sum = g_record_table_sum;
    gr->tables = g_record_tables;
    gr->table_gens = g_record_table_gens;
    gr->pre = g_capture_pre;
    gr->post = post;
    for (int i = 0; i < WS_COUNT_MAX; ++i) gr->ws_p[i] = g_capture_ws[i];
    gr->launches = captured;
    *out = gr;
    SQ_API_END
}

int sq_graph_launch(sq_graph* g) {
    SQ_API_BEGIN
    need(g != nullptr && g->exec != nullptr, "null graph");
    need(replay().mode == RP_OFF, "graph: a record or capture is open");
    // liveness on the host first: nothing below may read a freed table or state
    need(g_live_states.count(g->st) != 0, "graph: its state has been destroyed");
    for (size_t i = 0; i < g->tables.size(); ++i)
        need(g->table_gens[i] != 0 && table_generation(g->tables[i].first) == g->table_gens[i],
             "graph: a table it reads has been destroyed");
    State& s = S(g->st);
    need(same_layout(s, g->pre), "graph: the state's size or buffers differ from the captured ones");
    for (int i = 0; i < WS_COUNT_MAX; ++i)
        need(ws().p[i] == g->ws_p[i], "graph: the library's workspace has been reallocated");
    // every count and offset in the graph was recorded for one input: other
    // data could take other sizes, so it is refused before anything runs
    need(state_checksum(s) == g->input_sum, "graph: the state differs from the input the graph was recorded with");
    need(device_checksum(g->tables) == g->table_sum,
         "graph: a table the operators read differs from the one the graph was recorded with");
    SQ_CUDA(cudaGraphLaunch(g->exec, stream()));
    const cudaEvent_t ev = s.d2h_done;
    s = g->post;
    s.d2h_done = ev;
    s.d2h_pending = false;
    count_launch((int)g->launches);
    SQ_API_END
}

int sq_graph_destroy(sq_graph* g) {
    SQ_API_BEGIN
    if (!g) return SQ_OK;
    if (g->exec) SQ_CUDA(cudaGraphExecDestroy(g->exec));
    if (g->graph) SQ_CUDA(cudaGraphDestroy(g->graph));
    delete g;
    SQ_API_END
}

int sq_graph_debug_dot(const sq_graph* g, const char* path) {
    SQ_API_BEGIN
    need(g != nullptr && g->graph != nullptr && path != nullptr, "null pointer");
    SQ_CUDA(cudaGraphDebugDotPrint(g->graph, path, cudaGraphDebugDotFlagsVerbose));
    SQ_API_END
}

int sq_state_debug_layout(const sq_state* st, char* buf, uint64_t len) {
    SQ_API_BEGIN
    need(buf != nullptr && len > 0, "null pointer");
    const State& s = S(st);
    std::string o;
    char line[256];
    auto bufs = [&](const char* name, const Buffers& b) {
        snprintf(line, sizeof(line), "%s cap=%llu kalloc=%u amp=%p", name, (unsigned long long)b.cap, b.kalloc,
                 (void*)b.amp);
        o += line;
        for (uint32_t w = 0; w < b.kalloc; ++w) {
            snprintf(line, sizeof(line), " k%u=%p", w, (void*)b.keys[w]);
            o += line;
        }
        o += "\n";
    };
    snprintf(line, sizeof(line), "n=%llu swaps=%llu\n", (unsigned long long)s.n, (unsigned long long)s.swaps);
    o += line;
    bufs("live", s.live);
    bufs("spare", s.spare);
    const GroupCache& c = s.groups;
    for (int i = 0; i < 2; ++i) {
        snprintf(line, sizeof(line), "cache%d start=%p cnt=%p cap=%llu\n", i, (void*)c.start[i], (void*)c.cnt[i],
                 (unsigned long long)c.cap[i]);
        o += line;
    }
    snprintf(line, sizeof(line), "cache valid=%d cur=%d G=%llu\n", (int)c.valid, c.cur, (unsigned long long)c.G);
    o += line;
    for (int i = 0; i < WS_COUNT_MAX; ++i) {
        snprintf(line, sizeof(line), "ws%d=%p size=%zu\n", i, ws().p[i], ws().sz[i]);
        o += line;
    }
    snprintf(buf, len, "%s", o.c_str());
    SQ_API_END
}

int sq_state_device_arrays(sq_state* st, uint64_t** key_words, uint32_t* k, double** amps) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);  // the caller may write the arrays
    sync_words(s);
    if (key_words)
        for (uint32_t w = 0; w < regtable().k; ++w) key_words[w] = s.live.keys[w];
    if (k) *k = regtable().k;
    if (amps) *amps = (double*)s.live.amp;
    SQ_API_END
}

// ------------------------------------------------------------------ QRAM
int sq_qram_create(uint32_t address_size, uint32_t data_size, const uint64_t* memory, uint64_t n_words,
                   sq_qram** out) {
    SQ_API_BEGIN
    need(out != nullptr, "null pointer");
    need(address_size <= 40, "QRAM address_size > 40");
    need(data_size <= 64, "QRAM data_size > 64");
    const uint64_t words = 1ull << address_size;
    need(memory != nullptr && n_words >= words, "QRAM memory must hold 2^address_size words");
    // the highest bit any word uses decides the stored width (and is checked
    // against the data register at use); found and narrowed on the GPU, the
    // declared data size gives the first guess
    sq_qram* q = new sq_qram();
    q->t.address_size = address_size;
    q->t.data_size = data_size;
    q->t.n_words = words;
    try {
        uint32_t eb = 8;
        uint64_t all = 0;
        q->t.dev = qram_upload(memory, words, data_size <= 16 ? 2 : data_size <= 32 ? 4 : 8, &eb, &all);
        q->t.elem_bytes = eb;
        q->t.max_word = all;
    } catch (...) {
        delete q;
        throw;
    }
    table_born(q->t.dev);
    *out = q;
    SQ_API_END
}

int sq_qram_write(sq_qram* q, const uint64_t* memory, uint64_t n_words) {
    SQ_API_BEGIN
    need(q != nullptr && !q->t.lookup && q->t.pair_kind < 0, "not a QRAM table");
    need(memory != nullptr && n_words >= q->t.n_words, "QRAM memory must hold 2^address_size words");
    const uint64_t all = qram_rewrite(q->t, memory);  // writes nothing when a word does not fit
    const uint64_t fits = q->t.elem_bytes == 2 ? 0xffffull : q->t.elem_bytes == 4 ? 0xffffffffull : ~0ull;
    if (all & ~fits) fail(SQ_ERR_INVALID, "QRAM write: a word wider than the table's stored width (table unchanged)");
    q->t.max_word = all;
    SQ_API_END
}

int sq_qram_destroy(sq_qram* q) {
    SQ_API_BEGIN
    if (!q) return SQ_OK;
    table_dead(q->t.dev);
    dev_free(q->t.dev);  // stream-ordered: after every launch that reads it
    delete q;
    SQ_API_END
}

int sq_lookup_create(const uint64_t* dense, uint64_t dense_len, const uint64_t* keys, const uint64_t* words,
                     uint64_t n_sparse, sq_qram** out) {
    SQ_API_BEGIN
    need(out != nullptr, "null pointer");
    need(dense_len == 0 || dense != nullptr, "null pointer");
    need(n_sparse == 0 || (keys != nullptr && words != nullptr), "null pointer");
    need(dense_len + n_sparse > 0, "lookup: empty table");
    for (uint64_t i = 0; i < n_sparse; ++i) {
        need(keys[i] >= dense_len, "lookup: a sparse key inside the dense range");
        need(i == 0 || keys[i] > keys[i - 1], "lookup: sparse keys must ascend");
    }
    const uint64_t total = dense_len + 2 * n_sparse;
    std::vector<uint64_t> h(total);
    uint64_t all = 0;
    for (uint64_t i = 0; i < dense_len; ++i) {
        h[i] = dense[i];
        all |= dense[i];
    }
    for (uint64_t i = 0; i < n_sparse; ++i) {
        h[dense_len + i] = keys[i];
        h[dense_len + n_sparse + i] = words[i];
        all |= words[i];
    }
    sq_qram* q = new sq_qram();
    q->t.lookup = true;
    q->t.dense_len = dense_len;
    q->t.n_sparse = n_sparse;
    q->t.n_words = total;
    q->t.elem_bytes = 8;
    q->t.max_word = all;
    try {
        q->t.dev = dev_alloc(total * 8);
        SQ_CUDA(cudaMemcpyAsync(q->t.dev, h.data(), total * 8, cudaMemcpyHostToDevice, stream()));
        SQ_CUDA(cudaStreamSynchronize(stream()));  // the host copy goes out of scope
    } catch (...) {
        if (q->t.dev) dev_free(q->t.dev);
        delete q;
        throw;
    }
    table_born(q->t.dev);
    *out = q;
    SQ_API_END
}

// ------------------------------------------------------------------ angle tables
// The reference's per-entry angle computations, on the host with the C
// library, in the reference's expression order.
static uint64_t angle_rational(double x, uint32_t size) {  // get_rational: truncation; NaN -> 0
    if (std::isnan(x)) return 0;
    return (uint64_t)(x * (double)(1ull << size)) & wmask(size);
}
static int64_t angle_sext(uint64_t v, uint32_t w) {
    const uint64_t sign = 1ull << (w - 1);
    return (int64_t)((v ^ sign) - sign);
}
static uint64_t angle_word(int kind, uint32_t lw, uint32_t rw, uint32_t ow, uint64_t l, uint64_t r) {
    const double pi = 3.14159265358979323846;
    l &= wmask(lw);
    r &= wmask(rw);
    double out;
    if (kind == SQ_ANGLE_DIV_SQRT_ARCCOS) {  // quantum_arithmetic.cpp:413-432
        out = std::acos(std::sqrt(1.0 * l / r)) / pi / 2;
    } else {  // GetRotateAngle_Int_Int, quantum_arithmetic.cpp:458-487
        const int64_t x = angle_sext(l, lw), y = angle_sext(r, rw);
        if (x == 0 && y >= 0) out = 0.25;
        else if (x == 0 && y < 0) out = 0.75;
        else {
            out = std::atan2((double)y, (double)x) / pi / 2;
            if (out < 0) out += 1;
        }
    }
    return angle_rational(out, ow);
}

int sq_angle_word(int kind, uint32_t lhs_width, uint32_t rhs_width, uint32_t out_width, uint64_t lhs, uint64_t rhs,
                  uint64_t* word) {
    SQ_API_BEGIN
    need(word != nullptr, "null pointer");
    need(kind == SQ_ANGLE_DIV_SQRT_ARCCOS || kind == SQ_ANGLE_ROTATE, "angle: unknown kind");
    need(lhs_width >= 1 && lhs_width <= 63 && rhs_width >= 1 && rhs_width <= 63 && out_width >= 1 && out_width <= 63,
         "angle: widths must be 1..63");
    *word = angle_word(kind, lhs_width, rhs_width, out_width, lhs, rhs);
    SQ_API_END
}

int sq_angle_table_create(int kind, uint32_t lhs_width, uint32_t rhs_width, uint32_t out_width, const uint64_t* lhs,
                          const uint64_t* rhs, uint64_t n, sq_qram** out) {
    SQ_API_BEGIN
    need(out != nullptr && (n == 0 || (lhs != nullptr && rhs != nullptr)), "null pointer");
    need(kind == SQ_ANGLE_DIV_SQRT_ARCCOS || kind == SQ_ANGLE_ROTATE, "angle: unknown kind");
    need(lhs_width >= 1 && lhs_width <= 63 && rhs_width >= 1 && rhs_width <= 63 && out_width >= 1 && out_width <= 63,
         "angle: widths must be 1..63");
    need(n <= (1ull << 30), "angle: more than 2^30 pairs");
    uint64_t slots = 16;
    while (slots < 2 * n) slots <<= 1;  // load factor <= 1/2
    const uint64_t mask = slots - 1;
    std::vector<uint64_t> h(3 * slots, ~0ull);
    uint32_t probe_max = 0;
    uint64_t stored = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t l = lhs[i] & wmask(lhs_width), r = rhs[i] & wmask(rhs_width);
        const uint64_t base = pair_slot_hash(l, r);
        for (uint32_t p = 0;; ++p) {
            uint64_t* slot = &h[3 * ((base + p) & mask)];
            if (slot[0] == l && slot[1] == r) break;  // a repeat
            if (slot[0] == ~0ull && slot[1] == ~0ull) {
                slot[0] = l;
                slot[1] = r;
                slot[2] = angle_word(kind, lhs_width, rhs_width, out_width, l, r);
                probe_max = std::max(probe_max, p);
                ++stored;
                break;
            }
        }
    }
    sq_qram* q = new sq_qram();
    q->t.pair_kind = kind;
    q->t.pair_w[0] = lhs_width;
    q->t.pair_w[1] = rhs_width;
    q->t.pair_w[2] = out_width;
    q->t.pair_mask = mask;
    q->t.pair_probe = probe_max;
    q->t.n_words = 3 * slots;
    q->t.elem_bytes = 8;
    q->t.max_word = wmask(out_width);
    try {
        q->t.dev = dev_alloc(3 * slots * 8);
        SQ_CUDA(cudaMemcpyAsync(q->t.dev, h.data(), 3 * slots * 8, cudaMemcpyHostToDevice, stream()));
        SQ_CUDA(cudaStreamSynchronize(stream()));  // the host table goes out of scope
    } catch (...) {
        if (q->t.dev) dev_free(q->t.dev);
        delete q;
        throw;
    }
    table_born(q->t.dev);
    *out = q;
    SQ_API_END
}

int sq_qw_rotate_angle_words(const uint64_t* v, uint64_t n, uint32_t data_size, int positive_only,
                             uint32_t out_width, uint64_t* out) {
    SQ_API_BEGIN
    need(n == 0 || (v != nullptr && out != nullptr), "null pointer");
    need(data_size >= 2 && data_size <= 64, "GetQWRotateAngle: data_size out of range");
    need(out_width >= 1 && out_width <= 63, "GetQWRotateAngle: output width out of range");
    for (uint64_t i = 0; i < n; ++i) {
        double ratio;
        if (positive_only) {
            const uint64_t amax = (data_size >= 64 ? ~0ull : (1ull << data_size)) - 1;
            const uint64_t x = data_size >= 64 ? v[i] : v[i] % (amax + 1);
            ratio = x * 1.0 / amax;
        } else {
            const uint64_t amax = (1ull << (data_size - 1)) - 1;
            const uint64_t x = data_size >= 64 ? v[i] : v[i] % (1ull << data_size);
            const int64_t s = data_size >= 64 ? (int64_t)x
                                              : (int64_t)((x ^ (1ull << (data_size - 1))) - (1ull << (data_size - 1)));
            ratio = std::fabs((double)s) * 1.0 / amax;
        }
        ratio = std::max(0.0, std::min(1.0, ratio));
        const double a = std::acos(std::sqrt(ratio)) / M_PI / 2;
        out[i] = (uint64_t)(a * (double)(1ull << out_width));
    }
    SQ_API_END
}

// ------------------------------------------------------------------ elementwise
int sq_apply_program(sq_state* st, const sq_instr* prog, uint32_t n) {
    SQ_API_BEGIN
    need(prog != nullptr || n == 0, "null program");
    std::vector<sq_instr> p(prog, prog + n);
    for (auto& in : p) {
        // the ABI carries the opaque sq_qram*; the kernel wants its table record
        if ((in.op == SQ_OP_QRAM_LOAD || in.op == SQ_OP_LOOKUP_XOR) && in.qram)
            in.qram = reinterpret_cast<const sq_qram*>(&in.qram->t);
    }
    run_program(S(st), p.data(), n);
    SQ_API_END
}

int sq_add_uint_uint(sq_state* st, uint32_t lhs, uint32_t rhs, uint32_t res, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_ADD_UINT_UINT, cond);
    in.reg[0] = lhs; in.reg[1] = rhs; in.reg[2] = res;
    return run1(st, in);
}
int sq_add_uint_uint_inplace(sq_state* st, uint32_t lhs, uint32_t rhs, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_ADD_UINT_UINT_INPLACE, cond);
    in.reg[0] = lhs; in.reg[1] = rhs; in.dag = dag ? 1 : 0;
    return run1(st, in);
}
int sq_add_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_ADD_UINT_CONST, cond);
    in.reg[0] = lhs; in.reg[2] = res; in.imm[0] = c;
    return run1(st, in);
}
int sq_add_const_inplace(sq_state* st, uint32_t reg, uint64_t c, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_ADD_CONST_INPLACE, cond);
    in.reg[0] = reg; in.imm[0] = c; in.dag = dag ? 1 : 0;
    return run1(st, in);
}
int sq_mult_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_MULT_UINT_CONST, cond);
    in.reg[0] = lhs; in.reg[2] = res; in.imm[0] = c;
    return run1(st, in);
}
int sq_add_mult_uint_const(sq_state* st, uint32_t lhs, uint64_t c, uint32_t res, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_ADD_MULT_UINT_CONST, cond);
    in.reg[0] = lhs; in.reg[2] = res; in.imm[0] = c; in.dag = dag ? 1 : 0;
    return run1(st, in);
}
int sq_mul_uint_uint(sq_state* st, uint32_t lhs, uint32_t rhs, uint32_t res, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_MUL_UINT_UINT, cond);
    in.reg[0] = lhs; in.reg[1] = rhs; in.reg[2] = res;
    return run1(st, in);
}
int sq_add_anyint_inplace(sq_state* st, uint32_t lhs, uint32_t rhs, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_ADD_ANYINT_INPLACE, cond);
    in.reg[0] = lhs; in.reg[1] = rhs; in.dag = dag ? 1 : 0;
    return run1(st, in);
}
int sq_assign(sq_state* st, uint32_t src, uint32_t dst, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_ASSIGN, cond);
    in.reg[0] = src; in.reg[1] = dst;
    return run1(st, in);
}
int sq_shift(sq_state* st, uint32_t reg, uint32_t digits, int left, const sq_cond* cond) {
    sq_instr in = make_instr(left ? SQ_OP_SHIFT_LEFT : SQ_OP_SHIFT_RIGHT, cond);
    in.reg[0] = reg; in.imm[0] = digits;
    return run1(st, in);
}
int sq_swap(sq_state* st, uint32_t a, uint32_t b, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_SWAP_GENERAL, cond);
    in.reg[0] = a; in.reg[1] = b;
    return run1(st, in);
}
int sq_x_bool(sq_state* st, uint32_t reg, uint32_t digit, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_X_BOOL, cond);
    in.reg[0] = reg; in.imm[0] = digit;
    return run1(st, in);
}
int sq_flip_bools(sq_state* st, uint32_t reg, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_FLIP_BOOLS, cond);
    in.reg[0] = reg;
    return run1(st, in);
}
int sq_init_unsafe(sq_state* st, uint32_t reg, uint64_t value) {
    sq_instr in = make_instr(SQ_OP_INIT_UNSAFE, nullptr);
    in.reg[0] = reg; in.imm[0] = value;
    return run1(st, in);
}
int sq_qram_load(sq_state* st, const sq_qram* q, uint32_t addr, uint32_t data, const sq_cond* cond) {
    if (!q) {
        t_err = "QRAMLoad: null QRAM";
        return SQ_ERR_INVALID;
    }
    sq_instr in = make_instr(SQ_OP_QRAM_LOAD, cond);
    in.reg[0] = addr; in.reg[1] = data;
    in.qram = reinterpret_cast<const sq_qram*>(&q->t);
    return run1(st, in);
}
int sq_phase_bool(sq_state* st, uint32_t reg, uint32_t digit, double lambda, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_PHASE_BOOL, cond);
    in.reg[0] = reg; in.imm[0] = digit;
    in.c[0] = std::cos(lambda);
    in.c[1] = dag ? -std::sin(lambda) : std::sin(lambda);
    return run1(st, in);
}
int sq_global_phase(sq_state* st, double re, double im, const sq_cond* cond, int dag) {
    sq_instr in = make_instr(SQ_OP_GLOBAL_PHASE, cond);
    in.c[0] = re;
    in.c[1] = dag ? -im : im;
    return run1(st, in);
}
int sq_reflection_bool(sq_state* st, const uint32_t* regs, uint32_t nregs, int inverse, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_REFLECTION_BOOL, cond);
    for (uint32_t i = 0; i < nregs; ++i) {
        if (regs[i] >= 64) { t_err = "register id >= 64"; return SQ_ERR_INVALID; }
        in.imm[0] |= 1ull << regs[i];
    }
    in.imm[1] = inverse ? 1 : 0;
    return run1(st, in);
}
int sq_zero_cond_phase_flip(sq_state* st, const uint32_t* regs, uint32_t nregs, const sq_cond* cond) {
    sq_instr in = make_instr(SQ_OP_ZERO_COND_PHASE_FLIP, cond);
    for (uint32_t i = 0; i < nregs; ++i) {
        if (regs[i] >= 64) { t_err = "register id >= 64"; return SQ_ERR_INVALID; }
        in.imm[0] |= 1ull << regs[i];
    }
    return run1(st, in);
}

// ------------------------------------------------------------------ split / merge
static double cz_eps() { return regtable().clearzero_eps; }

// H on more than 12 bits: H^(x)n factorises over disjoint bit sets, so the
// low 12 bits run first, then the next (up to 12) bits, each pass grouping by
// every other bit. In the reference arithmetic each slot sees the same
// stage-ascending butterflies as in one pass; groups that one pass would treat
// as a singleton or a sparse bucket are rounded as in the FWHT instead (within
// 1e-15 relative).
static void hadamard_passes(State& s, Field f, uint32_t n, int mode, const DCondSet& cond) {
    for (uint32_t lo = 0; lo < n; lo += 12) {
        GroupSpec g;
        memset(&g, 0, sizeof(g));
        g.mode = mode;
        g.target = f;
        g.target.shift = (uint8_t)(f.shift + lo);
        g.target.width = (uint8_t)std::min<uint32_t>(12, n - lo);
        g.cond = cond;
        g.eps = cz_eps();
        group_transform(s, g);
    }
}

int sq_hadamard_int(sq_state* st, uint32_t reg, uint32_t n_digits, const sq_cond* cond) {
    SQ_API_BEGIN
    Field f = regtable().field(reg);
    need(n_digits <= f.width, "Hadamard_Int: n_digits larger than the register");
    if (n_digits == 0) return SQ_OK;
    hadamard_passes(S(st), f, n_digits, GM_HADAMARD_INT, resolve_cond(cond));
    SQ_API_END
}

int sq_hadamard_int_batched(sq_state* st, uint32_t reg, uint32_t width_reg, uint32_t max_digits, const sq_cond* cond) {
    SQ_API_BEGIN
    need(reg != width_reg, "batched Hadamard: width register must differ from the target");
    Field f = regtable().field(reg);
    Field w = regtable().field(width_reg);
    need(max_digits >= 1 && max_digits <= 8, "batched Hadamard: max_digits must be 1..8");
    need(max_digits <= f.width, "batched Hadamard: max_digits larger than the register");
    need(w.width >= 1, "batched Hadamard: empty width register");
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_HADAMARD_INT;
    g.target = f;
    g.target.width = (uint8_t)max_digits;
    g.varw = w;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(S(st), g);
    SQ_API_END
}

int sq_hadamard_int_full(sq_state* st, uint32_t reg, const sq_cond* cond) {
    SQ_API_BEGIN
    Field f = regtable().field(reg);
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_HADAMARD_FULL;
    g.target = f;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    if (f.width == 0) return SQ_OK;
    if (f.width > 12) {  // the register in passes of 12 bits
        hadamard_passes(S(st), f, f.width, GM_HADAMARD_INT, g.cond);
        return SQ_OK;
    }
    group_transform(S(st), g);
    SQ_API_END
}

int sq_hadamard_bool(sq_state* st, uint32_t reg, const sq_cond* cond) {
    SQ_API_BEGIN
    Field f = regtable().field(reg);
    need(f.width == 1, "Hadamard_Bool: size of output register must be 1");
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_HADAMARD_BOOL;
    g.target = f;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(S(st), g);
    SQ_API_END
}

static double abs_sqr(double re, double im) { return re * re + im * im; }

int sq_rot_bool(sq_state* st, uint32_t reg, uint32_t digit, const double* m8, const sq_cond* cond, int dag) {
    SQ_API_BEGIN
    need(m8 != nullptr, "null matrix");
    Field f = regtable().field(reg);
    need(digit < f.width, "Rot_Bool: digit >= register size");
    double m[8];
    memcpy(m, m8, sizeof(m));
    if (dag) {  // conjugate transpose
        double d[8] = {m8[0], -m8[1], m8[4], -m8[5], m8[2], -m8[3], m8[6], -m8[7]};
        memcpy(m, d, sizeof(m));
    }
    const double eps = 1e-14;  // Rot_Bool::_is_diagonal / _is_off_diagonal threshold (library epsilon)
    const bool diag = abs_sqr(m[2], m[3]) < eps && abs_sqr(m[4], m[5]) < eps;
    const bool off = abs_sqr(m[0], m[1]) < eps && abs_sqr(m[6], m[7]) < eps;
    State& s = S(st);
    if (diag || off) {
        // in-place: no new entries (basic_gates.cpp:110-171), then ClearZero
        sq_instr in = make_instr(diag ? SQ_OP_ROT_DIAGONAL : SQ_OP_ROT_OFF_DIAGONAL, cond);
        in.reg[0] = reg;
        in.imm[0] = digit;
        if (diag) {
            in.c[0] = m[0]; in.c[1] = m[1]; in.c[2] = m[6]; in.c[3] = m[7];
        } else {  // bit 0 -> multiply by m10, bit 1 -> multiply by m01
            in.c[0] = m[4]; in.c[1] = m[5]; in.c[2] = m[2]; in.c[3] = m[3];
        }
        run_program(s, &in, 1);
        clear_zero(s, cz_eps());
        return SQ_OK;
    }
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_ROT;
    g.target = f;
    g.target.shift = (uint8_t)(f.shift + digit);
    g.target.width = 1;
    for (int i = 0; i < 4; ++i) g.m[i] = make_double2(m[2 * i], m[2 * i + 1]);
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(s, g);
    SQ_API_END
}

int sq_condrot_rational_bool(sq_state* st, uint32_t reg_in, uint32_t reg_out, int dag) {
    return sq_condrot_rational_bool_cond(st, reg_in, reg_out, dag, nullptr);
}

int sq_condrot_rational_bool_cond(sq_state* st, uint32_t reg_in, uint32_t reg_out, int dag, const sq_cond* cond) {
    SQ_API_BEGIN
    need(reg_in != reg_out, "CondRot: input and output registers must differ");
    Field fi = regtable().field(reg_in);
    Field fo = regtable().field(reg_out);
    need(fi.type == SQ_RATIONAL && fo.type == SQ_BOOLEAN, "CondRot_Rational_Bool: input must be Rational, output Boolean");
    need(fo.width == 1, "CondRot_Rational_Bool: output register must be 1 bit");
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_CONDROT;
    g.target = fo;
    g.aux = fi;
    g.sign = dag ? -1.0 : 1.0;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(S(st), g);
    SQ_API_END
}

int sq_condrot_general_bool(sq_state* st, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values) {
    return sq_condrot_general_bool_cond(st, reg_in, reg_out, table, n_values, nullptr);
}

int sq_condrot_general_bool_cond(sq_state* st, uint32_t reg_in, uint32_t reg_out, const double* table, uint64_t n_values,
                                 const sq_cond* cond) {
    SQ_API_BEGIN
    need(reg_in != reg_out, "CondRot_General_Bool: input and output registers must differ");
    need(table != nullptr, "null matrix table");
    Field fi = regtable().field(reg_in);
    Field fo = regtable().field(reg_out);
    need(fo.type == SQ_BOOLEAN && fo.width == 1, "CondRot_General_Bool: output must be a 1-bit Boolean register");
    need(fi.width <= 24, "CondRot_General_Bool: input register wider than 24 bits");
    need(n_values == (1ull << fi.width), "CondRot_General_Bool: table must hold 2^width(in) matrices");
    double2* dev = (double2*)ws().get(WS_MATRIX, n_values * 4 * sizeof(double2));
    SQ_CUDA(cudaMemcpyAsync(dev, table, n_values * 4 * sizeof(double2), cudaMemcpyHostToDevice, stream()));
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_ROT;
    g.target = fo;
    g.aux = fi;
    g.mtable = dev;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(S(st), g);
    SQ_API_END
}

int sq_rot_general_unitary(sq_state* st, uint32_t reg, const double* mat, uint64_t dim, const sq_cond* cond, int dag) {
    SQ_API_BEGIN
    need(mat != nullptr, "null matrix");
    Field f = regtable().field(reg);
    need(f.width >= 1 && f.width <= 8, "Rot_GeneralUnitary: register width must be 1..8");
    need(dim == (1ull << f.width), "Rot_GeneralUnitary: matrix size does not match the register's size");
    double2* dev = (double2*)ws().get(WS_MATRIX, dim * dim * sizeof(double2));
    SQ_CUDA(cudaMemcpyAsync(dev, mat, dim * dim * sizeof(double2), cudaMemcpyHostToDevice, stream()));
    GroupSpec g;
    memset(&g, 0, sizeof(g));
    g.mode = GM_UNITARY;
    g.target = f;
    g.umat = dev;
    g.udag = dag ? 1 : 0;
    g.cond = resolve_cond(cond);
    g.eps = cz_eps();
    group_transform(S(st), g);
    SQ_API_END
}

int sq_hadamard_partial(sq_state* st, uint32_t reg, const uint32_t* positions, uint32_t n_positions, const sq_cond* cond) {
    SQ_API_BEGIN
    need(positions != nullptr || n_positions == 0, "Hadamard_Partial: null positions");
    Field f = regtable().field(reg);
    uint64_t set = 0;  // the reference takes a std::set: repeats collapse
    for (uint32_t i = 0; i < n_positions; ++i) {
        need(positions[i] < f.width, "Hadamard_Partial: position >= register size");
        set |= 1ull << positions[i];
    }
    const uint32_t n = (uint32_t)__builtin_popcountll(set);
    if (n == 0) return SQ_OK;
    if (n == 1) {  // the reference's active path: pairs equal except the bit
        GroupSpec g;
        memset(&g, 0, sizeof(g));
        g.mode = GM_HADAMARD_BOOL;
        g.target = f;
        g.target.shift = (uint8_t)(f.shift + __builtin_ctzll(set));
        g.target.width = 1;
        g.cond = resolve_cond(cond);
        g.eps = cz_eps();
        group_transform(S(st), g);
        return SQ_OK;
    }
    // Several positions: gather the set's bits to the low end of the
    // register (member index = from_map_position), H on those n low bits
    // (Hadamard_Int's groups and butterflies are Hadamard_Partial::operate's
    // on the gathered index), scatter back. Conditions on this register are
    // rewritten for the gathered layout.
    auto gather = [&](uint64_t v) {
        uint64_t out = 0, rest = 0;
        uint32_t lo = 0, hi = 0;
        for (uint32_t b = 0; b < f.width; ++b) {
            const uint64_t bit = (v >> b) & 1ull;
            if ((set >> b) & 1ull) out |= bit << lo++;
            else rest |= bit << hi++;
        }
        return out | (hi ? rest << n : 0);
    };
    sq_cond c2;
    memset(&c2, 0, sizeof(c2));
    if (cond) c2 = *cond;
    for (uint32_t i = 0; i < c2.count && i < SQ_MAX_CONDITIONS; ++i) {
        sq_condition& c = c2.c[i];
        if (c.reg != reg) continue;
        if (c.kind == SQ_COND_BIT) {
            need(c.param < f.width, "condition bit >= register size");
            c.param = (uint64_t)__builtin_ctzll(gather(1ull << c.param));
        } else if (c.kind == SQ_COND_VALUE) {
            if (f.width >= 64 || c.param <= wmask(f.width)) c.param = gather(c.param);
        }  // nonzero and all-ones do not depend on the bit order
    }
    sq_instr in;
    memset(&in, 0, sizeof(in));
    in.op = SQ_OP_BIT_GATHER;
    in.reg[0] = reg;
    in.imm[0] = set;
    const bool low = set == wmask(n);  // already the low n bits
    if (!low) run_program(S(st), &in, 1);
    hadamard_passes(S(st), f, n, GM_HADAMARD_INT, resolve_cond(&c2));
    in.dag = 1;
    if (!low) run_program(S(st), &in, 1);
    SQ_API_END
}

// ------------------------------------------------------------------ prune / norm / merge
int sq_set_group_strategy(int strategy) {
    SQ_API_BEGIN
    set_group_strategy(strategy);
    SQ_API_END
}
int sq_get_group_strategy(int* strategy) {
    SQ_API_BEGIN
    need(strategy != nullptr, "null pointer");
    *strategy = get_group_strategy();
    SQ_API_END
}

int sq_autotune_reset(void) {
    SQ_API_BEGIN
    autotune_reset();
    SQ_API_END
}
int sq_autotune_classes(uint64_t* classes, uint64_t* decided) {
    SQ_API_BEGIN
    const uint64_t c = autotune_classes(decided);
    if (classes) *classes = c;
    SQ_API_END
}

int sq_set_output_sizing(int mode) {
    SQ_API_BEGIN
    set_output_sizing(mode);
    SQ_API_END
}
int sq_get_output_sizing(int* mode) {
    SQ_API_BEGIN
    need(mode != nullptr, "null pointer");
    *mode = get_output_sizing();
    SQ_API_END
}

int sq_set_hash_groups_hint(uint64_t groups) {
    SQ_API_BEGIN
    set_hash_groups_hint(groups);
    SQ_API_END
}

int sq_set_single_pass_limit(uint64_t entries) {
    SQ_API_BEGIN
    set_single_pass_limit(entries);
    SQ_API_END
}

int sq_set_fwht_arithmetic(int mode) {
    SQ_API_BEGIN
    set_fwht_arithmetic(mode);
    SQ_API_END
}
int sq_get_fwht_arithmetic(int* mode) {
    SQ_API_BEGIN
    need(mode != nullptr, "null pointer");
    *mode = get_fwht_arithmetic();
    SQ_API_END
}

int sq_device_allocation_count(uint64_t* count) {
    SQ_API_BEGIN
    need(count != nullptr, "null pointer");
    *count = device_allocations();
    SQ_API_END
}

int sq_set_wait_limit(uint32_t polls) {
    SQ_API_BEGIN
    set_wait_limit(polls);
    SQ_API_END
}
int sq_get_wait_limit(uint32_t* polls) {
    SQ_API_BEGIN
    need(polls != nullptr, "null pointer");
    *polls = wait_limit();
    SQ_API_END
}
int sq_selftest_wait_timeout(uint32_t polls) {
    SQ_API_BEGIN
    selftest_wait_timeout(polls);
    SQ_API_END
}

int sq_set_clearzero_eps(double eps) {
    SQ_API_BEGIN
    need(eps >= 0.0, "negative eps");
    regtable().clearzero_eps = eps;
    SQ_API_END
}
int sq_get_clearzero_eps(double* eps) {
    SQ_API_BEGIN
    need(eps != nullptr, "null pointer");
    *eps = regtable().clearzero_eps;
    SQ_API_END
}

int sq_clear_zero(sq_state* st, double eps) {
    SQ_API_BEGIN
    clear_zero(S(st), eps);
    SQ_API_END
}

int sq_partial_trace_select(sq_state* st, const uint32_t* regs, const uint64_t* values, uint32_t n,
                            double* result) {
    SQ_API_BEGIN
    need(result != nullptr, "null pointer");
    need(n <= SQ_MAX_CONDITIONS, "PartialTraceSelect: at most SQ_MAX_CONDITIONS registers");
    need(n == 0 || (regs != nullptr && values != nullptr), "null pointer");
    if (n == 0) {  // partial_trace.cpp:151-152
        *result = 0.0;
        return SQ_OK;
    }
    sq_cond c;
    memset(&c, 0, sizeof(c));
    c.count = n;
    for (uint32_t i = 0; i < n; ++i) {
        c.c[i].kind = SQ_COND_VALUE;
        c.c[i].reg = regs[i];
        c.c[i].param = values[i];
    }
    Field none{};
    *result = select_entries(S(st), resolve_cond(&c), none, 0, 0);
    SQ_API_END
}

int sq_partial_trace_select_range(sq_state* st, uint32_t reg, uint64_t lo, uint64_t hi, double* result) {
    SQ_API_BEGIN
    need(result != nullptr, "null pointer");
    Field f = regtable().field(reg);
    need(f.width > 0, "PartialTraceSelectRange: empty register");
    DCondSet none;
    memset(&none, 0, sizeof(none));
    *result = select_entries(S(st), none, f, lo, hi);
    SQ_API_END
}

int sq_get_output(sq_state* st, const uint32_t* zero_regs, uint32_t n_zero, const uint32_t* idx_regs,
                  uint32_t n_idx, double* out, uint64_t out_len, double* prob) {
    SQ_API_BEGIN
    need(prob != nullptr && out != nullptr, "null pointer");
    need(n_zero <= SQ_MAX_CONDITIONS, "GetOutput: at most SQ_MAX_CONDITIONS post-selected registers");
    need(n_idx >= 1 && n_idx <= SQ_MAX_OUTPUT_FIELDS, "GetOutput: 1 to SQ_MAX_OUTPUT_FIELDS index registers");
    need(n_zero == 0 || zero_regs != nullptr, "null pointer");
    need(idx_regs != nullptr, "null pointer");
    const RegTable& rt = regtable();
    Field f[SQ_MAX_OUTPUT_FIELDS];
    uint32_t bits = 0;
    std::vector<uint32_t> used;
    for (uint32_t j = 0; j < n_idx; ++j) {
        f[j] = rt.field(idx_regs[j]);
        bits += f[j].width;
        used.push_back(idx_regs[j]);
    }
    need(bits <= 30, "GetOutput: the index registers exceed 30 bits");
    need(out_len == (1ull << bits), "GetOutput: out_len must be 2^(sum of index widths)");
    sq_cond c;
    memset(&c, 0, sizeof(c));
    c.count = n_zero;
    for (uint32_t i = 0; i < n_zero; ++i) {
        c.c[i].kind = SQ_COND_VALUE;
        c.c[i].reg = zero_regs[i];
        c.c[i].param = 0;
        used.push_back(zero_regs[i]);
    }
    for (uint32_t r = 0; r < rt.regs.size(); ++r) {
        if (!rt.regs[r].active || rt.regs[r].width == 0) continue;
        need(std::find(used.begin(), used.end(), r) != used.end(),
             "GetOutput: every active register must be post-selected or indexed");
    }
    *prob = get_output(S(st), resolve_cond(&c), f, n_idx, out);
    SQ_API_END
}

int sq_normalize(sq_state* st, double* norm_sq_out) {
    SQ_API_BEGIN
    State& s = S(st);
    const double sum = norm_sq(s);
    const double k = 1.0 / std::sqrt(sum);
    if (std::isnan(k)) fail(SQ_ERR_BAD_RESULT, "Normalize: norm is NaN");
    scale_amp(s, k);
    if (norm_sq_out) *norm_sq_out = sum;
    SQ_API_END
}

int sq_norm_sq(const sq_state* st, double* out) {
    SQ_API_BEGIN
    need(out != nullptr, "null pointer");
    *out = norm_sq(S(st));
    SQ_API_END
}

int sq_add_systems(sq_state* dst, const sq_state* src, double coef) {
    SQ_API_BEGIN
    need(dst != src, "add_systems: source and destination must differ");
    drop_groups(S(dst));
    add_systems(S(dst), S(src), coef);
    SQ_API_END
}

int sq_add_register_sync(sq_state* st, uint32_t type, uint32_t width, uint32_t* id_out) {
    SQ_API_BEGIN
    need(id_out != nullptr, "null pointer");
    State& s = S(st);
    drop_groups(s);
    const uint32_t id = regtable().add(type, width);
    *id_out = id;
    zero_field(s, regtable().field(id));
    SQ_API_END
}

int sq_add_register_with_hadamard(sq_state* st, uint32_t type, uint32_t width, uint32_t* id_out) {
    SQ_API_BEGIN
    need(id_out != nullptr, "null pointer");
    State& s = S(st);
    drop_groups(s);
    const uint32_t id = regtable().add(type, width);
    *id_out = id;
    Field f = regtable().field(id);
    zero_field(s, f);
    // every entry is alone in its group (the new register is 0 everywhere):
    // the singleton fan-out, its factor 1 instead of 2^(-n/2), no prune
    for (uint32_t lo = 0; lo < width; lo += 12) {
        GroupSpec g;
        memset(&g, 0, sizeof(g));
        g.mode = GM_HADAMARD_INT;
        g.target = f;
        g.target.shift = (uint8_t)(f.shift + lo);
        g.target.width = (uint8_t)std::min<uint32_t>(12, width - lo);
        g.eps = -1.0;
        g.unscaled = 1;
        group_transform(s, g);
    }
    SQ_API_END
}

int sq_remove_register_sync(sq_state* st, uint32_t id) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    Field f = regtable().field(id);
    zero_field(s, f);
    regtable().remove(id);
    SQ_API_END
}

int sq_split_register(sq_state* st, uint32_t first, uint32_t second_size, uint32_t* second_out) {
    SQ_API_BEGIN
    need(second_out != nullptr, "null pointer");
    State& s = S(st);
    drop_groups(s);
    RegTable& t = regtable();
    const RegEntry fe = t.at(first);
    need(second_size <= fe.width, "SplitRegister: second size larger than the register");
    // The low `second_size` bits of `first` become the new register in place:
    // no data moves. Allocate an id without bits, then hand it the low bits.
    const uint32_t id = t.add(fe.type, 0);
    RegEntry& se = t.regs[id];
    RegEntry& f2 = t.regs[first];
    se.width = second_size;
    se.word = fe.word;
    se.shift = fe.shift;
    f2.width = fe.width - second_size;
    f2.shift = fe.shift + second_size;
    if (f2.width == 0) f2.shift = fe.shift;
    (void)s;
    *second_out = id;
    SQ_API_END
}

int sq_combine_register(sq_state* st, uint32_t first, uint32_t second) {
    SQ_API_BEGIN
    State& s = S(st);
    drop_groups(s);
    RegTable& t = regtable();
    need(first != second, "CombineRegister: registers must differ");
    const RegEntry a = t.at(first);
    const RegEntry b = t.at(second);
    need(a.width + b.width <= 64, "CombineRegister: combined width > 64");
    if (b.width == 0) {
        t.remove(second);
        return SQ_OK;
    }
    if (a.width == 0 || (a.word == b.word && a.shift == b.shift + b.width)) {
        // adjacent (or empty first): metadata only
        RegEntry& fa = t.regs[first];
        fa.word = b.word;
        fa.shift = b.shift;
        fa.width = a.width + b.width;
        t.regs[second].width = 0;  // bits now belong to `first`
        t.remove(second);
        return SQ_OK;
    }
    // move both fields into a fresh field of the combined width
    Field fa = t.field(first), fb = t.field(second);
    t.free_bits(a.word, a.shift, a.width);
    t.free_bits(b.word, b.shift, b.width);
    uint32_t w, sh;
    if (!t.alloc_bits(a.width + b.width, &w, &sh)) {
        t.used[a.word] |= wmask(a.width) << a.shift;
        t.used[b.word] |= wmask(b.width) << b.shift;
        fail(SQ_ERR_CAPACITY, "packed key space exhausted");
    }
    Field dst;
    dst.word = (uint8_t)w;
    dst.shift = (uint8_t)sh;
    dst.width = (uint8_t)(a.width + b.width);
    dst.type = fa.type;
    move_field(s, fa, fb, dst);
    RegEntry& ea = t.regs[first];
    ea.word = w;
    ea.shift = sh;
    ea.width = a.width + b.width;
    t.regs[second].width = 0;
    t.remove(second);
    SQ_API_END
}

}  // extern "C"
