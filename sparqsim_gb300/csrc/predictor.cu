// predictor.cu — the learned output-size model of the split operators.
//
// A 3-layer FP32 MLP (48 -> 64 -> 64 -> 2, ReLU) maps a description of a
// split operator about to run (operator kind, target width, key words,
// log N, whether cached group ranges exist, and a 32-register sketch of the
// group keys) to two sizes: log2(groups / N) / 16 and log2(outputs / N) / 16.
// The group count sizes the hash table (no overflow retry); the output count
// gives the single-pass emit a capacity where the "fully populated" bound is
// too large to allocate. The exact count-then-scan path stays the fallback and
// the check on every prediction: a single pass whose outputs overflow the
// predicted capacity is redone exactly, so results never depend on the model.
//
// Training data is logged by the split operators themselves (features before,
// sizes after). Forward, backward and Adam are hand-written kernels; one
// training step is a fixed sequence of launches captured once into a CUDA
// graph and replayed. Every reduction runs in a fixed order, so gradients
// are deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "sq_internal.cuh"

namespace sq {

namespace {

constexpr int kIn = SQ_PRED_FEATURES, kHid = 64, kOut = 2;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kHid * kOut, kParams = kB3 + kOut;
static_assert(kParams == SQ_PRED_PARAMS, "parameter count");

// ---------------------------------------------------------------- kernels
// One block of 64 threads per row; thread h owns hidden unit h. Sums run in
// ascending input order. W is row-major [in][out].
__global__ void __launch_bounds__(kHid) fwd_kernel(const float* __restrict__ p, const float* __restrict__ x, int n,
                                                   float* __restrict__ z1, float* __restrict__ a1,
                                                   float* __restrict__ z2, float* __restrict__ a2,
                                                   float* __restrict__ y) {
    __shared__ float sx[kIn], s1[kHid], s2[kHid];
    const int r = blockIdx.x, h = threadIdx.x;
    if (r >= n) return;
    for (int i = h; i < kIn; i += kHid) sx[i] = x[(size_t)r * kIn + i];
    __syncthreads();
    float acc = p[kB1 + h];
    for (int i = 0; i < kIn; ++i) acc = fmaf(sx[i], p[kW1 + i * kHid + h], acc);
    const float r1 = acc > 0.f ? acc : 0.f;
    s1[h] = r1;
    if (z1) {
        z1[(size_t)r * kHid + h] = acc;
        a1[(size_t)r * kHid + h] = r1;
    }
    __syncthreads();
    acc = p[kB2 + h];
    for (int k = 0; k < kHid; ++k) acc = fmaf(s1[k], p[kW2 + k * kHid + h], acc);
    const float r2 = acc > 0.f ? acc : 0.f;
    s2[h] = r2;
    if (z2) {
        z2[(size_t)r * kHid + h] = acc;
        a2[(size_t)r * kHid + h] = r2;
    }
    __syncthreads();
    if (h < kOut) {
        float o = p[kB3 + h];
        for (int k = 0; k < kHid; ++k) o = fmaf(s2[k], p[kW3 + k * kOut + h], o);
        y[(size_t)r * kOut + h] = o;
    }
}

// Mean squared error over n rows x kOut outputs: dy = 2 (y - t) / (n kOut);
// loss written by one block in a fixed order.
__global__ void __launch_bounds__(256) loss_kernel(const float* __restrict__ y, const float* __restrict__ t, int n,
                                                   float* __restrict__ dy, float* __restrict__ loss) {
    __shared__ float part[256];
    const int m = n * kOut;
    const float scale = 2.f / (float)m;
    float acc = 0.f;
    for (int i = threadIdx.x; i < m; i += 256) {
        const float d = y[i] - t[i];
        dy[i] = scale * d;
        acc = fmaf(d, d, acc);
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = part[0] / (float)m;
}

// Deltas of the hidden layers, one block per row.
__global__ void __launch_bounds__(kHid) back_kernel(const float* __restrict__ p, const float* __restrict__ dy,
                                                    const float* __restrict__ z1, const float* __restrict__ z2, int n,
                                                    float* __restrict__ d1, float* __restrict__ d2) {
    __shared__ float sd2[kHid];
    const int r = blockIdx.x, h = threadIdx.x;
    if (r >= n) return;
    float acc = 0.f;
    for (int o = 0; o < kOut; ++o) acc = fmaf(dy[(size_t)r * kOut + o], p[kW3 + h * kOut + o], acc);
    const float g2 = z2[(size_t)r * kHid + h] > 0.f ? acc : 0.f;
    d2[(size_t)r * kHid + h] = g2;
    sd2[h] = g2;
    __syncthreads();
    acc = 0.f;
    for (int k = 0; k < kHid; ++k) acc = fmaf(sd2[k], p[kW2 + h * kHid + k], acc);
    d1[(size_t)r * kHid + h] = z1[(size_t)r * kHid + h] > 0.f ? acc : 0.f;
}

// G[i][o] = sum_r A[r][i] D[r][o] and Gb[o] = sum_r D[r][o], rows in order.
__global__ void __launch_bounds__(256) wgrad_kernel(const float* __restrict__ A, const float* __restrict__ D, int n,
                                                    int n_in, int n_out, float* __restrict__ G,
                                                    float* __restrict__ Gb) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n_in * n_out) {
        const int i = idx / n_out, o = idx % n_out;
        float acc = 0.f;
        for (int r = 0; r < n; ++r) acc = fmaf(A[(size_t)r * n_in + i], D[(size_t)r * n_out + o], acc);
        G[idx] = acc;
    } else if (idx < n_in * n_out + n_out) {
        const int o = idx - n_in * n_out;
        float acc = 0.f;
        for (int r = 0; r < n; ++r) acc += D[(size_t)r * n_out + o];
        Gb[o] = acc;
    }
}

// Adam (Kingma & Ba 2015) with bias correction; the step count lives on the
// device so that a captured training step can be replayed as is.
__global__ void __launch_bounds__(256) adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                                                   float* __restrict__ m, float* __restrict__ v,
                                                   unsigned* __restrict__ step, float lr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned t = *step + 1u;
    if (i < kParams) {
        const float b1 = 0.9f, b2 = 0.999f, e = 1e-8f;
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / (1.f - powf(b1, (float)t));
        const float vh = vi / (1.f - powf(b2, (float)t));
        p[i] -= lr * mh / (sqrtf(vh) + e);
    }
}
__global__ void step_kernel(unsigned* step) { *step += 1u; }

// Gather one minibatch: rows idx[off .. off + b) of (X, T); `off` advances on
// the device by b each replay.
__global__ void __launch_bounds__(256) gather_kernel(const float* __restrict__ X, const float* __restrict__ T,
                                                     const unsigned* __restrict__ idx, unsigned* __restrict__ off,
                                                     int b, int n_idx, float* __restrict__ xb,
                                                     float* __restrict__ tb) {
    const unsigned o = *off;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b * (kIn + kOut); i += gridDim.x * blockDim.x) {
        const int r = i / (kIn + kOut), c = i % (kIn + kOut);
        const unsigned src = idx[(o + (unsigned)r) % (unsigned)n_idx];
        if (c < kIn) xb[(size_t)r * kIn + c] = X[(size_t)src * kIn + c];
        else tb[(size_t)r * kOut + (c - kIn)] = T[(size_t)src * kOut + (c - kIn)];
    }
}
__global__ void advance_kernel(unsigned* off, int b) { *off += (unsigned)b; }

// ---------------------------------------------------------------- state
struct Net {
    float* p = nullptr;  // parameters
    float* g = nullptr;  // gradients (same layout)
    float* m = nullptr;
    float* v = nullptr;
    unsigned* ctr = nullptr;  // [0] Adam step, [1] minibatch offset
    float* loss = nullptr;
    int cap = 0;              // rows of the work arrays
    float *x = nullptr, *t = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *y = nullptr,
          *dy = nullptr, *d1 = nullptr, *d2 = nullptr;
    bool init = false;
    bool trained = false;
};
Net g_net;
bool g_enabled = false;
bool g_logging = false;
std::vector<float> g_log_x, g_log_t;
uint64_t g_predictions = 0;
constexpr size_t kLogMax = 1u << 20;

void ensure_net() {
    if (g_net.init) return;
    g_net.p = (float*)dev_alloc(kParams * 4);
    g_net.g = (float*)dev_alloc(kParams * 4);
    g_net.m = (float*)dev_alloc(kParams * 4);
    g_net.v = (float*)dev_alloc(kParams * 4);
    g_net.ctr = (unsigned*)dev_alloc(64);
    g_net.loss = (float*)dev_alloc(64);
    g_net.init = true;
}

void ensure_rows(int n) {
    if (g_net.cap >= n) return;
    float** bufs[] = {&g_net.x, &g_net.t, &g_net.z1, &g_net.a1, &g_net.z2, &g_net.a2, &g_net.y, &g_net.dy,
                      &g_net.d1, &g_net.d2};
    const size_t widths[] = {kIn, kOut, kHid, kHid, kHid, kHid, kOut, kOut, kHid, kHid};
    for (int i = 0; i < 10; ++i) {
        dev_free(*bufs[i]);
        *bufs[i] = nullptr;
    }
    for (int i = 0; i < 10; ++i) *bufs[i] = (float*)dev_alloc((size_t)n * widths[i] * 4);
    g_net.cap = n;
}

void reset_params(uint64_t seed) {
    ensure_net();
    std::vector<float> h(kParams, 0.f);
    std::mt19937_64 rng(seed);
    auto he = [&](int off, int fan_in, int count) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)fan_in));
        for (int i = 0; i < count; ++i) h[off + i] = nd(rng);
    };
    he(kW1, kIn, kIn * kHid);
    he(kW2, kHid, kHid * kHid);
    he(kW3, kHid, kHid * kOut);
    cudaStream_t st = stream();
    SQ_CUDA(cudaMemcpyAsync(g_net.p, h.data(), kParams * 4, cudaMemcpyHostToDevice, st));
    SQ_CUDA(cudaMemsetAsync(g_net.m, 0, kParams * 4, st));
    SQ_CUDA(cudaMemsetAsync(g_net.v, 0, kParams * 4, st));
    SQ_CUDA(cudaMemsetAsync(g_net.ctr, 0, 64, st));
    SQ_CUDA(cudaStreamSynchronize(st));
    g_net.trained = false;
}

// forward + loss + backward + weight gradients on rows already in g_net.x/t
void launch_grad(int n, cudaStream_t st) {
    fwd_kernel<<<n, kHid, 0, st>>>(g_net.p, g_net.x, n, g_net.z1, g_net.a1, g_net.z2, g_net.a2, g_net.y);
    loss_kernel<<<1, 256, 0, st>>>(g_net.y, g_net.t, n, g_net.dy, g_net.loss);
    back_kernel<<<n, kHid, 0, st>>>(g_net.p, g_net.dy, g_net.z1, g_net.z2, n, g_net.d1, g_net.d2);
    wgrad_kernel<<<(kIn * kHid + kHid + 255) / 256, 256, 0, st>>>(g_net.x, g_net.d1, n, kIn, kHid, g_net.g + kW1,
                                                                   g_net.g + kB1);
    wgrad_kernel<<<(kHid * kHid + kHid + 255) / 256, 256, 0, st>>>(g_net.a1, g_net.d2, n, kHid, kHid, g_net.g + kW2,
                                                                    g_net.g + kB2);
    wgrad_kernel<<<(kHid * kOut + kOut + 255) / 256, 256, 0, st>>>(g_net.a2, g_net.dy, n, kHid, kOut, g_net.g + kW3,
                                                                    g_net.g + kB3);
    count_launch(6);
}

}  // namespace

// ---------------------------------------------------------------- host interface
bool predictor_enabled() { return g_enabled && g_net.trained; }
bool predictor_logging() { return g_logging; }

bool predictor_predict(const float* x, float* y) {
    if (!predictor_enabled()) return false;
    if (!capturing()) {  // a capture repeats the recorded prediction
        ensure_rows(1);
        cudaStream_t st = stream();
        SQ_CUDA(cudaMemcpyAsync(g_net.x, x, kIn * 4, cudaMemcpyHostToDevice, st));
        prof_begin("predictor_forward");
        fwd_kernel<<<1, kHid, 0, st>>>(g_net.p, g_net.x, 1, nullptr, nullptr, nullptr, nullptr, g_net.y);
        prof_end(0.0);
        SQ_CUDA(cudaGetLastError());
        SQ_CUDA(cudaMemcpyAsync(y, g_net.y, kOut * 4, cudaMemcpyDeviceToHost, st));
        SQ_CUDA(cudaStreamSynchronize(st));
    }
    host_decision(y, kOut * 4);
    ++g_predictions;
    return true;
}

void predictor_log(const float* x, const float* t) {
    if (!g_logging || g_log_t.size() / kOut >= kLogMax) return;
    g_log_x.insert(g_log_x.end(), x, x + kIn);
    g_log_t.insert(g_log_t.end(), t, t + kOut);
}

uint64_t predictor_predictions() { return g_predictions; }

}  // namespace sq

using namespace sq;

extern "C" {

#define SQP_BEGIN try {
#define SQP_END                                      \
    return SQ_OK;                                    \
    }                                                \
    catch (const sq::Error& e) {                     \
        set_last_error(e.msg);                       \
        return e.code;                               \
    }                                                \
    catch (const std::exception& e) {                \
        set_last_error(e.what());                    \
        return SQ_ERR_INVALID;                       \
    }

int sq_predictor_reset(uint64_t seed) {
    SQP_BEGIN
    reset_params(seed);
    SQP_END
}

int sq_predictor_get_params(float* out, uint64_t n) {
    SQP_BEGIN
    if (!out || n != (uint64_t)kParams) fail(SQ_ERR_INVALID, "predictor: need SQ_PRED_PARAMS floats");
    ensure_net();
    host_read(out, g_net.p, kParams * 4);
    SQP_END
}

int sq_predictor_set_params(const float* in, uint64_t n) {
    SQP_BEGIN
    if (!in || n != (uint64_t)kParams) fail(SQ_ERR_INVALID, "predictor: need SQ_PRED_PARAMS floats");
    ensure_net();
    SQ_CUDA(cudaMemcpyAsync(g_net.p, in, kParams * 4, cudaMemcpyHostToDevice, stream()));
    SQ_CUDA(cudaMemsetAsync(g_net.m, 0, kParams * 4, stream()));
    SQ_CUDA(cudaMemsetAsync(g_net.v, 0, kParams * 4, stream()));
    SQ_CUDA(cudaMemsetAsync(g_net.ctr, 0, 64, stream()));
    SQ_CUDA(cudaStreamSynchronize(stream()));
    g_net.trained = true;
    SQP_END
}

int sq_predictor_gradient(const float* x, const float* t, uint64_t n, float* grad, float* loss) {
    SQP_BEGIN
    if (!x || !t || !grad || n == 0 || n > (1u << 20)) fail(SQ_ERR_INVALID, "predictor: bad gradient arguments");
    ensure_net();
    ensure_rows((int)n);
    cudaStream_t st = stream();
    SQ_CUDA(cudaMemcpyAsync(g_net.x, x, n * kIn * 4, cudaMemcpyHostToDevice, st));
    SQ_CUDA(cudaMemcpyAsync(g_net.t, t, n * kOut * 4, cudaMemcpyHostToDevice, st));
    launch_grad((int)n, st);
    SQ_CUDA(cudaGetLastError());
    SQ_CUDA(cudaMemcpyAsync(grad, g_net.g, kParams * 4, cudaMemcpyDeviceToHost, st));
    float l = 0.f;
    host_read(&l, g_net.loss, 4);
    if (loss) *loss = l;
    SQP_END
}

int sq_predictor_predict(const float* x, uint64_t n, float* y) {
    SQP_BEGIN
    if (!x || !y || n == 0 || n > (1u << 20)) fail(SQ_ERR_INVALID, "predictor: bad predict arguments");
    ensure_net();
    ensure_rows((int)n);
    cudaStream_t st = stream();
    SQ_CUDA(cudaMemcpyAsync(g_net.x, x, n * kIn * 4, cudaMemcpyHostToDevice, st));
    fwd_kernel<<<(unsigned)n, kHid, 0, st>>>(g_net.p, g_net.x, (int)n, nullptr, nullptr, nullptr, nullptr, g_net.y);
    count_launch();
    SQ_CUDA(cudaGetLastError());
    host_read(y, g_net.y, n * kOut * 4);
    SQP_END
}

// Minibatch Adam on (x, t): `epochs` passes over a fresh permutation each,
// batches of `batch` rows. One training step (gather, forward, loss,
// backward, three weight-gradient launches, Adam, counters) is captured into a
// CUDA graph once and replayed.
int sq_predictor_train(const float* x, const float* t, uint64_t n, uint32_t epochs, uint32_t batch, float lr,
                       uint64_t seed, float* final_loss) {
    SQP_BEGIN
    if (!x || !t || n == 0 || n > (1u << 22) || batch == 0 || batch > 4096)
        fail(SQ_ERR_INVALID, "predictor: bad training arguments");
    ensure_net();
    const int b = (int)std::min<uint64_t>(batch, n);
    ensure_rows(b);
    cudaStream_t st = stream();
    float* X = (float*)dev_alloc(n * kIn * 4);
    float* T = (float*)dev_alloc(n * kOut * 4);
    unsigned* idx = (unsigned*)dev_alloc(n * 4);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    try {
        SQ_CUDA(cudaMemcpyAsync(X, x, n * kIn * 4, cudaMemcpyHostToDevice, st));
        SQ_CUDA(cudaMemcpyAsync(T, t, n * kOut * 4, cudaMemcpyHostToDevice, st));
        SQ_CUDA(cudaMemsetAsync(g_net.ctr + 1, 0, 4, st));
        SQ_CUDA(cudaStreamSynchronize(st));
        SQ_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        gather_kernel<<<(b * (kIn + kOut) + 255) / 256, 256, 0, st>>>(X, T, idx, g_net.ctr + 1, b, (int)n, g_net.x,
                                                                      g_net.t);
        launch_grad(b, st);
        adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(g_net.p, g_net.g, g_net.m, g_net.v, g_net.ctr, lr);
        step_kernel<<<1, 1, 0, st>>>(g_net.ctr);
        advance_kernel<<<1, 1, 0, st>>>(g_net.ctr + 1, b);
        SQ_CUDA(cudaStreamEndCapture(st, &graph));
        SQ_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        std::vector<unsigned> perm(n);
        std::mt19937_64 rng(seed);
        const uint64_t steps_per_epoch = (n + b - 1) / b;
        for (uint32_t e = 0; e < epochs; ++e) {
            for (uint64_t i = 0; i < n; ++i) perm[i] = (unsigned)i;
            std::shuffle(perm.begin(), perm.end(), rng);
            SQ_CUDA(cudaMemcpyAsync(idx, perm.data(), n * 4, cudaMemcpyHostToDevice, st));
            SQ_CUDA(cudaMemsetAsync(g_net.ctr + 1, 0, 4, st));
            for (uint64_t s = 0; s < steps_per_epoch; ++s) {
                SQ_CUDA(cudaGraphLaunch(exec, st));
                count_launch(10);
            }
            SQ_CUDA(cudaStreamSynchronize(st));  // the permutation buffer is rewritten next epoch
        }
        float l = 0.f;
        host_read(&l, g_net.loss, 4);
        if (final_loss) *final_loss = l;
    } catch (...) {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        dev_free(X);
        dev_free(T);
        dev_free(idx);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    dev_free(X);
    dev_free(T);
    dev_free(idx);
    g_net.trained = true;
    SQP_END
}

int sq_predictor_enable(int on) {
    SQP_BEGIN
    g_enabled = on != 0;
    SQP_END
}

int sq_predictor_log_enable(int on) {
    SQP_BEGIN
    g_logging = on != 0;
    SQP_END
}

int sq_predictor_log_size(uint64_t* n) {
    SQP_BEGIN
    if (!n) fail(SQ_ERR_INVALID, "null pointer");
    *n = g_log_t.size() / kOut;
    SQP_END
}

int sq_predictor_log_read(float* x, float* t, uint64_t max_rows, uint64_t* rows) {
    SQP_BEGIN
    if (!rows) fail(SQ_ERR_INVALID, "null pointer");
    const uint64_t n = std::min<uint64_t>(max_rows, g_log_t.size() / kOut);
    if (n && (!x || !t)) fail(SQ_ERR_INVALID, "null buffer");
    if (n) {
        memcpy(x, g_log_x.data(), n * kIn * 4);
        memcpy(t, g_log_t.data(), n * kOut * 4);
    }
    *rows = n;
    SQP_END
}

int sq_predictor_log_clear(void) {
    SQP_BEGIN
    g_log_x.clear();
    g_log_t.clear();
    SQP_END
}

int sq_predictor_stats(uint64_t* predictions, uint64_t* overflows) {
    SQP_BEGIN
    if (predictions) *predictions = g_predictions;
    if (overflows) *overflows = single_pass_overflows();
    SQP_END
}

}  // extern "C"
