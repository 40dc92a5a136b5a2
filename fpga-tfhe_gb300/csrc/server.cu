// server.cu -- continuous-batching gate server over one engine context.
//
// The reference's test_bench server (test_bench/server/cloud.c:39-74) loads a
// cloud key, reads ciphertexts, runs a circuit gate by gate (bootsOR,
// bootsXNOR, bootsMUX; cloud.c:9-36) and writes the results.  This is that
// server as a request loop: many clients submit circuits (gate lists over
// their input ciphertexts); the server keeps every admitted circuit's wires
// resident in a device ciphertext pool, and each tick runs, as one batch,
// every gate of every admitted circuit whose inputs are available.  New
// circuits are admitted between ticks as pool slots free up (admission by
// device memory), so their first layer shares a launch with other circuits'
// later layers.  Results are bit-identical whatever the batch composition:
// each ciphertext's bootstrap is computed independently of its neighbours.
//
// Pipelining.  Ticks run in order on the context's stream, so a tick may use
// the outputs of the tick before it without the host waiting for them: a
// gate is schedulable as soon as all its inputs are scheduled.  The host
// builds and enqueues tick k + 1 (admission, readiness, index staging) while
// tick k runs on the device; at most two ticks are in flight, each with its
// own pinned staging buffers.  Readiness is incremental: every gate counts
// its unscheduled inputs and joins the ready queue when the count reaches
// zero, so a tick costs time in proportion to the gates it schedules, not to
// the gates of all active circuits.  A tick's completion is observed through
// its events: the first step() that finds them complete retires the tick --
// latencies from the device timestamps, outputs of the circuits it finished
// (gathered on the device and copied back in one transfer inside the tick),
// pool slots freed -- so one retire handles any number of circuits.
//
// Gates: the ten two-input bootstrapped gates (tfhe_gpu_gate ids 0..9), MUX
// (id 10, upstream bootsMUX: two bootstraps without key switch, one key
// switch), NOT (11) and COPY (12) without bootstrapping, CONSTANT (13, in0 =
// the bit).  Wire ids: [0, ninputs) are the circuit's inputs, ninputs + g is
// the output of gate g; gates must be listed in an order where each gate's
// inputs come earlier.  NOT / COPY / CONSTANT run at the start of a tick, in
// levels, so bootstrapped gates of the same tick may read them.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/tfhe_gpu.h"
#include "ctx.h"
#include "engine.h"

using namespace tfhe_gb300;

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

__global__ void k_gather(const int32_t* __restrict__ pool, const int32_t* __restrict__ idx,
                         int32_t* __restrict__ out, int width, int count) {
    const size_t total = (size_t)count * width;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / width, c = i - r * width;
        out[i] = pool[(size_t)idx[r] * width + c];
    }
}

__global__ void k_scatter(const int32_t* __restrict__ in, const int32_t* __restrict__ idx,
                          int32_t* __restrict__ pool, int width, int count) {
    const size_t total = (size_t)count * width;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / width, c = i - r * width;
        pool[(size_t)idx[r] * width + c] = in[i];
    }
}

// NOT / COPY / CONSTANT in place on pool slots: out = sign * in (+ const)
__global__ void k_linear(int32_t* __restrict__ pool, const int32_t* __restrict__ ops, int width,
                         int count) {
    // ops: count x 3 (dst slot, src slot or -1, mode: 0 copy, 1 negate, 2 const +mu, 3 const -mu)
    const size_t total = (size_t)count * width;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / width, c = i - r * width;
        const int dst = ops[3 * r], src = ops[3 * r + 1], mode = ops[3 * r + 2];
        int32_t v = 0;
        if (mode == 0) v = pool[(size_t)src * width + c];
        else if (mode == 1) v = (int32_t)(0u - (uint32_t)pool[(size_t)src * width + c]);
        else if (c == (size_t)width - 1) v = mode == 2 ? (1 << 29) : -(1 << 29);
        pool[(size_t)dst * width + c] = v;
    }
}

// Latency records keep the most recent kLatencyKeep entries of each kind
// (a long-running server would otherwise grow them without bound).
constexpr size_t kLatencyKeep = size_t(1) << 22;

void record(std::vector<double>& v, double x) {
    if (v.size() >= 2 * kLatencyKeep) v.erase(v.begin(), v.end() - kLatencyKeep);
    v.push_back(x);
}

int grid_for(size_t total) {
    size_t b = (total + 255) / 256;
    return (int)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

constexpr int kInFlight = 2;  // ticks in flight (staging buffers)

struct Gate {
    int32_t type, in[3];
};

int n_inputs(int32_t type) { return type == 10 ? 3 : (type <= 9 ? 2 : (type == 13 ? 0 : 1)); }
bool is_linear(int32_t type) { return type >= 11; }

struct Circuit {
    int64_t id;
    std::vector<Gate> gates;
    int32_t ninputs;
    std::vector<int32_t> outputs;        // wire ids
    std::vector<int32_t> input_ct;       // host copy until admitted
    std::vector<int32_t> slot;           // wire -> pool slot
    // readiness: users of each wire (CSR over wires), unscheduled inputs per gate
    std::vector<int32_t> user_off, users;
    std::vector<int32_t> pending;
    std::vector<int64_t> wire_tick;      // tick that produces the wire (-1: an input)
    std::vector<int32_t> wire_level;     // linear level within that tick (-1: a bootstrap)
    std::vector<double> produced;        // device completion time of the wire (s)
    int32_t unscheduled = 0;             // gates not yet in a tick
    double submitted = 0, admitted = 0, finished = 0;
    std::vector<int32_t> result;         // host result when finished
};

struct Pick {
    Circuit* c;
    int32_t g;
};

// One tick: what it runs, what it finishes, its events and staging.
struct Tick {
    std::vector<std::vector<Pick>> lin;         // linear gates by level
    std::vector<Pick> boot, mux;
    std::vector<Circuit*> finishing;            // circuits whose last gates are in this tick
    std::vector<int32_t> finishing_off;         // their first row in the result buffer
    cudaEvent_t start = nullptr, end = nullptr;
    int32_t* h_stage = nullptr;                 // pinned: indices, gate ids, uploads
    size_t h_stage_words = 0;
    int32_t* d_stage = nullptr;                 // device copy of h_stage
    size_t d_stage_words = 0;
    int32_t* h_res = nullptr;                   // pinned: finished circuits' outputs
    size_t h_res_words = 0;
    int32_t* d_res = nullptr;                   // device gather of those outputs
    size_t d_res_words = 0;
};

}  // namespace

struct tfhe_gpu_server {
    tfhe_gpu_ctx* ctx = nullptr;
    tfhe_gpu_form form = TFHE_GPU_SPLIT_FP32;
    int32_t width = 0;            // n + 1
    int32_t pool_slots = 0;
    int32_t max_batch = 0;
    int32_t ext_width = 0;        // kN + 1
    int32_t* d_pool = nullptr;    // pool_slots x width
    int32_t* d_a = nullptr;       // max_batch x width: gathered first operands
    int32_t* d_b = nullptr;       // max_batch x width: gathered second operands
    int32_t* d_x = nullptr;       // max_batch x width: gate combinations
    int32_t* d_u = nullptr;       // max_batch x ext_width: extracted samples
    int32_t* d_s = nullptr;       // max_batch/2 x ext_width: MUX sums
    int32_t* d_out = nullptr;     // max_batch x width: key-switched outputs
    std::vector<int32_t> free_slots;
    std::deque<std::unique_ptr<Circuit>> waiting;
    std::map<int64_t, std::unique_ptr<Circuit>> active;
    std::map<int64_t, std::unique_ptr<Circuit>> finished;
    std::deque<Pick> ready;                     // schedulable gates, in order of readiness
    std::vector<Circuit*> admitted_now;         // inputs to upload with the next tick
    Tick ticks[kInFlight];
    int64_t next_tick = 0;                      // index of the next tick to enqueue
    int64_t next_retire = 0;                    // index of the oldest tick not retired
    cudaEvent_t epoch = nullptr;                // device time origin
    double epoch_host = 0;
    int64_t next_id = 1;
    // statistics
    std::vector<double> gate_latency;   // per bootstrapped gate: inputs available -> done (s)
    std::vector<double> request_latency;
    int64_t gates_run = 0;
    double busy_s = 0;
    std::string last_error;
};

namespace {

tfhe_gpu_status srv_fail(tfhe_gpu_server* s, tfhe_gpu_status st, const std::string& m) {
    if (s) s->last_error = m;
    return st;
}

#define SCK(s, expr)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return srv_fail(s, e_ == cudaErrorMemoryAllocation ? TFHE_GPU_OOM : TFHE_GPU_DEVICE_ERROR, \
                            std::string(#expr) + ": " + cudaGetErrorString(e_));           \
    } while (0)

// grow a pinned host buffer (only while no transfer uses it)
cudaError_t grow_host(int32_t** p, size_t* have, size_t need) {
    if (need <= *have) return cudaSuccess;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *have = 0;
    size_t cap = std::max(need, (size_t)1 << 16);
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(p), cap * sizeof(int32_t), cudaHostAllocDefault);
    if (e == cudaSuccess) *have = cap;
    return e;
}

// grow a device buffer (only while no kernel uses it)
cudaError_t grow_dev(int32_t** p, size_t* have, size_t need) {
    if (need <= *have) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    size_t cap = std::max(need, (size_t)1 << 16);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), cap * sizeof(int32_t));
    if (e == cudaSuccess) *have = cap;
    return e;
}

double device_time(tfhe_gpu_server* s, cudaEvent_t ev) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->epoch, ev);
    return s->epoch_host + 1e-3 * ms;
}

// the gate's output wire is scheduled: its users lose one pending input
template <typename F>
void release_users(Circuit* c, int32_t g, F&& on_ready) {
    const int32_t w = c->ninputs + g;
    for (int32_t i = c->user_off[w]; i < c->user_off[w + 1]; ++i) {
        const int32_t u = c->users[i];
        if (--c->pending[u] == 0) on_ready(u);
    }
}

// Retire the oldest in-flight tick (its events have completed): device
// completion time, latencies, wire availability times, finished circuits.
tfhe_gpu_status retire_tick(tfhe_gpu_server* s, Tick& T) {
    const double t_end = device_time(s, T.end);
    float busy_ms = 0.f;
    cudaEventElapsedTime(&busy_ms, T.start, T.end);
    s->busy_s += 1e-3 * busy_ms;
    auto avail = [&](const Circuit* c, const Gate& G) {
        double r = c->admitted;
        for (int k = 0; k < n_inputs(G.type); ++k) r = std::max(r, c->produced[G.in[k]]);
        return r;
    };
    for (auto& level : T.lin)  // levels in order: a linear output is available with its inputs
        for (const Pick& p : level) p.c->produced[p.c->ninputs + p.g] = avail(p.c, p.c->gates[p.g]);
    for (auto* list : {&T.boot, &T.mux})
        for (const Pick& p : *list) {
            record(s->gate_latency, t_end - avail(p.c, p.c->gates[p.g]));
            p.c->produced[p.c->ninputs + p.g] = t_end;
        }
    const int32_t W = s->width;
    for (size_t i = 0; i < T.finishing.size(); ++i) {
        Circuit* c = T.finishing[i];
        c->result.assign(T.h_res + (size_t)T.finishing_off[i] * W,
                         T.h_res + (size_t)(T.finishing_off[i] + c->outputs.size()) * W);
        for (int32_t sl : c->slot) s->free_slots.push_back(sl);
        c->finished = t_end;
        record(s->request_latency, c->finished - c->submitted);
        auto it = s->active.find(c->id);
        s->finished[c->id] = std::move(it->second);
        s->active.erase(it);
    }
    T.lin.clear();
    T.boot.clear();
    T.mux.clear();
    T.finishing.clear();
    T.finishing_off.clear();
    ++s->next_retire;
    return TFHE_GPU_OK;
}

// Retire completed ticks in order; with `wait`, block for the oldest one.
tfhe_gpu_status retire(tfhe_gpu_server* s, bool wait) {
    while (s->next_retire < s->next_tick) {
        Tick& T = s->ticks[s->next_retire % kInFlight];
        cudaError_t e = wait ? cudaEventSynchronize(T.end) : cudaEventQuery(T.end);
        if (e == cudaErrorNotReady) return TFHE_GPU_OK;
        SCK(s, e);
        tfhe_gpu_status st = retire_tick(s, T);
        if (st != TFHE_GPU_OK) return st;
        wait = false;
    }
    return TFHE_GPU_OK;
}

// admit waiting circuits while their wires fit in the pool
void admit(tfhe_gpu_server* s) {
    while (!s->waiting.empty()) {
        Circuit* c = s->waiting.front().get();
        const size_t need = c->slot.size();
        if (need > s->free_slots.size()) break;
        for (size_t w = 0; w < need; ++w) {
            c->slot[w] = s->free_slots.back();
            s->free_slots.pop_back();
        }
        c->admitted = now_s();
        for (int32_t g = 0; g < (int32_t)c->gates.size(); ++g)
            if (c->pending[g] == 0) s->ready.push_back({c, g});
        s->admitted_now.push_back(c);
        s->active[c->id] = std::move(s->waiting.front());
        s->waiting.pop_front();
    }
}

// Choose the gates of tick k from the ready queue.
void schedule(tfhe_gpu_server* s, Tick& T, int64_t k) {
    std::deque<Pick> keep, next;
    int32_t slots = 0;  // bootstraps in this tick
    while (!s->ready.empty()) {
        const Pick p = s->ready.front();
        s->ready.pop_front();
        Circuit* c = p.c;
        const Gate& G = c->gates[p.g];
        const int32_t out = c->ninputs + p.g;
        if (is_linear(G.type)) {
            int lvl = 0;
            for (int q = 0; q < n_inputs(G.type); ++q) {
                const int32_t w = G.in[q];
                if (c->wire_tick[w] == k && c->wire_level[w] >= 0) lvl = std::max(lvl, c->wire_level[w] + 1);
            }
            if ((int)T.lin.size() <= lvl) T.lin.resize(lvl + 1);
            T.lin[lvl].push_back(p);
            c->wire_tick[out] = k;
            c->wire_level[out] = lvl;
            // a linear output is available within the tick
            release_users(c, p.g, [&](int32_t u) { s->ready.push_back({c, u}); });
        } else {
            const int need = G.type == 10 ? 2 : 1;
            if (slots + need > s->max_batch) {
                keep.push_back(p);
                continue;
            }
            slots += need;
            (G.type == 10 ? T.mux : T.boot).push_back(p);
            c->wire_tick[out] = k;
            c->wire_level[out] = -1;
            // a bootstrap's output is available to the next tick
            release_users(c, p.g, [&](int32_t u) { next.push_back({c, u}); });
        }
        if (--c->unscheduled == 0) T.finishing.push_back(c);
    }
    s->ready = std::move(keep);
    for (const Pick& p : next) s->ready.push_back(p);
}

// Enqueue tick T: uploads of newly admitted circuits, linear levels, the
// bootstraps, scatter, the finished circuits' outputs back to the host.
tfhe_gpu_status enqueue(tfhe_gpu_server* s, Tick& T) {
    tfhe_gpu_ctx* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const int32_t W = s->width, EW = s->ext_width;
    // staging layout (int32 words): [upload slots][linear ops 3 x nl]
    // [a, b, destination slots 3 x nb][gate ids nb][result slots][upload ciphertexts]
    size_t n_up = 0;
    for (Circuit* c : s->admitted_now) n_up += c->ninputs;
    size_t nl = 0;
    for (auto& level : T.lin) nl += level.size();
    const int32_t nr = (int32_t)T.boot.size(), nm = (int32_t)T.mux.size();
    const int32_t nb = nr + 2 * nm;
    size_t n_res = 0;
    for (Circuit* c : T.finishing) {
        T.finishing_off.push_back((int32_t)n_res);
        n_res += c->outputs.size();
    }
    const size_t o_lin = n_up, o_idx = o_lin + 3 * nl, o_gid = o_idx + 3 * (size_t)nb;
    const size_t o_res = o_gid + nb, o_ct = o_res + n_res;
    const size_t words = o_ct + n_up * W;
    SCK(s, grow_host(&T.h_stage, &T.h_stage_words, words));
    SCK(s, grow_dev(&T.d_stage, &T.d_stage_words, words));
    SCK(s, grow_host(&T.h_res, &T.h_res_words, n_res * W));
    SCK(s, grow_dev(&T.d_res, &T.d_res_words, n_res * W));
    int32_t* h = T.h_stage;
    {
        size_t i = 0;
        for (Circuit* c : s->admitted_now) {
            for (int32_t q = 0; q < c->ninputs; ++q) h[i + q] = c->slot[q];
            std::memcpy(h + o_ct + i * W, c->input_ct.data(), sizeof(int32_t) * (size_t)c->ninputs * W);
            i += c->ninputs;
            c->input_ct.clear();
            c->input_ct.shrink_to_fit();
        }
    }
    {
        size_t i = 0;
        for (auto& level : T.lin)
            for (const Pick& p : level) {
                const Gate& G = p.c->gates[p.g];
                h[o_lin + 3 * i] = p.c->slot[p.c->ninputs + p.g];
                h[o_lin + 3 * i + 1] = G.type == 13 ? -1 : p.c->slot[G.in[0]];
                h[o_lin + 3 * i + 2] = G.type == 12 ? 0 : (G.type == 11 ? 1 : (G.in[0] ? 2 : 3));
                ++i;
            }
    }
    // bootstraps: [plain gates | MUX first halves AND(a, b) | MUX second
    // halves ANDNY(a, c)]; the MUX halves are summed with (0, 1/8) before
    // their key switch (upstream bootsMUX)
    int32_t* ha = h + o_idx;
    int32_t* hb = ha + nb;
    int32_t* hd = hb + nb;
    int32_t* hg = h + o_gid;
    for (int32_t i = 0; i < nr; ++i) {
        const Pick& p = T.boot[i];
        const Gate& G = p.c->gates[p.g];
        ha[i] = p.c->slot[G.in[0]];
        hb[i] = p.c->slot[G.in[1]];
        hg[i] = G.type;
        hd[i] = p.c->slot[p.c->ninputs + p.g];
    }
    for (int32_t j = 0; j < nm; ++j) {
        const Pick& p = T.mux[j];
        const Gate& G = p.c->gates[p.g];
        const int32_t* sl = p.c->slot.data();
        ha[nr + j] = sl[G.in[0]];
        hb[nr + j] = sl[G.in[1]];
        hg[nr + j] = TFHE_GATE_AND;
        ha[nr + nm + j] = sl[G.in[0]];
        hb[nr + nm + j] = sl[G.in[2]];
        hg[nr + nm + j] = TFHE_GATE_ANDNY;
        hd[nr + j] = sl[p.c->ninputs + p.g];
    }
    {
        size_t i = 0;
        for (Circuit* c : T.finishing)
            for (int32_t w : c->outputs) h[o_res + i++] = c->slot[w];
    }
    s->admitted_now.clear();

    SCK(s, cudaEventRecord(T.start, st));
    SCK(s, cudaMemcpyAsync(T.d_stage, h, sizeof(int32_t) * words, cudaMemcpyHostToDevice, st));
    const int32_t* d = T.d_stage;
    if (n_up) {
        k_scatter<<<grid_for(n_up * W), 256, 0, st>>>(d + o_ct, d, s->d_pool, W, (int)n_up);
        SCK(s, cudaGetLastError());
    }
    {
        size_t off = 0;
        for (auto& level : T.lin) {
            k_linear<<<grid_for(level.size() * W), 256, 0, st>>>(s->d_pool, d + o_lin + 3 * off, W,
                                                                 (int)level.size());
            SCK(s, cudaGetLastError());
            off += level.size();
        }
    }
    if (nb > 0) {
        const int grid = grid_for((size_t)nb * W);
        k_gather<<<grid, 256, 0, st>>>(s->d_pool, d + o_idx, s->d_a, W, nb);
        k_gather<<<grid, 256, 0, st>>>(s->d_pool, d + o_idx + nb, s->d_b, W, nb);
        SCK(s, cudaGetLastError());
        SCK(s, launch_gate_combine(ctx->dp, d + o_gid, 0, s->d_a, s->d_b, s->d_x, nb, st));
        EpArgs a{};
        a.err = ctx->d_err;
        a.mu = 1 << 29;
        a.gsw = ctx->d_bk[s->form];
        // the automatic split-FP32 shape in its fixed summation order, so a
        // circuit's ciphertexts do not depend on the requests it shares
        // ticks with
        const int groups = s->form == TFHE_GPU_SPLIT_FP32 && ctx->groups_per_cta[s->form] == 0
                               ? 15 : ctx->groups_per_cta[s->form];
        // As in a gate batch: when the blind rotation splits into full waves
        // and a remainder wave on part of the SMs, the full waves' plain-gate
        // key switch runs on the side stream during the remainder.
        const int split = blind_rotate_tail_start((Form)s->form, groups, nb);
        const int k1 = std::min(split, nr);
        auto rotate = [&](int off, int cnt) -> cudaError_t {
            EpArgs b = a;
            b.x = s->d_x + (size_t)off * W;
            b.lwe_out = s->d_u + (size_t)off * EW;
            b.count = cnt;
            return launch_external_product(ctx->dp, (Form)s->form, kEpBlindRotate, ctx->tables, b,
                                           groups, st);
        };
        SCK(s, rotate(0, split ? split : nb));
        if (split && k1 > 0) {
            SCK(s, cudaEventRecord(ctx->ev_fork, st));
            SCK(s, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
            SCK(s, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, s->d_u, s->d_out, k1, ctx->side));
            SCK(s, cudaEventRecord(ctx->ev_join, ctx->side));
        }
        if (split) SCK(s, rotate(split, nb - split));
        const int k0 = split && k1 > 0 ? k1 : 0;
        SCK(s, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, s->d_u + (size_t)k0 * EW,
                                s->d_out + (size_t)k0 * W, nr - k0, st));
        if (nm) {
            SCK(s, launch_lwe_add2_const(s->d_u + (size_t)nr * EW, s->d_u + (size_t)(nr + nm) * EW,
                                         s->d_s, EW, 1 << 29, nm, st));
            SCK(s, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, s->d_s,
                                    s->d_out + (size_t)nr * W, nm, st));
        }
        if (split && k1 > 0) SCK(s, cudaStreamWaitEvent(st, ctx->ev_join, 0));
        k_scatter<<<grid_for((size_t)(nr + nm) * W), 256, 0, st>>>(s->d_out, d + o_idx + 2 * nb, s->d_pool,
                                                                     W, nr + nm);
        SCK(s, cudaGetLastError());
    }
    if (n_res) {
        k_gather<<<grid_for(n_res * W), 256, 0, st>>>(s->d_pool, d + o_res, T.d_res, W, (int)n_res);
        SCK(s, cudaGetLastError());
        SCK(s, cudaMemcpyAsync(T.h_res, T.d_res, sizeof(int32_t) * n_res * W, cudaMemcpyDeviceToHost, st));
    }
    SCK(s, cudaEventRecord(T.end, st));
    s->gates_run += nb;
    return TFHE_GPU_OK;
}

}  // namespace

extern "C" {

tfhe_gpu_status tfhe_gpu_server_create(tfhe_gpu_ctx* ctx, int32_t pool_slots, int32_t max_batch,
                                       tfhe_gpu_form form, tfhe_gpu_server** out) {
    if (!ctx || !out || pool_slots < 4 || max_batch < 2 ||
        (form != TFHE_GPU_FP64 && form != TFHE_GPU_SPLIT_FP32))
        return TFHE_GPU_BAD_PARAM;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return TFHE_GPU_DEVICE_ERROR;
    tfhe_gpu_server* s = new tfhe_gpu_server();
    s->ctx = ctx;
    s->form = form;
    s->width = ctx->P.n + 1;
    s->pool_slots = pool_slots;
    s->max_batch = max_batch;
    s->ext_width = ctx->P.k * ctx->P.N + 1;
    const size_t lw = (size_t)s->width * sizeof(int32_t);
    const size_t ew = (size_t)s->ext_width * sizeof(int32_t);
    bool ok = cudaMalloc(&s->d_pool, lw * pool_slots) == cudaSuccess &&
              cudaMalloc(&s->d_a, lw * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_b, lw * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_x, lw * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_u, ew * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_s, ew * (max_batch / 2 + 1)) == cudaSuccess &&
              cudaMalloc(&s->d_out, lw * max_batch) == cudaSuccess &&
              cudaEventCreate(&s->epoch) == cudaSuccess;
    for (Tick& T : s->ticks)
        ok = ok && cudaEventCreate(&T.start) == cudaSuccess && cudaEventCreate(&T.end) == cudaSuccess;
    if (ok) ok = cudaEventRecord(s->epoch, ctx->stream) == cudaSuccess &&
                 cudaEventSynchronize(s->epoch) == cudaSuccess;
    s->epoch_host = now_s();
    if (!ok) {
        tfhe_gpu_server_destroy(s);
        return TFHE_GPU_OOM;
    }
    s->free_slots.reserve(pool_slots);
    for (int32_t i = pool_slots - 1; i >= 0; --i) s->free_slots.push_back(i);
    *out = s;
    return TFHE_GPU_OK;
}

void tfhe_gpu_server_destroy(tfhe_gpu_server* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    cudaStreamSynchronize(s->ctx->side);
    cudaFree(s->d_pool);
    cudaFree(s->d_a);
    cudaFree(s->d_b);
    cudaFree(s->d_x);
    cudaFree(s->d_u);
    cudaFree(s->d_s);
    cudaFree(s->d_out);
    for (Tick& T : s->ticks) {
        if (T.start) cudaEventDestroy(T.start);
        if (T.end) cudaEventDestroy(T.end);
        if (T.h_stage) cudaFreeHost(T.h_stage);
        if (T.h_res) cudaFreeHost(T.h_res);
        cudaFree(T.d_stage);
        cudaFree(T.d_res);
    }
    if (s->epoch) cudaEventDestroy(s->epoch);
    delete s;
}

const char* tfhe_gpu_server_last_error(const tfhe_gpu_server* s) {
    return s ? s->last_error.c_str() : "null server";
}

tfhe_gpu_status tfhe_gpu_server_submit(tfhe_gpu_server* s, const int32_t* gates, int32_t ngates,
                                       int32_t ninputs, const int32_t* input_ct,
                                       const int32_t* output_wires, int32_t noutputs,
                                       int64_t* request_id) {
    if (!s || ngates < 0 || ninputs < 0 || noutputs < 1 || !output_wires || !request_id ||
        (ngates && !gates) || (ninputs && !input_ct))
        return TFHE_GPU_BAD_PARAM;
    const int32_t nwires = ninputs + ngates;
    if (nwires > s->pool_slots)
        return srv_fail(s, TFHE_GPU_BAD_PARAM, "circuit has more wires than the pool has slots");
    auto c = std::make_unique<Circuit>();
    c->ninputs = ninputs;
    c->gates.resize(ngates);
    c->pending.assign(ngates, 0);
    std::vector<int32_t> nuse(nwires + 1, 0);
    for (int32_t g = 0; g < ngates; ++g) {
        Gate& G = c->gates[g];
        G.type = gates[4 * g];
        for (int k = 0; k < 3; ++k) G.in[k] = gates[4 * g + 1 + k];
        if (G.type < 0 || G.type > 13) return srv_fail(s, TFHE_GPU_BAD_PARAM, "unknown gate type");
        for (int k = 0; k < n_inputs(G.type); ++k) {
            if (G.in[k] < 0 || G.in[k] >= ninputs + g)
                return srv_fail(s, TFHE_GPU_BAD_PARAM, "gate input must be an earlier wire");
            if (G.in[k] >= ninputs) {  // another gate's output: pending until it is scheduled
                ++c->pending[g];
                ++nuse[G.in[k]];
            }
        }
    }
    if (ngates == 0)
        return srv_fail(s, TFHE_GPU_BAD_PARAM, "circuit has no gates (its outputs are its inputs)");
    for (int32_t o = 0; o < noutputs; ++o)
        if (output_wires[o] < 0 || output_wires[o] >= nwires)
            return srv_fail(s, TFHE_GPU_BAD_PARAM, "bad output wire");
    c->user_off.assign(nwires + 1, 0);
    for (int32_t w = 0; w < nwires; ++w) c->user_off[w + 1] = c->user_off[w] + nuse[w];
    c->users.resize(c->user_off[nwires]);
    std::vector<int32_t> fill(c->user_off.begin(), c->user_off.end() - 1);
    for (int32_t g = 0; g < ngates; ++g)
        for (int k = 0; k < n_inputs(c->gates[g].type); ++k)
            if (c->gates[g].in[k] >= ninputs) c->users[fill[c->gates[g].in[k]]++] = g;
    c->id = s->next_id++;
    c->outputs.assign(output_wires, output_wires + noutputs);
    c->input_ct.assign(input_ct, input_ct + (size_t)ninputs * s->width);
    c->slot.assign(nwires, -1);
    c->wire_tick.assign(nwires, -1);
    c->wire_level.assign(nwires, -1);
    c->produced.assign(nwires, 0.0);
    c->unscheduled = ngates;
    c->submitted = now_s();
    *request_id = c->id;
    s->waiting.push_back(std::move(c));
    return TFHE_GPU_OK;
}

// One tick: retire completed ticks, admit circuits that fit, schedule every
// schedulable gate (up to max_batch bootstraps) and enqueue it as one batch
// without waiting for the device.  With two ticks already in flight it first
// waits for the older; with nothing to schedule it waits for the oldest tick
// in flight, so a loop of steps makes progress.  *ran = gates enqueued.
tfhe_gpu_status tfhe_gpu_server_step(tfhe_gpu_server* s, int32_t* ran) {
    if (!s) return TFHE_GPU_BAD_PARAM;
    if (ran) *ran = 0;
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return TFHE_GPU_DEVICE_ERROR;
    tfhe_gpu_status st = retire(s, false);
    if (st != TFHE_GPU_OK) return st;
    admit(s);
    if (s->ready.empty() && s->admitted_now.empty()) {
        // nothing to run: wait for the oldest tick in flight, if any
        return retire(s, true);
    }
    if (s->next_tick - s->next_retire >= kInFlight) {
        st = retire(s, true);  // frees the staging of tick next_tick - kInFlight
        if (st != TFHE_GPU_OK) return st;
        admit(s);
    }
    Tick& T = s->ticks[s->next_tick % kInFlight];
    schedule(s, T, s->next_tick);
    int32_t n = (int32_t)(T.boot.size() + T.mux.size());
    for (auto& level : T.lin) n += (int32_t)level.size();
    st = enqueue(s, T);
    if (st != TFHE_GPU_OK) return st;
    ++s->next_tick;
    if (ran) *ran = n;
    return TFHE_GPU_OK;
}

// Collect a finished request's output ciphertexts (noutputs x (n+1)).
// *done = 0 while it is still queued or running.
tfhe_gpu_status tfhe_gpu_server_poll(tfhe_gpu_server* s, int64_t request_id, int32_t* out,
                                     int32_t* done, double* latency_s) {
    if (!s || !done) return TFHE_GPU_BAD_PARAM;
    auto it = s->finished.find(request_id);
    if (it == s->finished.end()) {
        *done = 0;
        return TFHE_GPU_OK;
    }
    Circuit* c = it->second.get();
    if (out) std::memcpy(out, c->result.data(), sizeof(int32_t) * c->result.size());
    if (latency_s) *latency_s = c->finished - c->submitted;
    *done = 1;
    s->finished.erase(it);
    return TFHE_GPU_OK;
}

// stats[0..7] = queued circuits, active circuits, free pool slots,
// bootstraps run, busy seconds, recorded gate latencies, recorded request
// latencies, pool slots.  Latency arrays are copied when the pointers are
// non-null (up to *cap entries each; *cap returns the counts).
tfhe_gpu_status tfhe_gpu_server_stats(tfhe_gpu_server* s, double* stats, double* gate_lat,
                                      double* req_lat, int64_t* cap) {
    if (!s || !stats) return TFHE_GPU_BAD_PARAM;
    stats[0] = (double)s->waiting.size();
    stats[1] = (double)s->active.size();
    stats[2] = (double)s->free_slots.size();
    stats[3] = (double)s->gates_run;
    stats[4] = s->busy_s;
    stats[5] = (double)s->gate_latency.size();
    stats[6] = (double)s->request_latency.size();
    stats[7] = (double)s->pool_slots;
    if (cap) {
        const int64_t c0 = cap[0], c1 = cap[1];
        if (gate_lat)
            for (int64_t i = 0; i < c0 && i < (int64_t)s->gate_latency.size(); ++i) gate_lat[i] = s->gate_latency[i];
        if (req_lat)
            for (int64_t i = 0; i < c1 && i < (int64_t)s->request_latency.size(); ++i) req_lat[i] = s->request_latency[i];
        cap[0] = (int64_t)s->gate_latency.size();
        cap[1] = (int64_t)s->request_latency.size();
    }
    return TFHE_GPU_OK;
}

}  // extern "C"
