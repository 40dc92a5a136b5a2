// server.cu -- continuous-batching gate server over one engine context.
//
// The reference's test_bench server (test_bench/server/cloud.c:39-74) loads a
// cloud key, reads ciphertexts, runs a circuit gate by gate (bootsOR,
// bootsXNOR, bootsMUX; cloud.c:9-36) and writes the results.  This is that
// server as a request loop: many clients submit circuits (gate lists over
// their input ciphertexts); the server keeps every admitted circuit's wires
// resident in a device ciphertext pool, and each tick runs, as one batch,
// every gate of every admitted circuit whose inputs are ready.  New circuits
// are admitted between ticks as pool slots free up (admission by device
// memory), so their first layer shares a launch with other circuits' later
// layers.  Results are bit-identical whatever the batch composition: each
// ciphertext's bootstrap is computed independently of its neighbours.
//
// Gates: the ten two-input bootstrapped gates (tfhe_gpu_gate ids 0..9), MUX
// (id 10, upstream bootsMUX: two bootstraps without key switch, one key
// switch), NOT (11) and COPY (12) without bootstrapping, CONSTANT (13, in0 =
// the bit).  Wire ids: [0, ninputs) are the circuit's inputs, ninputs + g is
// the output of gate g; gates must be listed in an order where each gate's
// inputs come earlier.
#include <cuda_runtime.h>

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

struct Gate {
    int32_t type, in[3];
};

struct Circuit {
    int64_t id;
    std::vector<Gate> gates;
    int32_t ninputs;
    std::vector<int32_t> outputs;        // wire ids
    std::vector<int32_t> input_ct;       // host copy until admitted
    std::vector<int32_t> slot;           // wire -> pool slot
    std::vector<char> ready;             // wire ready
    std::vector<char> done;              // gate done
    std::vector<char> queued;            // gate in the ready list
    std::vector<double> ready_at;        // gate became ready (s)
    int32_t remaining = 0;
    double submitted = 0, admitted = 0, finished = 0;
    std::vector<int32_t> result;         // host result when finished
    bool is_done = false;
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
    int32_t* d_gates = nullptr;   // max_batch gate ids of the bootstraps
    int32_t* d_idx = nullptr;     // 3 x max_batch (a slots, b slots, destination slots)
    int32_t* d_lin = nullptr;     // 3 x max_batch
    int32_t* h_idx = nullptr;     // pinned staging, 4 x max_batch
    std::vector<int32_t> free_slots;
    std::deque<std::unique_ptr<Circuit>> waiting;
    std::map<int64_t, std::unique_ptr<Circuit>> active;
    std::map<int64_t, std::unique_ptr<Circuit>> finished;
    int64_t next_id = 1;
    // statistics
    std::vector<double> gate_latency;   // per bootstrapped gate: ready -> done (s)
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

bool is_boot(int32_t t) { return t >= 0 && t <= 10; }

// admit waiting circuits while their wires fit in the pool
tfhe_gpu_status admit(tfhe_gpu_server* s) {
    cudaStream_t st = s->ctx->stream;
    while (!s->waiting.empty()) {
        Circuit* c = s->waiting.front().get();
        const size_t need = c->slot.size();
        if (need > s->free_slots.size()) break;
        for (size_t w = 0; w < need; ++w) {
            c->slot[w] = s->free_slots.back();
            s->free_slots.pop_back();
        }
        // upload inputs (one copy per input; inputs are contiguous on the host)
        for (int32_t i = 0; i < c->ninputs; ++i) {
            SCK(s, cudaMemcpyAsync(s->d_pool + (size_t)c->slot[i] * s->width,
                                   c->input_ct.data() + (size_t)i * s->width,
                                   sizeof(int32_t) * s->width, cudaMemcpyHostToDevice, st));
            c->ready[i] = 1;
        }
        c->admitted = now_s();
        s->active[c->id] = std::move(s->waiting.front());
        s->waiting.pop_front();
    }
    return TFHE_GPU_OK;
}

}  // namespace

extern "C" {

tfhe_gpu_status tfhe_gpu_server_create(tfhe_gpu_ctx* ctx, int32_t pool_slots, int32_t max_batch,
                                       tfhe_gpu_form form, tfhe_gpu_server** out) {
    if (!ctx || !out || pool_slots < 4 || max_batch < 1 ||
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
              cudaMalloc(&s->d_gates, sizeof(int32_t) * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_idx, sizeof(int32_t) * 3 * max_batch) == cudaSuccess &&
              cudaMalloc(&s->d_lin, sizeof(int32_t) * 3 * max_batch) == cudaSuccess &&
              cudaMallocHost(&s->h_idx, sizeof(int32_t) * 4 * max_batch) == cudaSuccess;
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
    cudaFree(s->d_pool);
    cudaFree(s->d_a);
    cudaFree(s->d_b);
    cudaFree(s->d_x);
    cudaFree(s->d_u);
    cudaFree(s->d_s);
    cudaFree(s->d_out);
    cudaFree(s->d_gates);
    cudaFree(s->d_idx);
    cudaFree(s->d_lin);
    if (s->h_idx) cudaFreeHost(s->h_idx);
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
    c->id = s->next_id++;
    c->ninputs = ninputs;
    c->gates.resize(ngates);
    for (int32_t g = 0; g < ngates; ++g) {
        Gate& G = c->gates[g];
        G.type = gates[4 * g];
        for (int k = 0; k < 3; ++k) G.in[k] = gates[4 * g + 1 + k];
        const int nin = G.type == 10 ? 3 : (G.type <= 9 ? 2 : (G.type == 13 ? 0 : 1));
        if (G.type < 0 || G.type > 13) return srv_fail(s, TFHE_GPU_BAD_PARAM, "unknown gate type");
        for (int k = 0; k < nin; ++k)
            if (G.in[k] < 0 || G.in[k] >= ninputs + g)
                return srv_fail(s, TFHE_GPU_BAD_PARAM, "gate input must be an earlier wire");
    }
    for (int32_t o = 0; o < noutputs; ++o)
        if (output_wires[o] < 0 || output_wires[o] >= nwires)
            return srv_fail(s, TFHE_GPU_BAD_PARAM, "bad output wire");
    c->outputs.assign(output_wires, output_wires + noutputs);
    c->input_ct.assign(input_ct, input_ct + (size_t)ninputs * s->width);
    c->slot.assign(nwires, -1);
    c->ready.assign(nwires, 0);
    c->done.assign(ngates, 0);
    c->queued.assign(ngates, 0);
    c->ready_at.assign(ngates, 0.0);
    c->remaining = ngates;
    c->submitted = now_s();
    *request_id = c->id;
    s->waiting.push_back(std::move(c));
    return TFHE_GPU_OK;
}

// One scheduling tick: admit circuits that fit, run every ready gate of every
// admitted circuit (up to max_batch bootstraps) as one batch, retire finished
// circuits.  *ran = number of gates executed (0 when idle).
tfhe_gpu_status tfhe_gpu_server_step(tfhe_gpu_server* s, int32_t* ran) {
    if (!s) return TFHE_GPU_BAD_PARAM;
    if (ran) *ran = 0;
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return TFHE_GPU_DEVICE_ERROR;
    tfhe_gpu_status st0 = admit(s);
    if (st0 != TFHE_GPU_OK) return st0;
    cudaStream_t st = s->ctx->stream;
    const double t0 = now_s();
    // collect ready gates
    struct Pick {
        Circuit* c;
        int32_t g;
    };
    std::vector<Pick> boot, mux, lin;
    for (auto& kv : s->active) {
        Circuit* c = kv.second.get();
        for (int32_t g = 0; g < (int32_t)c->gates.size(); ++g) {
            if (c->done[g]) continue;
            const Gate& G = c->gates[g];
            const int nin = G.type == 10 ? 3 : (G.type <= 9 ? 2 : (G.type == 13 ? 0 : 1));
            bool rdy = true;
            for (int k = 0; k < nin; ++k) rdy = rdy && c->ready[G.in[k]];
            if (!rdy) continue;
            if (!c->queued[g]) {
                c->queued[g] = 1;
                c->ready_at[g] = t0;
            }
            if (G.type <= 9) {
                if ((int32_t)(boot.size() + 2 * mux.size()) + 1 <= s->max_batch) boot.push_back({c, g});
            } else if (G.type == 10) {
                if ((int32_t)(boot.size() + 2 * mux.size()) + 2 <= s->max_batch) mux.push_back({c, g});
            } else if ((int32_t)lin.size() < s->max_batch) {
                lin.push_back({c, g});
            }
        }
    }
    const int32_t W = s->width;
    int32_t* hi = s->h_idx;
    // linear gates first (no bootstrap): NOT, COPY, CONSTANT
    if (!lin.empty()) {
        for (size_t i = 0; i < lin.size(); ++i) {
            const Gate& G = lin[i].c->gates[lin[i].g];
            hi[3 * i] = lin[i].c->slot[lin[i].c->ninputs + lin[i].g];
            hi[3 * i + 1] = G.type == 13 ? -1 : lin[i].c->slot[G.in[0]];
            hi[3 * i + 2] = G.type == 12 ? 0 : (G.type == 11 ? 1 : (G.in[0] ? 2 : 3));
        }
        SCK(s, cudaMemcpyAsync(s->d_lin, hi, sizeof(int32_t) * 3 * lin.size(), cudaMemcpyHostToDevice, st));
        k_linear<<<grid_for(lin.size() * W), 256, 0, st>>>(s->d_pool, s->d_lin, W, (int)lin.size());
        SCK(s, cudaGetLastError());
        SCK(s, cudaStreamSynchronize(st));  // pinned staging is reused below
    }
    // All bootstraps of the tick in one blind-rotation launch.  Items:
    // [plain gates | MUX first halves AND(a, b) | MUX second halves
    // ANDNY(a, c)]; the MUX halves are summed with (0, 1/8) before their key
    // switch (upstream bootsMUX).
    const int32_t nr = (int32_t)boot.size(), nm = (int32_t)mux.size();
    const int32_t nb = nr + 2 * nm;
    if (nb > 0) {
        int32_t* ha = hi;
        int32_t* hb = hi + nb;
        int32_t* hd = hi + 2 * nb;
        int32_t* hg = hi + 3 * nb;
        for (int32_t i = 0; i < nr; ++i) {
            const Gate& G = boot[i].c->gates[boot[i].g];
            ha[i] = boot[i].c->slot[G.in[0]];
            hb[i] = boot[i].c->slot[G.in[1]];
            hg[i] = G.type;
            hd[i] = boot[i].c->slot[boot[i].c->ninputs + boot[i].g];
        }
        for (int32_t j = 0; j < nm; ++j) {
            const Gate& G = mux[j].c->gates[mux[j].g];
            const int32_t* sl = mux[j].c->slot.data();
            ha[nr + j] = sl[G.in[0]];
            hb[nr + j] = sl[G.in[1]];
            hg[nr + j] = TFHE_GATE_AND;
            ha[nr + nm + j] = sl[G.in[0]];
            hb[nr + nm + j] = sl[G.in[2]];
            hg[nr + nm + j] = TFHE_GATE_ANDNY;
            hd[nr + j] = sl[mux[j].c->ninputs + mux[j].g];
        }
        SCK(s, cudaMemcpyAsync(s->d_idx, hi, sizeof(int32_t) * 3 * nb, cudaMemcpyHostToDevice, st));
        SCK(s, cudaMemcpyAsync(s->d_gates, hg, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, st));
        const int grid = grid_for((size_t)nb * W);
        k_gather<<<grid, 256, 0, st>>>(s->d_pool, s->d_idx, s->d_a, W, nb);
        k_gather<<<grid, 256, 0, st>>>(s->d_pool, s->d_idx + nb, s->d_b, W, nb);
        SCK(s, cudaGetLastError());
        tfhe_gpu_ctx* ctx = s->ctx;
        SCK(s, launch_gate_combine(ctx->dp, s->d_gates, 0, s->d_a, s->d_b, s->d_x, nb, st));
        EpArgs a{};
        a.err = ctx->d_err;
        a.x = s->d_x;
        a.mu = 1 << 29;
        a.lwe_out = s->d_u;
        a.gsw = ctx->d_bk[s->form];
        a.count = nb;
        SCK(s, launch_external_product(ctx->dp, (Form)s->form, kEpBlindRotate, ctx->tables, a,
                                       ctx->groups_per_cta[s->form], st));
        const int32_t EW = s->ext_width;
        SCK(s, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, s->d_u, s->d_out, nr, st));
        if (nm) {
            SCK(s, launch_lwe_add2_const(s->d_u + (size_t)nr * EW, s->d_u + (size_t)(nr + nm) * EW,
                                         s->d_s, EW, 1 << 29, nm, st));
            SCK(s, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, s->d_s,
                                    s->d_out + (size_t)nr * W, nm, st));
        }
        const int sgrid = grid_for((size_t)(nr + nm) * W);
        k_scatter<<<sgrid, 256, 0, st>>>(s->d_out, s->d_idx + 2 * nb, s->d_pool, W, nr + nm);
        SCK(s, cudaGetLastError());
        SCK(s, cudaStreamSynchronize(st));
    }
    const double t1 = now_s();
    s->busy_s += t1 - t0;
    // mark done, record latencies
    auto mark = [&](std::vector<Pick>& picks, bool boots) {
        for (auto& p : picks) {
            p.c->done[p.g] = 1;
            p.c->ready[p.c->ninputs + p.g] = 1;
            p.c->remaining--;
            if (boots) record(s->gate_latency, t1 - p.c->ready_at[p.g]);
        }
    };
    mark(lin, false);
    mark(boot, true);
    mark(mux, true);
    s->gates_run += (int64_t)(boot.size() + mux.size() * 2);
    if (ran) *ran = (int32_t)(boot.size() + mux.size() + lin.size());
    // retire finished circuits: copy outputs back, free slots
    for (auto it = s->active.begin(); it != s->active.end();) {
        Circuit* c = it->second.get();
        if (c->remaining > 0) {
            ++it;
            continue;
        }
        c->result.resize((size_t)c->outputs.size() * W);
        for (size_t o = 0; o < c->outputs.size(); ++o)
            SCK(s, cudaMemcpyAsync(c->result.data() + o * W,
                                   s->d_pool + (size_t)c->slot[c->outputs[o]] * W,
                                   sizeof(int32_t) * W, cudaMemcpyDeviceToHost, st));
        SCK(s, cudaStreamSynchronize(st));
        for (int32_t sl : c->slot) s->free_slots.push_back(sl);
        c->finished = now_s();
        c->is_done = true;
        record(s->request_latency, c->finished - c->submitted);
        s->finished[c->id] = std::move(it->second);
        it = s->active.erase(it);
    }
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
