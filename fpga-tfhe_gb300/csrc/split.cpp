// split.cpp -- one circuit layer over several engine contexts (GPUs).
//
// The gates of a layer are independent and the cloud key is read-only, so a
// layer shards without any exchange inside it: the gate list is cut into
// contiguous, balanced shards (sizes differ by at most one), shard i runs on
// context i -- normally one context per GPU, each holding its own copy of
// the keys -- and every shard writes its outputs straight into its slice of
// the caller's output array, which is the gather in layer order.  The shards
// run concurrently, one host thread per context, each through the
// host-buffer gate entry point (copies in, gates, copies out, on that
// context's device and stream).  Nothing crosses devices; the only exchange
// between layers is the caller's next input, as on one GPU.
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

extern "C" tfhe_gpu_status tfhe_gpu_bootsGates_host_split(tfhe_gpu_ctx* const* ctxs, int32_t nctx,
                                                          const int32_t* gates, int32_t uniform_gate,
                                                          int32_t* out, const int32_t* ca,
                                                          const int32_t* cb, int32_t count,
                                                          tfhe_gpu_form form) {
    if (!ctxs || nctx < 1 || count < 0) return TFHE_GPU_BAD_PARAM;
    for (int32_t i = 0; i < nctx; ++i) {
        if (!ctxs[i]) return TFHE_GPU_BAD_PARAM;
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) {  // a context serves one thread at a time
                ctxs[i]->last_error = "bootsGates_host_split: the same context appears twice";
                return TFHE_GPU_BAD_PARAM;
            }
        if (ctxs[i]->P.n != ctxs[0]->P.n) {
            ctxs[i]->last_error = "bootsGates_host_split: contexts with different parameters";
            return TFHE_GPU_BAD_PARAM;
        }
    }
    if (count == 0) return TFHE_GPU_OK;
    const size_t w = (size_t)ctxs[0]->P.n + 1;
    std::vector<tfhe_gpu_status> st(nctx, TFHE_GPU_OK);
    auto shard = [&](int32_t i) {
        const int32_t lo = (int32_t)((int64_t)count * i / nctx);
        const int32_t hi = (int32_t)((int64_t)count * (i + 1) / nctx);
        if (hi <= lo) return;
        st[i] = tfhe_gpu_bootsGates_host(ctxs[i], gates ? gates + lo : nullptr, uniform_gate,
                                         out + (size_t)lo * w, ca + (size_t)lo * w, cb + (size_t)lo * w,
                                         hi - lo, form);
    };
    std::vector<std::thread> threads;
    threads.reserve(nctx - 1);
    for (int32_t i = 1; i < nctx; ++i) threads.emplace_back(shard, i);
    shard(0);
    for (auto& t : threads) t.join();
    for (int32_t i = 0; i < nctx; ++i)
        if (st[i] != TFHE_GPU_OK) return st[i];  // the failing context's last_error says why
    return TFHE_GPU_OK;
}
