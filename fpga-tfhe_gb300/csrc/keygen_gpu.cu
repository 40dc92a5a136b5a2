// keygen_gpu.cu -- the arithmetic of bootstrapping-key generation on the
// device.  The host draws every random value in the reference's order
// (keygen.cpp, numeric-functions.cpp:11-34), so the keys are bit-identical
// to the host path; the n (k+1) l negacyclic products a * s (about 4 G
// integer multiply-adds for the default set) run here instead.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace tfhe_gb300 {
namespace {

constexpr int kMaxN = 1024;
constexpr int kMaxK = 2;

// One CTA per TGSW row: the row's masks and the TLWE key in shared memory,
// each thread accumulates N / blockDim.x coefficients of sum_i a_i * s_i.
__global__ void __launch_bounds__(256) k_tgsw_finish(int32_t* __restrict__ bk,
                                                     const int32_t* __restrict__ tlwe_key,
                                                     const int32_t* __restrict__ lwe_key, int N, int k,
                                                     int l, int Bgbit) {
    __shared__ uint32_t sa[kMaxK * kMaxN];
    __shared__ uint32_t sk[kMaxK * kMaxN];
    const int kpl = (k + 1) * l;
    const int row = blockIdx.x;
    int32_t* g = bk + (size_t)row * (k + 1) * N;
    for (int i = threadIdx.x; i < k * N; i += blockDim.x) {
        sa[i] = (uint32_t)g[i];
        sk[i] = (uint32_t)tlwe_key[i];
    }
    __syncthreads();
    const int p = row % kpl;
    const int pi = p / l, pj = p % l;
    const uint32_t message = (uint32_t)lwe_key[row / kpl] * (1u << (32 - (pj + 1) * Bgbit));
    for (int x = threadIdx.x; x < N; x += blockDim.x) {
        uint32_t acc = 0;
        for (int poly = 0; poly < k; ++poly) {
            const uint32_t* a = sa + poly * N;
            const uint32_t* key = sk + poly * N;
            // coefficient x of a * key: sum_j key[j] a[x - j], negated where x - j wraps
            for (int j = 0; j <= x; ++j) acc += key[j] * a[x - j];
            for (int j = x + 1; j < N; ++j) acc -= key[j] * a[x - j + N];
        }
        uint32_t b = (uint32_t)g[(size_t)k * N + x] + acc;
        if (x == 0 && pi == k) b += message;
        g[(size_t)k * N + x] = (int32_t)b;
        if (x == 0 && pi < k) g[(size_t)pi * N] = (int32_t)((uint32_t)g[(size_t)pi * N] + message);
    }
}

}  // namespace

cudaError_t launch_tgsw_finish(const DevParams& P, int32_t* bk, const int32_t* tlwe_key,
                               const int32_t* lwe_key, cudaStream_t st) {
    if (P.N > kMaxN || P.k > kMaxK) return cudaErrorInvalidValue;
    const int rows = P.n * (P.k + 1) * P.l;
    if (rows <= 0) return cudaSuccess;
    k_tgsw_finish<<<rows, 256, 0, st>>>(bk, tlwe_key, lwe_key, P.N, P.k, P.l, P.Bgbit);
    return cudaGetLastError();
}

}  // namespace tfhe_gb300
