// keyswitch.cu -- batched LWE key switching (dimension kN -> n).
//
// Restates lweKeySwitch / lweKeySwitchTranslate_fromArray
// (kernel/src/lwe-keyswitch-functions.cpp:114-129, 228-241): start from
// (0, b); for each input coefficient a_i and digit level j take the
// base-2^basebit digit of a_i + 2^(32 - (1 + basebit t)) and subtract the
// table row KS[i][j][digit] (lweSubTo, lwe-functions.cpp:222-234) when the
// digit is non-zero.  Integer arithmetic, results are bit-exact.
//
// GB300 layout and schedule: the table is [kN][t][base][row_stride] int32
// with rows padded to a multiple of 4 words (16-byte loads).  A CTA owns G
// ciphertexts and walks the (i, j) pairs once; every thread holds four
// output coefficients of all G ciphertexts in registers and loads the
// base-1 non-zero rows of each (i, j) once for the whole group, so each
// table row read from L2 serves G ciphertexts.  The table (62 MB for the
// default set) stays L2-resident across the CTAs of a launch.
#include "engine.h"

namespace tfhe_gb300 {

namespace {

constexpr int kKsGroup = 8;      // ciphertexts per CTA
constexpr int kKsMaxBase = 4;    // basebit <= 2

__global__ void __launch_bounds__(256) k_keyswitch(const int32_t* __restrict__ ks, int row_stride,
                                                   const int32_t* __restrict__ in,
                                                   int32_t* __restrict__ out, int count, int n,
                                                   int n_in, int t, int basebit) {
    extern __shared__ __align__(16) uint32_t s_in[];  // kKsGroup x (n_in + 1)
    const int c0 = blockIdx.x * kKsGroup;
    const int G = min(kKsGroup, count - c0);
    const int w_in = n_in + 1;
    for (int i = threadIdx.x; i < G * w_in; i += blockDim.x)
        s_in[i] = (uint32_t)in[(size_t)c0 * w_in + i];
    __syncthreads();

    const int base = 1 << basebit;
    const uint32_t mask = (uint32_t)base - 1;
    const uint32_t prec_offset = 1u << (32 - (1 + basebit * t));
    const int nvec = (n + 1 + 3) >> 2;  // int4 chunks of a row
    const int v = threadIdx.x;
    const bool live = v < nvec;

    uint4 acc[kKsGroup];
#pragma unroll
    for (int g = 0; g < kKsGroup; ++g) acc[g] = make_uint4(0, 0, 0, 0);

    for (int i = 0; i < n_in; ++i) {
        for (int j = 0; j < t; ++j) {
            const int shift = 32 - (j + 1) * basebit;
            uint4 row[kKsMaxBase];
#pragma unroll
            for (int h = 0; h < kKsMaxBase; ++h) row[h] = make_uint4(0, 0, 0, 0);
            if (live) {
                const int4* rp =
                    reinterpret_cast<const int4*>(ks + ((size_t)(i * t + j) * base) * row_stride);
#pragma unroll
                for (int h = 1; h < kKsMaxBase; ++h) {
                    if (h < base) {
                        const int4 r = __ldg(rp + (size_t)h * (row_stride >> 2) + v);
                        row[h] = make_uint4((uint32_t)r.x, (uint32_t)r.y, (uint32_t)r.z,
                                            (uint32_t)r.w);
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < kKsGroup; ++g) {
                if (g >= G) break;
                const uint32_t aij = ((s_in[g * w_in + i] + prec_offset) >> shift) & mask;
#pragma unroll
                for (int h = 1; h < kKsMaxBase; ++h) {
                    const uint32_t m = (aij == (uint32_t)h) ? 0xffffffffu : 0u;
                    acc[g].x -= row[h].x & m;
                    acc[g].y -= row[h].y & m;
                    acc[g].z -= row[h].z & m;
                    acc[g].w -= row[h].w & m;
                }
            }
        }
    }
    if (!live) return;
    for (int g = 0; g < G; ++g) {
        int32_t* o = out + (size_t)(c0 + g) * (n + 1);
        const uint32_t vals[4] = {acc[g].x, acc[g].y, acc[g].z, acc[g].w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int q = 4 * v + e;
            if (q < n) o[q] = (int32_t)vals[e];
            if (q == n) o[q] = (int32_t)(vals[e] + s_in[g * w_in + n_in]);
        }
    }
}

}  // namespace

cudaError_t launch_keyswitch(const DevParams& P, const int32_t* ks, int32_t row_stride,
                             const int32_t* in, int32_t* out, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (P.ks_basebit < 1 || P.ks_basebit > 2 || (row_stride & 3) || row_stride < P.n + 1)
        return cudaErrorInvalidValue;
    const int n_in = P.k * P.N;
    const int nvec = (P.n + 1 + 3) / 4;
    const int threads = ((nvec + 31) / 32) * 32;
    if (threads > 256) return cudaErrorInvalidValue;
    const size_t smem = (size_t)kKsGroup * (n_in + 1) * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(k_keyswitch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = (count + kKsGroup - 1) / kKsGroup;
    k_keyswitch<<<grid, threads, smem, st>>>(ks, row_stride, in, out, count, P.n, n_in, P.ks_t,
                                             P.ks_basebit);
    return cudaGetLastError();
}

}  // namespace tfhe_gb300
