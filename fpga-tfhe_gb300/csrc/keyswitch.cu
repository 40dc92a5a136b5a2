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
// ciphertexts and a span of n_in / split input coefficients; each thread owns
// four output coefficients (one 16-byte column) of all G of them, in
// registers.  The CTA walks its (i, j) pairs once: for two levels j at a
// time it loads the base-1 non-zero rows of each level (independent 16-byte
// loads, coalesced across the warp), then applies them to its G ciphertexts.
// The digits are computed once per CTA in the prologue (8 digits of 2 bits
// packed per coefficient in shared memory), so a digit costs a shift and a
// mask; it is the same for every lane of a warp, so the row choice is a
// warp-uniform branch.  Each table row read from L2 serves G ciphertexts.
// With split > 1 the partial sums of the split CTAs are added into the
// zeroed output with integer atomics (exact mod 2^32 in any order): more
// CTAs in flight for a latency-bound loop, and a small batch spread over
// many SMs instead of one.
#include "engine.h"

namespace tfhe_gb300 {

namespace {

constexpr int kKsGroup = 8;  // ciphertexts per CTA
constexpr int kKsJBlock = 2;  // digit levels loaded together (measured best: 63 registers, 6 CTAs per SM)

__device__ __forceinline__ void sub4(uint4& a, const uint4& r) {
    a.x -= r.x;
    a.y -= r.y;
    a.z -= r.z;
    a.w -= r.w;
}

// basebit = 2 (base 4), t a multiple of kKsJBlock and <= 16; n_in a
// multiple of split.
__global__ void __launch_bounds__(160) k_keyswitch_b4(const int32_t* __restrict__ ks, int row_stride,
                                                      const int32_t* __restrict__ in,
                                                      int32_t* __restrict__ out, int count, int n,
                                                      int n_in, int t, int split) {
    extern __shared__ __align__(16) uint32_t s_dig[];  // kKsGroup x span packed digits
    __shared__ uint32_t s_b[kKsGroup];
    const int grp = blockIdx.x / split, part = blockIdx.x - grp * split;
    const int span = n_in / split, i0 = part * span;
    const int c0 = grp * kKsGroup;
    const int G = min(kKsGroup, count - c0);
    const int w_in = n_in + 1;
    const uint32_t prec_offset = 1u << (32 - (1 + 2 * t));
    for (int idx = threadIdx.x; idx < G * span; idx += blockDim.x) {
        const int g = idx / span, i = idx - g * span;
        const uint32_t aibar = (uint32_t)in[(size_t)(c0 + g) * w_in + i0 + i] + prec_offset;
        // digit j = (aibar >> (32 - 2(j+1))) & 3, packed at bits 2j
        uint32_t packed = 0;
        for (int j = 0; j < t; ++j) packed |= ((aibar >> (30 - 2 * j)) & 3u) << (2 * j);
        s_dig[g * span + i] = packed;
    }
    // the body b is added once, by the first part
    if (threadIdx.x < G) s_b[threadIdx.x] = part == 0 ? (uint32_t)in[(size_t)(c0 + threadIdx.x) * w_in + n_in] : 0u;
    __syncthreads();

    const int nvec = (n + 1 + 3) >> 2;
    const int v = threadIdx.x;
    const bool live = v < nvec;
    const int vv = live ? v : 0;  // idle lanes load a valid column and drop it
    const int rs4 = row_stride >> 2;

    uint4 acc[kKsGroup];
#pragma unroll
    for (int g = 0; g < kKsGroup; ++g) acc[g] = make_uint4(0, 0, 0, 0);

    const int4* base = reinterpret_cast<const int4*>(ks);
#pragma unroll 1
    for (int ii = 0; ii < span; ++ii) {
        const int i = i0 + ii;
        // the coefficient's packed digits of every ciphertext, read once
        // (measured: 2.95 -> 2.89 ms for 4096 against a read per level pair)
        uint32_t dgi[kKsGroup];
#pragma unroll
        for (int g = 0; g < kKsGroup; ++g) dgi[g] = g < G ? s_dig[g * span + ii] : 0u;
#pragma unroll 1
        for (int j0 = 0; j0 < t; j0 += kKsJBlock) {
            uint4 row[kKsJBlock][3];
#pragma unroll
            for (int jj = 0; jj < kKsJBlock; ++jj) {
                const int4* rp = base + ((size_t)(i * t + j0 + jj) * 4) * rs4 + vv;
#pragma unroll
                for (int h = 1; h < 4; ++h) {
                    const int4 r = __ldg(rp + (size_t)h * rs4);
                    row[jj][h - 1] = make_uint4((uint32_t)r.x, (uint32_t)r.y, (uint32_t)r.z,
                                                (uint32_t)r.w);
                }
            }
#pragma unroll
            for (int g = 0; g < kKsGroup; ++g) {
                if (g >= G) break;
                const uint32_t dg = dgi[g] >> (2 * j0);
#pragma unroll
                for (int jj = 0; jj < kKsJBlock; ++jj) {
                    switch ((dg >> (2 * jj)) & 3u) {
                    case 1: sub4(acc[g], row[jj][0]); break;
                    case 2: sub4(acc[g], row[jj][1]); break;
                    case 3: sub4(acc[g], row[jj][2]); break;
                    default: break;
                    }
                }
            }
        }
    }
    if (!live) return;
#pragma unroll
    for (int g = 0; g < kKsGroup; ++g) {
        if (g >= G) break;
        int32_t* o = out + (size_t)(c0 + g) * (n + 1);
        const uint32_t vals[4] = {acc[g].x, acc[g].y, acc[g].z, acc[g].w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int q = 4 * v + e;
            if (q > n) break;
            const uint32_t val = vals[e] + (q == n ? s_b[g] : 0u);
            if (split == 1) o[q] = (int32_t)val;
            else atomicAdd(reinterpret_cast<unsigned*>(o + q), val);
        }
    }
}

}  // namespace

cudaError_t launch_keyswitch(const DevParams& P, const int32_t* ks, int32_t row_stride,
                             const int32_t* in, int32_t* out, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (P.ks_basebit != 2 || P.ks_t % kKsJBlock || P.ks_t > 16 || (row_stride & 3) ||
        row_stride < P.n + 1)
        return cudaErrorInvalidValue;
    const int n_in = P.k * P.N;
    const int nvec = (P.n + 1 + 3) / 4;
    const int threads = ((nvec + 31) / 32) * 32;
    if (threads > 160) return cudaErrorInvalidValue;
    // split the input coefficients over enough CTAs to have about 4096 in
    // flight (27 per SM, 4 resident at a time): 8 for 4096 ciphertexts, 64
    // for a single one
    const int groups = (count + kKsGroup - 1) / kKsGroup;
    int split = 1;
    while (split < 64 && groups * split < 4096 && n_in % (2 * split) == 0) split *= 2;
    const size_t smem = (size_t)kKsGroup * (n_in / split) * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(k_keyswitch_b4,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (split > 1) {
        e = cudaMemsetAsync(out, 0, (size_t)count * (P.n + 1) * sizeof(int32_t), st);
        if (e != cudaSuccess) return e;
    }
    k_keyswitch_b4<<<groups * split, threads, smem, st>>>(ks, row_stride, in, out, count, P.n, n_in,
                                                          P.ks_t, split);
    return cudaGetLastError();
}

}  // namespace tfhe_gb300
