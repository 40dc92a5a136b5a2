// bootstrap.cu -- FFT-domain kernels of the GB300 TFHE engine:
//   * key conversion (TGSW time domain -> engine FFT layout, both forms)
//   * the external product, MuxRotate and the blind-rotation loop, one
//     kernel template (EpMode) built on a fused step:
//       rotate (X^a - 1) -> gadget digits -> twisted FFT-512 -> MAC against
//       the key -> inverse FFT-512 -> Torus32 -> accumulate
//   * bootstrap front end (modulus switch, rotated test vector) and sample
//     extraction, fused into the blind-rotation kernel
//   * small kernels: gate combination, X^a - 1 rotation, extraction
//   * the Lagrange processor (polynomial <-> Lagrange half-complex form in
//     the reference's layout)
//
// Reference call stack restated here (paths inside shreks99/fpga-tfhe):
//   tfhe_blindRotate_FFT         kernel/src/tfhe_blindRotate_FFT/tfhe_blindRotate_FFT.cpp:61-147
//   tfhe_MuxRotate_FFT_FPGA      .../tfhe_MuxRotate_FFT.cpp:56-85
//   tLweMulByXaiMinusOne_FPGA    .../tfhe_MuxRotate_FFT.cpp:5-33
//   tGswFFTExternMulToTLwe_FPGA  .../tGswFFTExternMulToTLwe.cpp:203-247
//   decompose                    .../tGswFFTExternMulToTLwe.cpp:76-95
//   ifft (Int -> Lagrange)       .../tGswFFTExternMulToTLwe.cpp:97-130
//   MAC                          .../tGswFFTExternMulToTLwe.cpp:166-197
//   TorusPolynomial_fft          .../TorusPolynomial_fft.cpp:4-43
//   modulus switch / test vector kernel/src/tfhe_bootstrap_woKS_FFT/tfhe_bootstrap_woKS_FFT.cpp:3-10,57-66
//   X^{2N-b} rotation            kernel/src/tfhe_blindRotateAndExtract/mulByXaiOrCopy.cpp:25-41
#include <cooperative_groups.h>
#include <math.h>

#include "async_copy.cuh"
#include "engine.h"
#include "fft512.cuh"

namespace tfhe_gb300 {

namespace {

constexpr int kN = 1024;
constexpr int kHalf = 512;
// Table layout (complex entries): W^(tq) as [q][t] (512), W^(8jq) as [q][j]
// (64), psi^t W^(tq) as [q][t] (512), then psi^x (512).  The blind-rotation
// and external-product kernels keep only the "hot" part [kTabB, kTabB +
// kHotSize) in shared memory: W^(8jq) at 0, psi^t W^(tq) at 64.
constexpr int kTabA = 0;
constexpr int kTabB = 512;
constexpr int kTabT = 576;
constexpr int kTabPsi = 1088;
constexpr int kTabSize = 1600;
constexpr int kHotSize = 576;

// ----------------------------------------------------------------------
// helpers
// ----------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ const cpx<R>* table_ptr(const Tables& T);
template <>
__device__ __forceinline__ const cpx<float>* table_ptr<float>(const Tables& T) {
    return reinterpret_cast<const cpx<float>*>(T.tw32);
}
template <>
__device__ __forceinline__ const cpx<double>* table_ptr<double>(const Tables& T) {
    return reinterpret_cast<const cpx<double>*>(T.tw64);
}

__device__ __forceinline__ int32_t mod_switch_2n(int32_t phase) {
    // numeric-functions.cpp:59-65 with Msize = 2N = 2048
    const uint64_t interv = ((UINT64_C(1) << 63) / 2048u) * 2;
    const uint64_t half_interval = interv / 2;
    const uint64_t phase64 = ((uint64_t)(int64_t)phase << 32) + half_interval;
    return (int32_t)(phase64 / interv);
}

// (X^a * p)[x] for a in [0, 2N): s = (x - a) mod 2N; +p[s] or -p[s - N].
__device__ __forceinline__ int32_t rot_coef(const int32_t* p, int x, int a) {
    const int s = (x - a) & (2 * kN - 1);
    const int32_t v = p[s & (kN - 1)];
    return s < kN ? v : (int32_t)(0u - (uint32_t)v);
}

// Coefficient i of X^{2N - barb} tv: the rotated test vector the blind
// rotation starts from.  tv = nullptr is the constant mu of the gate
// bootstrap (tfhe_bootstrap_woKS_FFT.cpp:63-66, mulByXaiOrCopy.cpp:25-41),
// else the polynomial of item c (programmable bootstrap).
__device__ __forceinline__ int32_t test_vector_coef(const EpArgs& a, int c, int barb, int i) {
    if (!a.tv) return (((i + barb) & (2 * kN - 1)) < kN) ? a.mu : -a.mu;
    return rot_coef(a.tv + (size_t)c * a.tv_stride, i, (2 * kN - barb) & (2 * kN - 1));
}

// Rounding the inverse transform's FP32 output to Torus32 without a float ->
// int64 conversion (on this part that conversion issues to the narrow FP64
// pipe).  M = 1.5 * 2^23: for |y| < 2^22 the sum y + M rounds y to the
// nearest integer, whose two's complement is then the low bits of the sum's
// encoding.
constexpr float kRoundMagic = 12582912.0f;
constexpr int32_t kRoundMagicBits = 0x4B400000;

// round(v / 512) mod 2^32 for |v / 512| < 2^22 (the high key part's product:
// about 2^18 typical, the exactness limit of FP32 is 2^24): one FMA and one
// integer add; both halves of a packed pair at once.
__device__ __forceinline__ void round_small_pair(cpx<float> z, uint32_t& a0, uint32_t& a1) {
    const float2 r = __ffma2_rn(pk(z), bc(0x1p-9f), bc(kRoundMagic));
    a0 = (uint32_t)(__float_as_int(r.x) - kRoundMagicBits);
    a1 = (uint32_t)(__float_as_int(r.y) - kRoundMagicBits);
}

// round(v / 512) mod 2^32 for any |v / 512| < 2^53 (the low key part's
// product, up to about 2^36): the multiple of 2^32 is removed exactly in
// FP32 (q = rint(v / 2^41), a = v - q 2^41 exact, |a| <= 2^40), and the
// remainder (|a / 512| <= 2^31) goes through a float -> int32 conversion,
// which does not use the FP64 pipe.  (A remainder of exactly +2^31
// saturates one unit short: an error of one unit in the low part.)
__device__ __forceinline__ void round_wrap_pair(cpx<float> z, uint32_t& a0, uint32_t& a1) {
    const float2 q = __fadd2_rn(__ffma2_rn(pk(z), bc(0x1p-41f), bc(kRoundMagic)), bc(-kRoundMagic));
    const float2 a = __ffma2_rn(make_float2(-q.x, -q.y), bc(0x1p41f), pk(z));
    const float2 sc = __fmul2_rn(a, bc(0x1p-9f));
    a0 = (uint32_t)__float2int_rn(sc.x);
    a1 = (uint32_t)__float2int_rn(sc.y);
}

// Gadget digit of u at `decal` as a transform input: ((u >> decal) & mask) -
// halfBg.  FP32: the masked digit m < 2^22 ORed into the encoding of the
// magic constant is the float M + m, and one subtraction of M + halfBg
// gives m - halfBg exactly.
template <typename R>
__device__ __forceinline__ R digit_value(uint32_t u, int decal, uint32_t mask, int halfBg) {
    if constexpr (sizeof(R) == 4) {
        return __int_as_float((int32_t)(((u >> decal) & mask) | (uint32_t)kRoundMagicBits)) -
               (kRoundMagic + (float)halfBg);
    } else {
        return (R)((int)((u >> decal) & mask) - halfBg);
    }
}

// Both digits of a folded point (coefficients x and x + 512) as one
// complex transform input; FP32: one packed subtraction.
template <typename R>
__device__ __forceinline__ cpx<R> digit_pair(uint32_t u0, uint32_t u1, int decal, uint32_t mask, int halfBg) {
    if constexpr (sizeof(R) == 4) {
        const float f0 = __int_as_float((int32_t)(((u0 >> decal) & mask) | (uint32_t)kRoundMagicBits));
        const float f1 = __int_as_float((int32_t)(((u1 >> decal) & mask) | (uint32_t)kRoundMagicBits));
        return unpk(__fadd2_rn(make_float2(f0, f1), bc(-(kRoundMagic + (float)halfBg))));
    } else {
        return {digit_value<R>(u0, decal, mask, halfBg), digit_value<R>(u1, decal, mask, halfBg)};
    }
}

template <typename R>
__device__ __forceinline__ int64_t to_int(R v);
template <>
__device__ __forceinline__ int64_t to_int<double>(double v) {
    // reference semantics: int64_t(double) truncates (TorusPolynomial_fft.cpp:40)
    return __double2ll_rz(v);
}

// ----------------------------------------------------------------------
// shared-memory plan of the FFT kernels
//   [tables: kTabSize cpx<R>] then per 64-thread group:
//   [acc: 2 x 1024 int32][NB x 2 exchange buffers of 576 cpx<R>]
// NB = number of transforms run together (max of L and the parts).
// ----------------------------------------------------------------------
template <typename R, int NB>
struct SmemPlan {
    static constexpr size_t tables = kHotSize * sizeof(cpx<R>);
    static constexpr size_t acc = 2 * kN * sizeof(int32_t);
    static constexpr size_t scratch = NB * 2 * kScratchStride * sizeof(cpx<R>);
    static constexpr size_t group = acc + scratch;
    static size_t total(int groups) { return tables + groups * group; }
};

template <typename R>
__device__ __forceinline__ FftScratch<R> scratch_at(char* base) {
    cpx<R>* s = reinterpret_cast<cpx<R>*>(base);
    return {s, s + kScratchStride};
}

template <typename R>
__device__ __forceinline__ void load_tables(cpx<R>* dst, const Tables& T) {
    const cpx<R>* src = table_ptr<R>(T);
    for (int i = threadIdx.x; i < kTabSize; i += blockDim.x) dst[i] = src[i];
}

template <typename R>
__device__ __forceinline__ FftTwiddles<R> twiddles_at(const cpx<R>* tables) {
    return {tables + kTabA, tables + kTabB};
}

// the hot tables (twist-folded pass-A twiddles, pass-B twiddles)
template <typename R>
__device__ __forceinline__ void load_hot_tables(cpx<R>* dst, const Tables& T) {
    const cpx<R>* src = table_ptr<R>(T) + kTabB;
    for (int i = threadIdx.x; i < kHotSize; i += blockDim.x) dst[i] = src[i];
}

template <typename R>
__device__ __forceinline__ FftTwiddles<R> hot_twiddles(const cpx<R>* hot) {
    return {hot + (kTabT - kTabB), hot};
}

// ----------------------------------------------------------------------
// the fused step: out = EP(ROT ? (X^a - 1) acc : acc);
//                 acc = (ROT ? acc : 0) + out
// A key row p of a TGSW in engine layout is [2 outputs][PARTS][512
// key_index order] complex values; `Keys` says where rows come from:
//   GlobalKeys -- straight from global memory (L2), 16-byte loads, with an
//                 L1 prefetch of the rows ahead of the transform;
//   RingKeys   -- from a shared-memory ring filled by a producer warp with
//                 bulk copies (see k_blind_rotate_ring).
// FB digit polynomials are transformed together (fft512_forward_tw_multi), and
// IB parts of an output polynomial are transformed back together.  IP: the
// in-place transforms (fft512_forward_ip / fft512_inverse_ip: one group
// barrier per transform instead of two), alternating the two exchange
// buffers of each stream from one transform to the next.  EARLY: a block's
// key rows are tested for arrival before its forward transforms and waited
// for after them.
// ----------------------------------------------------------------------
template <typename R, int PARTS, int NB>
struct StepCtx {
    FftTwiddles<R> tw;  // smem twiddles: a = psi^t W^(tq) (twist folded), b = W^(8jq)
    FftIdx ix;          // this thread's exchange slots
    FftScratch<R> s[NB];
    int32_t* acc;       // smem 2 x N
    int t, bar_id;
    int Bgbit, split;
    uint32_t offset;
};

template <typename R, int PARTS>
struct GlobalKeys {
    static constexpr size_t kRow = (size_t)2 * PARTS * kHalf;
    const cpx<R>* gsw;
    __device__ __forceinline__ void prefetch(int p0, int np, int t) const {
        const int lines = (int)(np * kRow * sizeof(cpx<R>) / 128);
        const char* gb = reinterpret_cast<const char*>(gsw + (size_t)p0 * kRow);
        for (int ln = t; ln < lines; ln += 64)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(gb + (size_t)ln * 128));
    }
    __device__ __forceinline__ const cpx<R>* acquire(int p) const { return gsw + (size_t)p * kRow; }
    __device__ __forceinline__ bool poll(int) const { return true; }
    __device__ __forceinline__ const cpx<R>* acquire_polled(int p, bool) const { return acquire(p); }
    __device__ __forceinline__ void release(int) const {}
    static constexpr bool kShared = false;
};

template <bool SHARED>
__device__ __forceinline__ float4 key_load4(const float4* p) {
    if constexpr (SHARED) return *p;
    else return __ldg(p);
}

template <typename R, int PARTS, bool SHARED>
__device__ __forceinline__ void mac_row(cpx<R> (&out)[2][PARTS][8], const cpx<R> (&v)[8],
                                        const cpx<R>* __restrict__ g, int t) {
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int pt = 0; pt < PARTS; ++pt) {
            const cpx<R>* gk = g + (j * PARTS + pt) * kHalf;
            if constexpr (sizeof(R) == 4) {
                const float4* g4 = reinterpret_cast<const float4*>(gk);
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const float4 w = key_load4<SHARED>(g4 + qq * 64 + t);
                    const cpx<R> k0 = {(R)w.x, (R)w.y}, k1 = {(R)w.z, (R)w.w};
                    out[j][pt][2 * qq] = cmac(out[j][pt][2 * qq], v[2 * qq], k0);
                    out[j][pt][2 * qq + 1] = cmac(out[j][pt][2 * qq + 1], v[2 * qq + 1], k1);
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const cpx<R> k0 = gk[key_index<R>(t, q)];
                    out[j][pt][q] = cmac(out[j][pt][q], v[q], k0);
                }
            }
        }
}

// Levels lev0 .. lev0 + NBK - 1 of input polynomial jp: digits, NBK forward
// transforms run together, and their key rows multiply-accumulated.
template <int NBK, bool IP, bool EARLY, typename R, int PARTS, int NB, typename Keys>
__device__ __forceinline__ void forward_levels(const StepCtx<R, PARTS, NB>& S, Keys& keys,
                                               cpx<R> (&out)[2][PARTS][8], const uint32_t (&r0)[8],
                                               const uint32_t (&r1)[8], int p0, int lev0, uint32_t mask,
                                               int halfBg, int which) {
    const int t = S.t;
    bool landed[NBK];
#pragma unroll
    for (int b = 0; b < NBK; ++b) landed[b] = EARLY ? keys.poll(p0 + lev0 + b) : false;
    cpx<R> v[NBK][8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
#pragma unroll
        for (int b = 0; b < NBK; ++b) {
            const int decal = 32 - (lev0 + b + 1) * S.Bgbit;
            v[b][r] = digit_pair<R>(r0[r], r1[r], decal, mask, halfBg);
        }
    }
    if constexpr (IP) {
        cpx<R>* x[NBK];
#pragma unroll
        for (int b = 0; b < NBK; ++b) x[b] = which ? S.s[b].b1 : S.s[b].b0;
        fft512_forward_ip<NBK>(v, x, S.tw, S.ix, t, S.bar_id);
    } else {
        fft512_forward_tw_multi<NBK>(v, *reinterpret_cast<const FftScratch<R>(*)[NBK]>(S.s), S.tw, S.ix, t,
                                     S.bar_id);
    }
#pragma unroll
    for (int b = 0; b < NBK; ++b) {
        const int p = p0 + lev0 + b;
        mac_row<R, PARTS, Keys::kShared>(out, v[b], EARLY ? keys.acquire_polled(p, landed[b]) : keys.acquire(p),
                                         t);
        keys.release(p);
    }
}

template <typename R, int PARTS, bool ROT, int L, int FB, int IB, int NB, bool IP = false, bool EARLY = false,
          typename Keys>
__device__ __forceinline__ void ep_step(const StepCtx<R, PARTS, NB>& S, Keys& keys, int a) {
    static_assert(PARTS % IB == 0 && FB <= NB && IB <= NB, "batch sizes");
    const int t = S.t;
    const int halfBg = 1 << (S.Bgbit - 1);
    const uint32_t mask = (1u << S.Bgbit) - 1;

    cpx<R> out[2][PARTS][8];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int pt = 0; pt < PARTS; ++pt)
#pragma unroll
            for (int q = 0; q < 8; ++q) out[j][pt][q] = {(R)0, (R)0};
    int which = 0;  // IP: the exchange buffer of the next transform

#pragma unroll 1
    for (int jp = 0; jp < 2; ++jp) {
        keys.prefetch(jp * L, L, t);
        const int32_t* src = S.acc + jp * kN;
        uint32_t r0[8], r1[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int x0 = t + 64 * r;
            if (ROT) {
                r0[r] = (uint32_t)rot_coef(src, x0, a) - (uint32_t)src[x0];
                r1[r] = (uint32_t)rot_coef(src, x0 + kHalf, a) - (uint32_t)src[x0 + kHalf];
            } else {
                r0[r] = (uint32_t)src[x0];
                r1[r] = (uint32_t)src[x0 + kHalf];
            }
            r0[r] += S.offset;
            r1[r] += S.offset;
        }
        // blocks of FB levels, then the remaining L % FB together
#pragma unroll
        for (int lev0 = 0; lev0 + FB <= L; lev0 += FB) {
            forward_levels<FB, IP, EARLY>(S, keys, out, r0, r1, jp * L, lev0, mask, halfBg, which);
            which ^= 1;
        }
        if constexpr (L % FB != 0) {
            forward_levels<L % FB, IP, EARLY>(S, keys, out, r0, r1, jp * L, L - L % FB, mask, halfBg, which);
            which ^= 1;
        }
    }

    // back to the coefficient domain (j unrolled: out[j] must stay in registers)
    const R inv = (R)(1.0 / 512.0);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        uint32_t c0[8], c1[8];
#pragma unroll
        for (int pt0 = 0; pt0 < PARTS; pt0 += IB) {
            cpx<R> v[IB][8];
#pragma unroll
            for (int b = 0; b < IB; ++b)
#pragma unroll
                for (int q = 0; q < 8; ++q) v[b][q] = out[j][pt0 + b][q];
            if constexpr (IP) {
                cpx<R>* x[IB];
#pragma unroll
                for (int b = 0; b < IB; ++b) x[b] = which ? S.s[b].b1 : S.s[b].b0;
                fft512_inverse_ip<IB>(v, x, S.tw, S.ix, t, S.bar_id);
            } else {
                fft512_inverse_tw_multi<IB>(v, *reinterpret_cast<const FftScratch<R>(*)[IB]>(S.s), S.tw, S.ix,
                                            t, S.bar_id);
            }
            which ^= 1;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
#pragma unroll
                for (int b = 0; b < IB; ++b) {
                    const int pt = pt0 + b;
                    const cpx<R> z = v[b][q];
                    uint32_t a0, a1;
                    if constexpr (sizeof(R) == 4) {
                        if (PARTS == 2 && pt == 0) round_small_pair(z, a0, a1);
                        else round_wrap_pair(z, a0, a1);
                    } else {
                        a0 = (uint32_t)(uint64_t)to_int<R>(z.x * inv);
                        a1 = (uint32_t)(uint64_t)to_int<R>(z.y * inv);
                    }
                    if (PARTS == 1) {
                        c0[q] = a0;
                        c1[q] = a1;
                    } else if (pt == 0) {  // high part, scaled by 2^split
                        c0[q] = a0 << S.split;
                        c1[q] = a1 << S.split;
                    } else {
                        c0[q] += a0;
                        c1[q] += a1;
                    }
                }
            }
        }
        int32_t* dst = S.acc + j * kN;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int x0 = t + 64 * q;
            if (ROT) {
                dst[x0] = (int32_t)((uint32_t)dst[x0] + c0[q]);
                dst[x0 + kHalf] = (int32_t)((uint32_t)dst[x0 + kHalf] + c1[q]);
            } else {
                dst[x0] = (int32_t)c0[q];
                dst[x0 + kHalf] = (int32_t)c1[q];
            }
        }
    }
    group_sync(S.bar_id);
}

// Rounding of one transformed-back polynomial part into c0/c1 (the 16
// coefficients x0 = t + 64q and x0 + 512 of this thread): FP32 parts --
// the high part (pt = 0) rounded and shifted by the split, the low part
// (pt = 1) added; FP64 -- the reference's truncating conversion.
template <typename R, int PARTS>
__device__ __forceinline__ void round_part(const cpx<R> (&v)[8], int pt, int split, uint32_t (&c0)[8],
                                           uint32_t (&c1)[8]) {
    if constexpr (sizeof(R) == 4) {
        if (PARTS == 2 && pt == 0) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t a0, a1;
                round_small_pair(v[q], a0, a1);
                c0[q] = a0 << split;
                c1[q] = a1 << split;
            }
        } else if (PARTS == 2) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t a0, a1;
                round_wrap_pair(v[q], a0, a1);
                c0[q] += a0;
                c1[q] += a1;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) round_wrap_pair(v[q], c0[q], c1[q]);
        }
    } else {
        const R inv = (R)(1.0 / 512.0);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            c0[q] = (uint32_t)(uint64_t)to_int<R>(v[q].x * inv);
            c1[q] = (uint32_t)(uint64_t)to_int<R>(v[q].y * inv);
        }
    }
}

// out[j][pt] into v, (j, pt) uniform at run time, indices compile-time so
// that out stays in registers.
template <typename R, int PARTS>
__device__ __forceinline__ void pick_part(cpx<R> (&v)[8], const cpx<R> (&out)[2][PARTS][8], int j, int pt) {
#pragma unroll
    for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int pp = 0; pp < PARTS; ++pp)
            if (jj == j && pp == pt) {
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = out[jj][pp][q];
            }
}

// out[j][pt] += w, (j, pt) uniform at run time.
template <typename R, int PARTS>
__device__ __forceinline__ void add_part(cpx<R> (&out)[2][PARTS][8], const cpx<R> (&w)[8], int j, int pt) {
#pragma unroll
    for (int jj = 0; jj < 2; ++jj)
#pragma unroll
        for (int pp = 0; pp < PARTS; ++pp)
            if (jj == j && pp == pt) {
#pragma unroll
                for (int q = 0; q < 8; ++q) out[jj][pp][q] = cadd(out[jj][pp][q], w[q]);
            }
}

// The fused step of the shared-ring kernel, with one copy of each transform
// in the code: the levels and the (output, part) pairs are run-time loops
// (a fully unrolled step overflows the instruction cache).  In-place
// transforms, alternating the two exchange buffers.
template <typename R, int PARTS, int L, typename Keys>
__device__ __forceinline__ void ep_step_lean(const StepCtx<R, PARTS, 1>& S, Keys& keys, int a) {
    const int t = S.t;
    const int halfBg = 1 << (S.Bgbit - 1);
    const uint32_t mask = (1u << S.Bgbit) - 1;
    int which = 0;  // the exchange buffer of the next transform

    cpx<R> out[2][PARTS][8];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int pt = 0; pt < PARTS; ++pt)
#pragma unroll
            for (int q = 0; q < 8; ++q) out[j][pt][q] = {(R)0, (R)0};

#pragma unroll 1
    for (int jp = 0; jp < 2; ++jp) {
        const int32_t* src = S.acc + jp * kN;
        uint32_t r0[8], r1[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int x0 = t + 64 * r;
            r0[r] = (uint32_t)rot_coef(src, x0, a) - (uint32_t)src[x0] + S.offset;
            r1[r] = (uint32_t)rot_coef(src, x0 + kHalf, a) - (uint32_t)src[x0 + kHalf] + S.offset;
        }
#pragma unroll 1
        for (int lev = 0; lev < L; ++lev) {
            const int decal = 32 - (lev + 1) * S.Bgbit;
            cpx<R> v[8];
#pragma unroll
            for (int r = 0; r < 8; ++r)
                v[r] = digit_pair<R>(r0[r], r1[r], decal, mask, halfBg);
            fft512_forward_ip1(v, which ? S.s[0].b1 : S.s[0].b0, S.tw, S.ix, t, S.bar_id);
            which ^= 1;
            const int p = jp * L + lev;
            mac_row<R, PARTS, Keys::kShared>(out, v, keys.acquire(p), t);
            keys.release(p);
        }
    }

    uint32_t c0[8], c1[8];
#pragma unroll 1
    for (int u = 0; u < 2 * PARTS; ++u) {
        const int j = u / PARTS, pt = u % PARTS;
        cpx<R> v[8];
        pick_part<R, PARTS>(v, out, j, pt);
        fft512_inverse_ip1(v, which ? S.s[0].b1 : S.s[0].b0, S.tw, S.ix, t, S.bar_id);
        which ^= 1;
        round_part<R, PARTS>(v, pt, S.split, c0, c1);
        if (pt == PARTS - 1) {
            int32_t* dst = S.acc + j * kN;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int x0 = t + 64 * q;
                dst[x0] = (int32_t)((uint32_t)dst[x0] + c0[q]);
                dst[x0 + kHalf] = (int32_t)((uint32_t)dst[x0 + kHalf] + c1[q]);
            }
        }
    }
    group_sync(S.bar_id);
}

struct KParams {
    int n, Bgbit, split;
    uint32_t offset;
};

template <typename R, int PARTS, int MODE, int GROUPS, int L>
__global__ void __launch_bounds__(64 * GROUPS, 1) k_external_product(KParams kp, Tables T, EpArgs a) {
    constexpr int NB = L > PARTS ? L : PARTS;
    using Ctx = StepCtx<R, PARTS, NB>;
    using Plan = SmemPlan<R, NB>;
    extern __shared__ __align__(128) char smem[];
    cpx<R>* tables = reinterpret_cast<cpx<R>*>(smem);
    load_hot_tables<R>(tables, T);
    __syncthreads();

    const int g = threadIdx.x >> 6;
    const int t = threadIdx.x & 63;
    const int c = blockIdx.x * GROUPS + g;
    if (c >= a.count) return;

    char* gbase = smem + Plan::tables + (size_t)g * Plan::group;
    Ctx S;
    S.tw = hot_twiddles<R>(tables);
    S.ix = make_fft_idx(t);
    S.acc = reinterpret_cast<int32_t*>(gbase);
#pragma unroll
    for (int b = 0; b < NB; ++b)
        S.s[b] = scratch_at<R>(gbase + Plan::acc + (size_t)b * 2 * kScratchStride * sizeof(cpx<R>));
    S.t = t;
    S.bar_id = 1 + g;
    S.Bgbit = kp.Bgbit;
    S.split = kp.split;
    S.offset = kp.offset;

    const size_t gsw_elems = (size_t)2 * L * 2 * PARTS * kHalf;
    const cpx<R>* gsw_base = reinterpret_cast<const cpx<R>*>(a.gsw);

    if (MODE == kEpBlindRotate) {
        const int n = kp.n;
        if (a.acc_in) {
            const int32_t* src = a.acc_in + (size_t)c * 2 * kN;
            for (int i = t; i < 2 * kN; i += 64) S.acc[i] = src[i];
        } else {
            // test vector mu * sum X^j rotated by X^{2N - barb}: the sign of
            // coefficient x is + when (x + barb) mod 2N < N
            const int32_t* xs = a.x + (size_t)c * (n + 1);
            const int barb = mod_switch_2n(xs[n]);
            for (int i = t; i < kN; i += 64) {
                S.acc[i] = 0;
                S.acc[kN + i] = test_vector_coef(a, c, barb, i);
            }
        }
        group_sync(S.bar_id);
        const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
        const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
        // the rotation amount of step i + 1 is loaded during step i
        int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
#pragma unroll 1
        for (int i = 0; i < n; ++i) {
            const int ai = a_next;
            if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
            if (ai == 0) continue;  // tfhe_blindRotate_FFT.cpp:114
            GlobalKeys<R, PARTS> keys{gsw_base + (size_t)i * gsw_elems};
            ep_step<R, PARTS, true, L, L, PARTS, NB>(S, keys, ai);
        }
        if (a.acc_out) {
            int32_t* dst = a.acc_out + (size_t)c * 2 * kN;
            for (int i = t; i < 2 * kN; i += 64) dst[i] = S.acc[i];
        }
        if (a.lwe_out) {
            // tLweExtractLweSample: a'_0 = a_0, a'_j = -a_{N-j}, b' = b_0
            int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
            for (int i = t; i < kN; i += 64)
                dst[i] = i == 0 ? S.acc[0] : (int32_t)(0u - (uint32_t)S.acc[kN - i]);
            if (t == 0) dst[kN] = S.acc[kN];
        }
    } else {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN;
        for (int i = t; i < 2 * kN; i += 64) S.acc[i] = src[i];
        group_sync(S.bar_id);
        const cpx<R>* gsw = reinterpret_cast<const cpx<R>*>(
            reinterpret_cast<const char*>(a.gsw) + a.gsw_stride * (size_t)c);
        GlobalKeys<R, PARTS> keys{gsw};
        if (MODE == kEpPlain) {
            ep_step<R, PARTS, false, L, L, PARTS, NB>(S, keys, 0);
        } else {
            const int ai = a.bara[c];
            if (ai != 0) ep_step<R, PARTS, true, L, L, PARTS, NB>(S, keys, ai);
        }
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN;
        for (int i = t; i < 2 * kN; i += 64) dst[i] = S.acc[i];
    }
}

// ----------------------------------------------------------------------
// Blind rotation with the bootstrapping key streamed through shared memory.
//
// A CTA runs GROUPS ciphertexts (64 threads each) plus one producer warp.
// Every ciphertext of the CTA walks the same key rows in the same order
// (row r = step i * 2l + p), so the producer streams each 16 KB row once per
// CTA with a bulk copy into a ring of S slots, and all groups read it from
// shared memory: one key read per CTA instead of one per ciphertext, and no
// L2 latency on the multiply-accumulate.  Slot hand-off uses two mbarriers
// per slot: full (the copy's byte count landed) and empty (every consumer
// thread has read the row).  A group that skips a step (a_i = 0) still waits
// and releases its rows, so the ring stays in step.  Every wait is bounded;
// a timeout sets *err (TFHE_GPU_TIMEOUT for the host) and the kernel runs to
// its end without further waiting on the ring.
// ----------------------------------------------------------------------
template <typename R, int PARTS, int S>
struct RingKeys {
    static constexpr size_t kRow = (size_t)2 * PARTS * kHalf;
    static constexpr size_t kRowBytes = kRow * sizeof(cpx<R>);
    static constexpr bool kShared = true;
    cpx<R>* ring;
    uint64_t* full;
    uint64_t* empty;
    uint32_t row0;
    int32_t* err;
    volatile int* abort;   // CTA-wide: set by the first wait that gives up
    // In-line producer (one thread of the CTA when there is no producer
    // warp): before taking row r it issues rows up to r + S - 1, waiting only
    // for rows it needs itself (<= r) and skipping ahead rows whose slot is
    // still held.
    bool producer;
    const char* src;       // key rows in global memory
    uint32_t total;        // rows to stream
    uint32_t next_issue;   // first row not issued yet

    __device__ __forceinline__ void give_up() {
        *abort = 1;
        atomicExch(err, 3);
    }
    __device__ __forceinline__ void issue_one() {
        const uint32_t slot = next_issue % S;
        mbar_arrive_expect_tx(&full[slot], (uint32_t)kRowBytes);
        bulk_copy_g2s(reinterpret_cast<char*>(ring) + slot * kRowBytes,
                      src + (size_t)next_issue * kRowBytes, (uint32_t)kRowBytes, &full[slot]);
        ++next_issue;
    }
    __device__ __forceinline__ void issue_upto(uint32_t r) {
        while (next_issue < total && next_issue < r + S) {
            const uint32_t slot = next_issue % S;
            if (next_issue >= S) {
                const uint32_t parity = ((next_issue / S) - 1) & 1;
                if (next_issue <= r) {
                    if (!mbar_wait_bounded(&empty[slot], parity, abort)) {
                        give_up();
                        next_issue = total;  // stop streaming; consumers give up and finish
                        return;
                    }
                } else if (!mbar_try_wait(&empty[slot], parity)) {
                    return;
                }
            }
            issue_one();
        }
    }
    // Issue every row up to `last` (inclusive), waiting for their slots: used
    // before the producer blocks on another group, for rows that group needs.
    // Deadlock-free as long as the rows whose slots are reused (<= last - S)
    // are released by consumers that need only rows already issued.
    __device__ __forceinline__ void issue_through(uint32_t last) {
        while (next_issue < total && next_issue <= last) {
            if (next_issue >= S &&
                !mbar_wait_bounded(&empty[next_issue % S], ((next_issue / S) - 1) & 1, abort)) {
                give_up();
                next_issue = total;
                return;
            }
            issue_one();
        }
    }
    // wait until every issued copy has landed (end of kernel)
    __device__ __forceinline__ void drain() {
        for (uint32_t r = next_issue > S ? next_issue - S : 0; r < next_issue; ++r)
            if (!mbar_wait_bounded(&full[r % S], (r / S) & 1)) atomicExch(err, 3);
    }
    __device__ __forceinline__ void prefetch(int, int, int) const {}
    __device__ __forceinline__ const cpx<R>* acquire(int p) {
        const uint32_t r = row0 + (uint32_t)p;
        if (producer) issue_upto(r);
        const uint32_t slot = r % S;
        if (!mbar_wait_bounded(&full[slot], (r / S) & 1, abort)) give_up();
        return ring + slot * kRow;
    }
    // acquire() in two parts, so that the arrival test's round trip overlaps
    // other work: poll() issues rows (producer) and tests once whether row p
    // has landed; acquire_polled() waits (bounded) only if it had not.
    __device__ __forceinline__ bool poll(int p) {
        const uint32_t r = row0 + (uint32_t)p;
        if (producer) issue_upto(r);
        return mbar_try_wait(&full[r % S], (r / S) & 1);
    }
    __device__ __forceinline__ const cpx<R>* acquire_polled(int p, bool landed) {
        const uint32_t r = row0 + (uint32_t)p;
        const uint32_t slot = r % S;
        if (!landed && !mbar_wait_bounded(&full[slot], (r / S) & 1, abort)) give_up();
        return ring + slot * kRow;
    }
    // per_warp: one lane arrives for its whole warp once the warp has read
    // the row (the slot's count is then the number of consumer warps); else
    // every consumer thread arrives
    bool per_warp;
    __device__ __forceinline__ void release(int p) const {
        if (per_warp) {
            __syncwarp();
            if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[(row0 + (uint32_t)p) % S]);
        } else {
            mbar_arrive(&empty[(row0 + (uint32_t)p) % S]);
        }
    }
};

template <typename R, int PARTS, int GROUPS, int L, int S, int NB = 1>
struct RingPlan {
    static constexpr size_t kRowBytes = (size_t)2 * PARTS * kHalf * sizeof(cpx<R>);
    static constexpr size_t tables = kHotSize * sizeof(cpx<R>);
    static constexpr size_t ring_off = (tables + 127) & ~(size_t)127;
    static constexpr size_t bar_off = ring_off + S * kRowBytes;
    static constexpr size_t flag_off = bar_off + 2 * S * sizeof(uint64_t);
    static constexpr size_t group_off = (flag_off + sizeof(int) + 127) & ~(size_t)127;
    static constexpr size_t acc = 2 * kN * sizeof(int32_t);
    static constexpr size_t group = acc + NB * 2 * kScratchStride * sizeof(cpx<R>);
    static constexpr size_t total = group_off + GROUPS * group;
};

// NB = 1: one transform at a time (ep_step_lean).  NB > 1: the l forward
// and the PARTS inverse transforms of a step run together (ep_step), which
// needs NB exchange buffer pairs per group and about 250 registers, so at
// most four groups per CTA.  NB <= 2 uses the in-place transforms (one group
// barrier per transform; measured faster), NB = 3 the two-barrier form (the
// in-place form took its 608-gate wave from 4.57 to 4.90 ms).
template <typename R, int PARTS, int GROUPS, int L, int S, bool INLINE, int NB = 1>
__global__ void __launch_bounds__(64 * GROUPS + (INLINE ? 0 : 32), 1)
    k_blind_rotate_ring(KParams kp, Tables T, EpArgs a) {
    using Plan = RingPlan<R, PARTS, GROUPS, L, S, NB>;
    constexpr int kpl = 2 * L;
    // measured on the two-at-a-time form (NB = 2), not faster for the others:
    // one slot release per consumer warp (6.48 -> 6.45 ms per 912-gate wave)
    // and the rows' arrival tested before the transforms (6.45 -> 6.41 ms;
    // the 4-per-SM form went from 4.58 to 4.98 ms with it)
    constexpr bool kPerWarp = NB == 2;
    extern __shared__ __align__(128) char smem[];
    cpx<R>* tables = reinterpret_cast<cpx<R>*>(smem);
    cpx<R>* ring = reinterpret_cast<cpx<R>*>(smem + Plan::ring_off);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + Plan::bar_off);
    uint64_t* empty = full + S;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + Plan::flag_off);
    const int active = min(GROUPS, a.count - (int)blockIdx.x * GROUPS);
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], (kPerWarp ? 2 : 64) * active);
        }
        *abort = 0;
        fence_mbar_init();
    }
    load_hot_tables<R>(tables, T);
    __syncthreads();

    const int warp = threadIdx.x >> 5;
    const int n = kp.n;
    const uint32_t total_rows = (uint32_t)n * kpl;
    RingKeys<R, PARTS, S> keys{ring, full, empty, 0, a.err, abort, false,
                               reinterpret_cast<const char*>(a.gsw), total_rows, 0, kPerWarp};
    if (!INLINE && warp == 2 * GROUPS) {
        // producer warp: one lane streams all n * 2l key rows in order
        if ((threadIdx.x & 31) == 0 && !a.stall_keys) {
            for (uint32_t r = 0; r < total_rows; ++r) {
                keys.issue_upto(r);  // blocks on row r's slot, issues up to r + S - 1
                if (keys.next_issue <= r) break;  // timed out
            }
            keys.drain();
        }
        return;
    }

    const int g = threadIdx.x >> 6;
    const int t = threadIdx.x & 63;
    const int c = blockIdx.x * GROUPS + g;
    if (g >= active) return;
    keys.producer = INLINE && threadIdx.x == 0 && !a.stall_keys;

    char* gbase = smem + Plan::group_off + (size_t)g * Plan::group;
    StepCtx<R, PARTS, NB> St;
    St.tw = hot_twiddles<R>(tables);
    St.ix = make_fft_idx(t);
    St.acc = reinterpret_cast<int32_t*>(gbase);
#pragma unroll
    for (int b = 0; b < NB; ++b)
        St.s[b] = scratch_at<R>(gbase + Plan::acc + (size_t)b * 2 * kScratchStride * sizeof(cpx<R>));
    St.t = t;
    St.bar_id = 1 + g;
    St.Bgbit = kp.Bgbit;
    St.split = kp.split;
    St.offset = kp.offset;

    if (a.acc_in) {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN;
        for (int i = t; i < 2 * kN; i += 64) St.acc[i] = src[i];
    } else {
        const int32_t* xs = a.x + (size_t)c * (n + 1);
        const int barb = mod_switch_2n(xs[n]);
        for (int i = t; i < kN; i += 64) {
            St.acc[i] = 0;
            St.acc[kN + i] = test_vector_coef(a, c, barb, i);
        }
    }
    group_sync(St.bar_id);
    const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
    const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
    int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const int ai = a_next;
        if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
        keys.row0 = (uint32_t)i * kpl;
        if (ai == 0) {  // tfhe_blindRotate_FFT.cpp:114 -- rows still pass through
            for (int p = 0; p < kpl; ++p) {
                keys.acquire(p);
                keys.release(p);
            }
            continue;
        }
        if constexpr (NB == 1) ep_step_lean<R, PARTS, L>(St, keys, ai);
        else ep_step<R, PARTS, true, L, (NB < L ? NB : L), PARTS, NB, (NB <= 2), kPerWarp>(St, keys, ai);
    }
    if (keys.producer) keys.drain();
    if (a.acc_out) {
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN;
        for (int i = t; i < 2 * kN; i += 64) dst[i] = St.acc[i];
    }
    if (a.lwe_out) {
        int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
        for (int i = t; i < kN; i += 64)
            dst[i] = i == 0 ? St.acc[0] : (int32_t)(0u - (uint32_t)St.acc[kN - i]);
        if (t == 0) dst[kN] = St.acc[kN];
    }
}

// ----------------------------------------------------------------------
// Blind rotation with one ciphertext over 2l groups (lowest latency).
//
// Group g = (jp, lev) = (g / l, g % l) decomposes input polynomial jp at
// level lev, runs that one forward transform and writes the transformed
// digits D_g to shared memory.  After a CTA barrier, owner group (j, pt) =
// (g / 2, g % 2) for g < 4 multiplies all 2l of them with part (j, pt) of
// each key row, transforms back, rounds, and adds its part into the
// accumulator with integer shared-memory atomics (exact mod 2^32 in any
// order, so the result does not depend on timing).  The owners issue their
// key loads (4 float4 per row, from L2) before the barrier, so the latency
// overlaps the other groups' transforms; the next step's rows are
// prefetched into L2.  A step's critical path is one forward transform, 2l
// rows of products and one inverse transform, against the pair kernel's l
// forward and PARTS inverse transforms.  Split-FP32 only.
// ----------------------------------------------------------------------
template <int L>
struct SpreadPlan {
    static constexpr int kGroups = 2 * L;
    static constexpr size_t tables = kHotSize * sizeof(cpx<float>);
    static constexpr size_t acc_off = tables;
    static constexpr size_t d_off = acc_off + 2 * kN * sizeof(int32_t);
    static constexpr size_t scratch_off = d_off + kGroups * kHalf * sizeof(cpx<float>);
    static constexpr size_t scratch = 2 * kScratchStride * sizeof(cpx<float>);
    static constexpr size_t total = scratch_off + kGroups * scratch;
};

template <int L>
__global__ void __launch_bounds__(128 * L, 1) k_blind_rotate_spread(KParams kp, Tables T, EpArgs a) {
    using Plan = SpreadPlan<L>;
    constexpr int kRows = 2 * L;
    constexpr int kRowElems = 2 * 2 * kHalf;  // complex values per key row
    extern __shared__ __align__(128) char smem[];
    cpx<float>* tables = reinterpret_cast<cpx<float>*>(smem);
    int32_t* acc = reinterpret_cast<int32_t*>(smem + Plan::acc_off);
    cpx<float>* dsh = reinterpret_cast<cpx<float>*>(smem + Plan::d_off);  // [g][q][t]
    const int c = blockIdx.x;
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int jp = g / L, lev = g - jp * L;
    const bool owner = g < 4;
    const int oj = g >> 1, opt = g & 1;
    const int n = kp.n;
    load_hot_tables<float>(tables, T);
    if (a.acc_in) {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN;
        for (int i = threadIdx.x; i < 2 * kN; i += blockDim.x) acc[i] = src[i];
    } else {
        const int32_t* xs = a.x + (size_t)c * (n + 1);
        const int barb = mod_switch_2n(xs[n]);
        for (int i = threadIdx.x; i < kN; i += blockDim.x) {
            acc[i] = 0;
            acc[kN + i] = test_vector_coef(a, c, barb, i);
        }
    }
    __syncthreads();

    const FftTwiddles<float> tw = hot_twiddles<float>(tables);
    const FftIdx ix = make_fft_idx(t);
    const FftScratch<float> sc = scratch_at<float>(smem + Plan::scratch_off + (size_t)g * Plan::scratch);
    const int bar_id = 1 + g;
    const int halfBg = 1 << (kp.Bgbit - 1);
    const uint32_t mask = (1u << kp.Bgbit) - 1;
    const int decal = 32 - (lev + 1) * kp.Bgbit;
    const cpx<float>* gsw = reinterpret_cast<const cpx<float>*>(a.gsw);
    const size_t step_elems = (size_t)kRows * kRowElems;
    const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
    const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
    int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
    if (threadIdx.x < kRows) bulk_prefetch_l2(gsw + (size_t)threadIdx.x * kRowElems, kRowElems * sizeof(cpx<float>));
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const int ai = a_next;
        if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
        if (ai == 0) continue;  // tfhe_blindRotate_FFT.cpp:114 (uniform over the CTA)
        const cpx<float>* step_keys = gsw + (size_t)i * step_elems;
        if (i + 1 < n && threadIdx.x < kRows)  // the next step's rows into L2
            bulk_prefetch_l2(step_keys + step_elems + (size_t)threadIdx.x * kRowElems,
                             kRowElems * sizeof(cpx<float>));
        // the owners' key loads go out first: their L2 latency overlaps the
        // rotation, the digits and the forward transform
        float4 kk[kRows][4];
        if (owner) {
#pragma unroll
            for (int p = 0; p < kRows; ++p) {
                const float4* g4 =
                    reinterpret_cast<const float4*>(step_keys + (size_t)p * kRowElems + (oj * 2 + opt) * kHalf);
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) kk[p][qq] = __ldg(g4 + qq * 64 + t);
            }
        }
        cpx<float> v[8];
        {
            const int32_t* src = acc + jp * kN;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int x0 = t + 64 * r;
                const uint32_t u0 = (uint32_t)rot_coef(src, x0, ai) - (uint32_t)src[x0] + kp.offset;
                const uint32_t u1 =
                    (uint32_t)rot_coef(src, x0 + kHalf, ai) - (uint32_t)src[x0 + kHalf] + kp.offset;
                v[r] = digit_pair<float>(u0, u1, decal, mask, halfBg);
            }
        }
        fft512_forward_ip1(v, sc.b0, tw, ix, t, bar_id);
#pragma unroll
        for (int q = 0; q < 8; ++q) dsh[(g * 8 + q) * 64 + t] = v[q];
        __syncthreads();  // every D written, every read of acc done
        if (owner) {
            cpx<float> o[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = {0.f, 0.f};
#pragma unroll
            for (int p = 0; p < kRows; ++p)
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const cpx<float> d0 = dsh[(p * 8 + 2 * qq) * 64 + t];
                    const cpx<float> d1 = dsh[(p * 8 + 2 * qq + 1) * 64 + t];
                    o[2 * qq] = cmac(o[2 * qq], d0, cpx<float>{kk[p][qq].x, kk[p][qq].y});
                    o[2 * qq + 1] = cmac(o[2 * qq + 1], d1, cpx<float>{kk[p][qq].z, kk[p][qq].w});
                }
            fft512_inverse_ip1(o, sc.b0, tw, ix, t, bar_id);
            uint32_t c0[8] = {}, c1[8] = {};  // the low part adds into them
            round_part<float, 2>(o, opt, kp.split, c0, c1);
            int32_t* dst = acc + oj * kN;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int x0 = t + 64 * q;
                atomicAdd(reinterpret_cast<unsigned*>(dst + x0), c0[q]);
                atomicAdd(reinterpret_cast<unsigned*>(dst + x0 + kHalf), c1[q]);
            }
        }
        __syncthreads();  // the accumulator is updated before the next step reads it
    }
    if (a.acc_out) {
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN;
        for (int i = threadIdx.x; i < 2 * kN; i += blockDim.x) dst[i] = acc[i];
    }
    if (a.lwe_out) {
        // tLweExtractLweSample: a'_0 = a_0, a'_j = -a_{N-j}, b' = b_0
        int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
        for (int i = threadIdx.x; i < kN; i += blockDim.x)
            dst[i] = i == 0 ? acc[0] : (int32_t)(0u - (uint32_t)acc[kN - i]);
        if (threadIdx.x == 0) dst[kN] = acc[kN];
    }
}

// ----------------------------------------------------------------------
// Blind rotation with one ciphertext over a cluster of two CTAs (two SMs).
//
// The spread kernel's work split across two SMs: CTA r of the cluster holds
// accumulator polynomial r, runs the l forward transforms of polynomial r
// (one per group) and owns output polynomial r (groups 0 and 1: the high and
// the low key part).  Each group writes its transformed digits D_(r,lev) to
// its own shared memory and pushes them into the peer CTA's (distributed
// shared memory); once the peer's digits have landed the owners multiply all 2l rows
// -- l local, l from the peer -- in row order with their part of each key
// row, transform back, round and add into the local accumulator with
// integer atomics.  The accumulator never crosses SMs, only 4 KB of digits
// per group and step do.
//
// The pushes are asynchronous stores (st.async) that count their bytes on
// the receiving CTA's mbarrier for that step: the owners wait (bounded) for
// the peer's l x 4 KB to land, with no cluster-wide barrier and no release
// fence on the sender.  Pushes alternate between two buffers, each with its
// own mbarrier.  A push into buffer b at step k cannot overtake the peer's
// reads of b at step k - 2: the pushing CTA has by then received the peer's
// step k - 1 digits, which the peer sends only after its step k - 2
// products.  Each SM carries half the spread kernel's shared-memory traffic
// and transforms; the products are summed in the same order as every other
// shape, so the ciphertexts are bit-identical to the spread kernel's.
// Split-FP32 only, 1 CTA per SM (the shared-memory request is padded so
// that the two CTAs take two SMs).
// ----------------------------------------------------------------------
template <int L>
struct Spread2Plan {
    static constexpr size_t tables = kHotSize * sizeof(cpx<float>);
    static constexpr size_t acc_off = tables;                                     // own polynomial
    static constexpr size_t dloc_off = acc_off + kN * sizeof(int32_t);           // [lev][q][t]
    static constexpr size_t drem_off = dloc_off + L * kHalf * sizeof(cpx<float>);  // [buf][lev][q][t]
    static constexpr size_t scratch_off = drem_off + 2 * L * kHalf * sizeof(cpx<float>);
    static constexpr size_t scratch = 2 * kScratchStride * sizeof(cpx<float>);
    static constexpr size_t bar_off = scratch_off + L * scratch;  // 2 mbarriers, abort flag
    static constexpr size_t total = bar_off + 2 * sizeof(uint64_t) + 16;
    static constexpr size_t request = total > 120 * 1024 ? total : 120 * 1024;  // one CTA per SM
};

template <int L>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(64 * L, 1)
    k_blind_rotate_spread2(KParams kp, Tables T, EpArgs a) {
    static_assert(L >= 2, "two owner groups per CTA");
    namespace cg = cooperative_groups;
    using Plan = Spread2Plan<L>;
    constexpr int kRows = 2 * L;
    constexpr int kRowElems = 2 * 2 * kHalf;  // complex values per key row
    extern __shared__ __align__(128) char smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();  // this CTA's polynomial
    cpx<float>* tables = reinterpret_cast<cpx<float>*>(smem);
    int32_t* acc = reinterpret_cast<int32_t*>(smem + Plan::acc_off);
    cpx<float>* dloc = reinterpret_cast<cpx<float>*>(smem + Plan::dloc_off);
    cpx<float>* drem = reinterpret_cast<cpx<float>*>(smem + Plan::drem_off);
    uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Plan::bar_off);  // per buffer
    volatile int* abort = reinterpret_cast<volatile int*>(smem + Plan::bar_off + 2 * sizeof(uint64_t));
    // the peer's digit buffers and their mbarriers, as shared::cluster addresses
    const uint32_t drem_peer = cluster_map(smem_u32(drem), (uint32_t)(r ^ 1));
    const uint32_t dbar_peer = cluster_map(smem_u32(dbar), (uint32_t)(r ^ 1));
    const int c = blockIdx.x >> 1;
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int lev = g;
    const bool owner = g < 2;
    const int opt = g & 1;
    const int n = kp.n;
    load_hot_tables<float>(tables, T);
    if (a.acc_in) {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN + (size_t)r * kN;
        for (int i = threadIdx.x; i < kN; i += blockDim.x) acc[i] = src[i];
    } else {
        const int32_t* xs = a.x + (size_t)c * (n + 1);
        const int barb = mod_switch_2n(xs[n]);
        for (int i = threadIdx.x; i < kN; i += blockDim.x) acc[i] = r == 0 ? 0 : test_vector_coef(a, c, barb, i);
    }
    if (threadIdx.x == 0) {
        mbar_init(&dbar[0], 1);
        mbar_init(&dbar[1], 1);
        *abort = 0;
        fence_mbar_init();
    }
    cluster.sync();  // both CTAs' barriers initialised before any push

    const FftTwiddles<float> tw = hot_twiddles<float>(tables);
    const FftIdx ix = make_fft_idx(t);
    const FftScratch<float> sc = scratch_at<float>(smem + Plan::scratch_off + (size_t)g * Plan::scratch);
    const int bar_id = 1 + g;
    const int halfBg = 1 << (kp.Bgbit - 1);
    const uint32_t mask = (1u << kp.Bgbit) - 1;
    const int decal = 32 - (lev + 1) * kp.Bgbit;
    const cpx<float>* gsw = reinterpret_cast<const cpx<float>*>(a.gsw);
    const size_t step_elems = (size_t)kRows * kRowElems;
    const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
    const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
    int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
    if (threadIdx.x < kRows && (threadIdx.x & 1) == r)
        bulk_prefetch_l2(gsw + (size_t)threadIdx.x * kRowElems, kRowElems * sizeof(cpx<float>));
    uint32_t k = 0;  // steps taken (the same in both CTAs)
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const int ai = a_next;
        if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
        if (ai == 0) continue;  // tfhe_blindRotate_FFT.cpp:114 (uniform over the cluster)
        const int buf = (int)(k & 1);
        // this step's incoming digits: one arrival and l x 4 KB of stores
        if (threadIdx.x == 0) mbar_arrive_expect_tx(&dbar[buf], (uint32_t)(L * kHalf * sizeof(cpx<float>)));
        const cpx<float>* step_keys = gsw + (size_t)i * step_elems;
        if (i + 1 < n && threadIdx.x < kRows && (threadIdx.x & 1) == r)  // next step's rows into L2
            bulk_prefetch_l2(step_keys + step_elems + (size_t)threadIdx.x * kRowElems,
                             kRowElems * sizeof(cpx<float>));
        float4 kk[kRows][4];
        if (owner) {  // part (r, opt) of every row, issued before the transform
#pragma unroll
            for (int p = 0; p < kRows; ++p) {
                const float4* g4 =
                    reinterpret_cast<const float4*>(step_keys + (size_t)p * kRowElems + (r * 2 + opt) * kHalf);
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) kk[p][qq] = __ldg(g4 + qq * 64 + t);
            }
        }
        cpx<float> v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int x0 = t + 64 * q;
            const uint32_t u0 = (uint32_t)rot_coef(acc, x0, ai) - (uint32_t)acc[x0] + kp.offset;
            const uint32_t u1 = (uint32_t)rot_coef(acc, x0 + kHalf, ai) - (uint32_t)acc[x0 + kHalf] + kp.offset;
            v[q] = digit_pair<float>(u0, u1, decal, mask, halfBg);
        }
        fft512_forward_ip1(v, sc.b0, tw, ix, t, bar_id);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int e = (lev * 8 + q) * 64 + t;
            dloc[e] = v[q];
            st_async_f2(drem_peer + (uint32_t)((buf * L * kHalf + e) * sizeof(cpx<float>)), v[q].x, v[q].y,
                        dbar_peer + (uint32_t)(buf * sizeof(uint64_t)));
        }
        __syncthreads();  // every local D in place; every read of acc done
        if (owner) {
            if (!mbar_wait_cluster_bounded(&dbar[buf], (k >> 1) & 1, abort)) {  // the peer's D landed
                *abort = 1;
                atomicExch(a.err, 3);
            }
            cpx<float> o[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = {0.f, 0.f};
#pragma unroll
            for (int p = 0; p < kRows; ++p) {
                const int jp = p / L, lv = p - jp * L;
                const cpx<float>* D = jp == r ? dloc + lv * kHalf : drem + (buf * L + lv) * kHalf;
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const cpx<float> d0 = D[(2 * qq) * 64 + t];
                    const cpx<float> d1 = D[(2 * qq + 1) * 64 + t];
                    o[2 * qq] = cmac(o[2 * qq], d0, cpx<float>{kk[p][qq].x, kk[p][qq].y});
                    o[2 * qq + 1] = cmac(o[2 * qq + 1], d1, cpx<float>{kk[p][qq].z, kk[p][qq].w});
                }
            }
            fft512_inverse_ip1(o, sc.b0, tw, ix, t, bar_id);
            uint32_t c0[8] = {}, c1[8] = {};  // the low part adds into them
            round_part<float, 2>(o, opt, kp.split, c0, c1);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int x0 = t + 64 * q;
                atomicAdd(reinterpret_cast<unsigned*>(acc + x0), c0[q]);
                atomicAdd(reinterpret_cast<unsigned*>(acc + x0 + kHalf), c1[q]);
            }
        }
        ++k;
        __syncthreads();  // the accumulator is updated before the next step reads it
    }
    if (a.acc_out) {
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN + (size_t)r * kN;
        for (int i = threadIdx.x; i < kN; i += blockDim.x) dst[i] = acc[i];
    }
    if (a.lwe_out) {
        // tLweExtractLweSample: a'_0 = a_0, a'_j = -a_{N-j} (polynomial 0),
        // b' = b_0 (polynomial 1)
        int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
        if (r == 0) {
            for (int i = threadIdx.x; i < kN; i += blockDim.x)
                dst[i] = i == 0 ? acc[0] : (int32_t)(0u - (uint32_t)acc[kN - i]);
        } else if (threadIdx.x == 0) {
            dst[kN] = acc[0];
        }
    }
    cluster.sync();  // no CTA leaves while its peer could still address its shared memory
}

// ----------------------------------------------------------------------
// The FP64 form's blind rotation over a cluster of two CTAs (lowest FP64
// latency).  The same split as k_blind_rotate_spread2: CTA r holds
// accumulator polynomial r and runs its l forward transforms (one per group),
// pushes the transformed digits into the peer's shared memory (asynchronous
// stores counted on the peer's mbarrier, two alternating buffers), and owns
// output polynomial r.  The FP64 key has one part, so one owner group per
// CTA (group 0) multiplies all 2l rows in row order with output r's part of
// each key row, transforms back and truncates like the reference
// (TorusPolynomial_fft.cpp:40).  The transforms, the products and their
// order are those of the other FP64 shapes.  A single FP64 gate then runs on
// two SMs' FP64 pipes instead of one 64-thread group.
// ----------------------------------------------------------------------
template <int L>
struct Spread2F64Plan {
    static constexpr size_t tables = kHotSize * sizeof(cpx<double>);
    static constexpr size_t acc_off = tables;                                       // own polynomial
    static constexpr size_t dloc_off = acc_off + kN * sizeof(int32_t);             // [lev][q][t]
    static constexpr size_t drem_off = dloc_off + L * kHalf * sizeof(cpx<double>);  // [buf][lev][q][t]
    static constexpr size_t scratch_off = drem_off + 2 * L * kHalf * sizeof(cpx<double>);
    static constexpr size_t scratch = 2 * kScratchStride * sizeof(cpx<double>);
    static constexpr size_t bar_off = scratch_off + L * scratch;  // 2 mbarriers, abort flag
    static constexpr size_t total = bar_off + 2 * sizeof(uint64_t) + 16;
    static constexpr size_t request = total > 120 * 1024 ? total : 120 * 1024;  // one CTA per SM
    static_assert(dloc_off % 16 == 0 && drem_off % 16 == 0 && bar_off % 8 == 0, "alignment");
};

template <int L>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(64 * L, 1)
    k_blind_rotate_spread2_f64(KParams kp, Tables T, EpArgs a) {
    namespace cg = cooperative_groups;
    using Plan = Spread2F64Plan<L>;
    constexpr int kRows = 2 * L;
    constexpr int kRowElems = 2 * kHalf;  // complex values per key row (two outputs, one part)
    constexpr int kEarly = L;             // rows whose key values the owner loads before the transform
    extern __shared__ __align__(128) char smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();  // this CTA's polynomial
    cpx<double>* tables = reinterpret_cast<cpx<double>*>(smem);
    int32_t* acc = reinterpret_cast<int32_t*>(smem + Plan::acc_off);
    cpx<double>* dloc = reinterpret_cast<cpx<double>*>(smem + Plan::dloc_off);
    cpx<double>* drem = reinterpret_cast<cpx<double>*>(smem + Plan::drem_off);
    uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Plan::bar_off);  // per buffer
    volatile int* abort = reinterpret_cast<volatile int*>(smem + Plan::bar_off + 2 * sizeof(uint64_t));
    const uint32_t drem_peer = cluster_map(smem_u32(drem), (uint32_t)(r ^ 1));
    const uint32_t dbar_peer = cluster_map(smem_u32(dbar), (uint32_t)(r ^ 1));
    const int c = blockIdx.x >> 1;
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int lev = g;
    const bool owner = g == 0;
    const int n = kp.n;
    load_hot_tables<double>(tables, T);
    if (a.acc_in) {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN + (size_t)r * kN;
        for (int i = threadIdx.x; i < kN; i += blockDim.x) acc[i] = src[i];
    } else {
        const int32_t* xs = a.x + (size_t)c * (n + 1);
        const int barb = mod_switch_2n(xs[n]);
        for (int i = threadIdx.x; i < kN; i += blockDim.x) acc[i] = r == 0 ? 0 : test_vector_coef(a, c, barb, i);
    }
    if (threadIdx.x == 0) {
        mbar_init(&dbar[0], 1);
        mbar_init(&dbar[1], 1);
        *abort = 0;
        fence_mbar_init();
    }
    cluster.sync();  // both CTAs' barriers initialised before any push

    const FftTwiddles<double> tw = hot_twiddles<double>(tables);
    const FftIdx ix = make_fft_idx(t);
    const FftScratch<double> sc = scratch_at<double>(smem + Plan::scratch_off + (size_t)g * Plan::scratch);
    const int bar_id = 1 + g;
    const int halfBg = 1 << (kp.Bgbit - 1);
    const uint32_t mask = (1u << kp.Bgbit) - 1;
    const int decal = 32 - (lev + 1) * kp.Bgbit;
    const cpx<double>* gsw = reinterpret_cast<const cpx<double>*>(a.gsw);
    const size_t step_elems = (size_t)kRows * kRowElems;
    const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
    const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
    int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
    if (threadIdx.x < kRows)  // output r's part of the first step's rows into L2
        bulk_prefetch_l2(gsw + (size_t)threadIdx.x * kRowElems + r * kHalf, kHalf * sizeof(cpx<double>));
    uint32_t k = 0;  // steps taken (the same in both CTAs)
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const int ai = a_next;
        if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
        if (ai == 0) continue;  // tfhe_blindRotate_FFT.cpp:114 (uniform over the cluster)
        const int buf = (int)(k & 1);
        // this step's incoming digits: one arrival and l x 8 KB of stores
        if (threadIdx.x == 0) mbar_arrive_expect_tx(&dbar[buf], (uint32_t)(L * kHalf * sizeof(cpx<double>)));
        const cpx<double>* step_keys = gsw + (size_t)i * step_elems;
        if (i + 1 < n && threadIdx.x < kRows)  // the next step's rows into L2
            bulk_prefetch_l2(step_keys + step_elems + (size_t)threadIdx.x * kRowElems + r * kHalf,
                             kHalf * sizeof(cpx<double>));
        // the owner's first rows go out before the transform, so their L2
        // latency overlaps it
        double2 kk[kEarly][8];
        if (owner) {
#pragma unroll
            for (int p = 0; p < kEarly; ++p) {
                const double2* g2 = reinterpret_cast<const double2*>(step_keys + (size_t)p * kRowElems + r * kHalf);
#pragma unroll
                for (int q = 0; q < 8; ++q) kk[p][q] = __ldg(g2 + key_index<double>(t, q));
            }
        }
        cpx<double> v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int x0 = t + 64 * q;
            const uint32_t u0 = (uint32_t)rot_coef(acc, x0, ai) - (uint32_t)acc[x0] + kp.offset;
            const uint32_t u1 = (uint32_t)rot_coef(acc, x0 + kHalf, ai) - (uint32_t)acc[x0 + kHalf] + kp.offset;
            v[q] = digit_pair<double>(u0, u1, decal, mask, halfBg);
        }
        fft512_forward_ip1(v, sc.b0, tw, ix, t, bar_id);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int e = (lev * 8 + q) * 64 + t;
            dloc[e] = v[q];
            st_async_d2(drem_peer + (uint32_t)((buf * L * kHalf + e) * sizeof(cpx<double>)), v[q].x, v[q].y,
                        dbar_peer + (uint32_t)(buf * sizeof(uint64_t)));
        }
        __syncthreads();  // every local D in place; every read of acc done
        if (owner) {
            if (!mbar_wait_cluster_bounded(&dbar[buf], (k >> 1) & 1, abort)) {  // the peer's D landed
                *abort = 1;
                atomicExch(a.err, 3);
            }
            cpx<double> o[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = {0.0, 0.0};
#pragma unroll
            for (int p = 0; p < kRows; ++p) {
                const int jp = p / L, lv = p - jp * L;
                const cpx<double>* D = jp == r ? dloc + lv * kHalf : drem + (buf * L + lv) * kHalf;
                const double2* g2 = reinterpret_cast<const double2*>(step_keys + (size_t)p * kRowElems + r * kHalf);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const double2 w = p < kEarly ? kk[p < kEarly ? p : 0][q] : __ldg(g2 + key_index<double>(t, q));
                    o[q] = cmac(o[q], D[q * 64 + t], cpx<double>{w.x, w.y});
                }
            }
            fft512_inverse_ip1(o, sc.b0, tw, ix, t, bar_id);
            uint32_t c0[8], c1[8];
            round_part<double, 1>(o, 0, kp.split, c0, c1);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int x0 = t + 64 * q;
                acc[x0] = (int32_t)((uint32_t)acc[x0] + c0[q]);
                acc[x0 + kHalf] = (int32_t)((uint32_t)acc[x0 + kHalf] + c1[q]);
            }
        }
        ++k;
        __syncthreads();  // the accumulator is updated before the next step reads it
    }
    if (a.acc_out) {
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN + (size_t)r * kN;
        for (int i = threadIdx.x; i < kN; i += blockDim.x) dst[i] = acc[i];
    }
    if (a.lwe_out) {
        // tLweExtractLweSample: a'_0 = a_0, a'_j = -a_{N-j} (polynomial 0),
        // b' = b_0 (polynomial 1)
        int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
        if (r == 0) {
            for (int i = threadIdx.x; i < kN; i += blockDim.x)
                dst[i] = i == 0 ? acc[0] : (int32_t)(0u - (uint32_t)acc[kN - i]);
        } else if (threadIdx.x == 0) {
            dst[kN] = acc[0];
        }
    }
    cluster.sync();  // no CTA leaves while its peer could still address its shared memory
}

// ----------------------------------------------------------------------
// Blind rotation with two 64-thread halves per ciphertext (low latency).
//
// Half h of a ciphertext decomposes and transforms input polynomial h (rows
// h l .. h l + l - 1 of every key step), multiply-accumulates them into the
// partial products of both output polynomials, hands the partial of output
// 1 - h to the other half through shared memory, and transforms back only
// output h.  Each half reads and writes only accumulator polynomial h, so the
// halves meet once per step (the partial exchange).  Per step and half: l
// forward and PARTS inverse transforms instead of 2l and 2 PARTS, so a
// ciphertext takes about half the time; used when a batch has at most three
// ciphertexts per SM to spread (the last partial wave of a large batch,
// small batches, single gates).  Key rows come through the same shared ring
// as k_blind_rotate_ring; each row is read by one half of every ciphertext.
// ----------------------------------------------------------------------
__device__ __forceinline__ void pair_sync(int bar_id) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(2 * kFftThreads) : "memory");
}

// h is the half; out[h] and out[1 - h] are picked by uniform branches so
// that the accumulators stay in registers with one copy of the code.
template <typename R, int PARTS, int L, typename Keys>
__device__ __forceinline__ void ep_step_half(const StepCtx<R, PARTS, 1>& S, Keys& keys, int a, int h,
                                             cpx<R>* peer_inbox, int pair_bar) {
    const int t = S.t;
    const int halfBg = 1 << (S.Bgbit - 1);
    const uint32_t mask = (1u << S.Bgbit) - 1;

    cpx<R> out[2][PARTS][8];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int pt = 0; pt < PARTS; ++pt)
#pragma unroll
            for (int q = 0; q < 8; ++q) out[j][pt][q] = {(R)0, (R)0};

    {
        const int32_t* src = S.acc + h * kN;
        uint32_t r0[8], r1[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int x0 = t + 64 * r;
            r0[r] = (uint32_t)rot_coef(src, x0, a) - (uint32_t)src[x0] + S.offset;
            r1[r] = (uint32_t)rot_coef(src, x0 + kHalf, a) - (uint32_t)src[x0 + kHalf] + S.offset;
        }
#pragma unroll 1
        for (int lev = 0; lev < L; ++lev) {
            cpx<R> v[8];
            const int decal = 32 - (lev + 1) * S.Bgbit;
#pragma unroll
            for (int r = 0; r < 8; ++r)
                v[r] = digit_pair<R>(r0[r], r1[r], decal, mask, halfBg);
            fft512_forward_tw(v, S.s[0], S.tw, S.ix, t, S.bar_id);
            const int p = h * L + lev;
            mac_row<R, PARTS, Keys::kShared>(out, v, keys.acquire(p), t);
            keys.release(p);
        }
    }
    // every row of this step is issued before the producer waits on its pair
    if (keys.producer) keys.issue_through(keys.row0 + 2 * L - 1);

    // exchange: both halves' forward transforms are done, so their scratch
    // buffers are free; write the partial of output 1 - h into the other
    // half's scratch, then read this half's own
    pair_sync(pair_bar);
#pragma unroll
    for (int pt = 0; pt < PARTS; ++pt) {
        cpx<R> w[8];
        pick_part<R, PARTS>(w, out, 1 - h, pt);
#pragma unroll
        for (int q = 0; q < 8; ++q) peer_inbox[pt * kScratchStride + q * 64 + t] = w[q];
    }
    pair_sync(pair_bar);
    // the next step's first rows land during this step's inverse transforms
    if (keys.producer) keys.issue_upto(keys.row0 + 2 * L - 1);
    {
        const cpx<R>* inbox = S.s[0].b0;
#pragma unroll
        for (int pt = 0; pt < PARTS; ++pt) {
            cpx<R> w[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) w[q] = inbox[pt * kScratchStride + q * 64 + t];
            add_part<R, PARTS>(out, w, h, pt);
        }
    }
    group_sync(S.bar_id);  // the inbox is the transform's scratch

    uint32_t c0[8], c1[8];
#pragma unroll 1
    for (int pt = 0; pt < PARTS; ++pt) {
        cpx<R> v[8];
        pick_part<R, PARTS>(v, out, h, pt);
        fft512_inverse_tw(v, S.s[0], S.tw, S.ix, t, S.bar_id);
        round_part<R, PARTS>(v, pt, S.split, c0, c1);
    }
    int32_t* dst = S.acc + h * kN;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int x0 = t + 64 * q;
        dst[x0] = (int32_t)((uint32_t)dst[x0] + c0[q]);
        dst[x0 + kHalf] = (int32_t)((uint32_t)dst[x0 + kHalf] + c1[q]);
    }
    group_sync(S.bar_id);
}

template <typename R, int PARTS, int PAIRS, int L, int S>
struct PairPlan {
    static constexpr size_t kRowBytes = (size_t)2 * PARTS * kHalf * sizeof(cpx<R>);
    static constexpr size_t tables = kHotSize * sizeof(cpx<R>);
    static constexpr size_t ring_off = (tables + 127) & ~(size_t)127;
    static constexpr size_t bar_off = ring_off + S * kRowBytes;
    static constexpr size_t flag_off = bar_off + 2 * S * sizeof(uint64_t);
    static constexpr size_t pair_off = (flag_off + sizeof(int) + 127) & ~(size_t)127;
    static constexpr size_t acc = 2 * kN * sizeof(int32_t);
    static constexpr size_t half_scratch = 2 * kScratchStride * sizeof(cpx<R>);
    static constexpr size_t pair = acc + 2 * half_scratch;
    static constexpr size_t total = pair_off + PAIRS * pair;
};

template <typename R, int PARTS, int PAIRS, int L, int S>
__global__ void __launch_bounds__(128 * PAIRS, 1) k_blind_rotate_pair(KParams kp, Tables T, EpArgs a) {
    using Plan = PairPlan<R, PARTS, PAIRS, L, S>;
    static_assert(1 + 2 * PAIRS + PAIRS <= 16, "named barriers");
    static_assert(PARTS * kScratchStride >= PARTS * kHalf, "inbox fits the scratch");
    constexpr int kpl = 2 * L;
    extern __shared__ __align__(128) char smem[];
    cpx<R>* tables = reinterpret_cast<cpx<R>*>(smem);
    cpx<R>* ring = reinterpret_cast<cpx<R>*>(smem + Plan::ring_off);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + Plan::bar_off);
    uint64_t* empty = full + S;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + Plan::flag_off);
    const int active = min(PAIRS, a.count - (int)blockIdx.x * PAIRS);
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 64 * active);  // one half of every ciphertext reads a row
        }
        *abort = 0;
        fence_mbar_init();
    }
    load_hot_tables<R>(tables, T);
    __syncthreads();

    const int pr = threadIdx.x >> 7;
    const int h = (threadIdx.x >> 6) & 1;
    const int t = threadIdx.x & 63;
    const int c = blockIdx.x * PAIRS + pr;
    if (pr >= active) return;
    const int n = kp.n;
    RingKeys<R, PARTS, S> keys{ring, full, empty, 0, a.err, abort, threadIdx.x == 0 && !a.stall_keys,
                               reinterpret_cast<const char*>(a.gsw), (uint32_t)n * kpl, 0, false};

    char* pbase = smem + Plan::pair_off + (size_t)pr * Plan::pair;
    StepCtx<R, PARTS, 1> St;
    St.tw = hot_twiddles<R>(tables);
    St.ix = make_fft_idx(t);
    St.acc = reinterpret_cast<int32_t*>(pbase);
    St.s[0] = scratch_at<R>(pbase + Plan::acc + h * Plan::half_scratch);
    cpx<R>* peer_inbox = reinterpret_cast<cpx<R>*>(pbase + Plan::acc + (1 - h) * Plan::half_scratch);
    St.t = t;
    St.bar_id = 1 + 2 * pr + h;
    const int pair_bar = 1 + 2 * PAIRS + pr;
    St.Bgbit = kp.Bgbit;
    St.split = kp.split;
    St.offset = kp.offset;

    // half h owns accumulator polynomial h
    int32_t* mine = St.acc + h * kN;
    if (a.acc_in) {
        const int32_t* src = a.acc_in + (size_t)c * 2 * kN + h * kN;
        for (int i = t; i < kN; i += 64) mine[i] = src[i];
    } else {
        const int32_t* xs = a.x + (size_t)c * (n + 1);
        const int barb = mod_switch_2n(xs[n]);
        for (int i = t; i < kN; i += 64)
            mine[i] = h == 0 ? 0 : test_vector_coef(a, c, barb, i);
    }
    group_sync(St.bar_id);
    const int32_t* bara = a.bara ? a.bara + (size_t)c * n : nullptr;
    const int32_t* xs = a.x ? a.x + (size_t)c * (n + 1) : nullptr;
    int a_next = bara ? bara[0] : mod_switch_2n(xs[0]);
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const int ai = a_next;
        if (i + 1 < n) a_next = bara ? bara[i + 1] : mod_switch_2n(xs[i + 1]);
        keys.row0 = (uint32_t)i * kpl;
        if (ai == 0) {  // tfhe_blindRotate_FFT.cpp:114 -- this half's rows still pass through
            for (int p = h * L; p < h * L + L; ++p) {
                keys.acquire(p);
                keys.release(p);
            }
            continue;
        }
        ep_step_half<R, PARTS, L>(St, keys, ai, h, peer_inbox, pair_bar);
    }
    if (keys.producer) {
        keys.issue_through(keys.total - 1);  // rows of a skipped last step
        keys.drain();
    }
    pair_sync(pair_bar);  // both polynomials final
    if (a.acc_out) {
        int32_t* dst = a.acc_out + (size_t)c * 2 * kN + h * kN;
        for (int i = t; i < kN; i += 64) dst[i] = mine[i];
    }
    if (a.lwe_out) {
        // tLweExtractLweSample: a'_0 = a_0, a'_j = -a_{N-j}, b' = b_0
        int32_t* dst = a.lwe_out + (size_t)c * (kN + 1);
        const int tt = h * 64 + t;
        for (int i = tt; i < kN; i += 128)
            dst[i] = i == 0 ? St.acc[0] : (int32_t)(0u - (uint32_t)St.acc[kN - i]);
        if (tt == 0) dst[kN] = St.acc[kN];
    }
}

// ----------------------------------------------------------------------
// key conversion: one 64-thread group per polynomial
// ----------------------------------------------------------------------
__device__ __forceinline__ void twisted_forward64(const double* coef, cpx<double> (&v)[8],
                                                  const FftScratch<double>& s,
                                                  const FftTwiddles<double>& tw,
                                                  const cpx<double>* psi, int t, int bar) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int x0 = t + 64 * r;
        v[r] = cmul(cpx<double>{coef[x0], coef[x0 + kHalf]}, psi[x0]);
    }
    fft512_forward(v, s, tw, t, bar);
}

// Per polynomial smem: 1024 doubles of coefficients + scratch.
constexpr size_t kConvGroupBytes = kN * sizeof(double) + 2 * kScratchStride * sizeof(cpx<double>);
constexpr size_t kConvTableBytes = kTabSize * sizeof(cpx<double>);

template <int FORM>
__global__ void __launch_bounds__(256) k_tgsw_to_fft(Tables T, const int32_t* __restrict__ in,
                                                     void* out, int npoly, int split) {
    extern __shared__ __align__(128) char smem[];
    cpx<double>* tables = reinterpret_cast<cpx<double>*>(smem);
    load_tables<double>(tables, T);
    __syncthreads();
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int poly = blockIdx.x * (blockDim.x >> 6) + g;
    if (poly >= npoly) return;
    char* gbase = smem + kConvTableBytes + (size_t)g * kConvGroupBytes;
    double* coef = reinterpret_cast<double*>(gbase);
    FftScratch<double> s = scratch_at<double>(gbase + kN * sizeof(double));
    const int32_t* src = in + (size_t)poly * kN;
    const int bar = 1 + g;

    if (FORM == kFormFp64) {
        for (int i = t; i < kN; i += 64) coef[i] = (double)src[i];
        group_sync(bar);
        cpx<double> v[8];
        twisted_forward64(coef, v, s, twiddles_at<double>(tables), tables + kTabPsi, t, bar);
        cpx<double>* dst = reinterpret_cast<cpx<double>*>(out) + (size_t)poly * kHalf;
#pragma unroll
        for (int q = 0; q < 8; ++q) dst[key_index<double>(t, q)] = v[q];
    } else {
        // split K = Khi * 2^s + Klo, Klo in [-2^(s-1), 2^(s-1))
        cpx<float>* dst = reinterpret_cast<cpx<float>*>(out) + (size_t)poly * 2 * kHalf;
        for (int part = 0; part < 2; ++part) {
            for (int i = t; i < kN; i += 64) {
                const int64_t K = src[i];
                const int64_t half = (int64_t)1 << (split - 1);
                const int64_t lo = ((K + half) & (((int64_t)1 << split) - 1)) - half;
                const int64_t hi = (K - lo) >> split;
                coef[i] = (double)(part == 0 ? hi : lo);
            }
            group_sync(bar);
            cpx<double> v[8];
            twisted_forward64(coef, v, s, twiddles_at<double>(tables), tables + kTabPsi, t, bar);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                dst[part * kHalf + key_index<float>(t, q)] = {(float)v[q].x, (float)v[q].y};
            group_sync(bar);
        }
    }
}

// engine FP64 layout -> integer coefficients (rounded to nearest)
__global__ void __launch_bounds__(256) k_fft64_to_tgsw(Tables T, const void* in,
                                                       int32_t* __restrict__ out, int npoly) {
    extern __shared__ __align__(128) char smem[];
    cpx<double>* tables = reinterpret_cast<cpx<double>*>(smem);
    load_tables<double>(tables, T);
    __syncthreads();
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int poly = blockIdx.x * (blockDim.x >> 6) + g;
    if (poly >= npoly) return;
    char* gbase = smem + kConvTableBytes + (size_t)g * kConvGroupBytes;
    FftScratch<double> s = scratch_at<double>(gbase + kN * sizeof(double));
    const cpx<double>* src = reinterpret_cast<const cpx<double>*>(in) + (size_t)poly * kHalf;
    cpx<double> v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = src[key_index<double>(t, q)];
    fft512_inverse(v, s, twiddles_at<double>(tables), t, 1 + g);
    int32_t* dst = out + (size_t)poly * kN;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const cpx<double> z = cmulc(v[q], tables[kTabPsi + t + 64 * q]);
        dst[t + 64 * q] = (int32_t)(uint32_t)(uint64_t)llrint(z.x / 512.0);
        dst[t + 64 * q + kHalf] = (int32_t)(uint32_t)(uint64_t)llrint(z.y / 512.0);
    }
}

// ----------------------------------------------------------------------
// Lagrange half-complex form in the reference layout: value m' is
// P(w^(2m'+1)), w = e^{i pi/N}.  Engine frequency m is P(psi^(4m+1)).
// ----------------------------------------------------------------------
__device__ __forceinline__ void engine_to_ref_index(int m, int* ref, bool* conj) {
    const int e = (4 * m + 1) & 2047;
    if (e < kN) {
        *ref = (e - 1) >> 1;
        *conj = false;
    } else {
        *ref = (2048 - e - 1) >> 1;
        *conj = true;
    }
}

// in: count polynomials (int32 coefficients), out: count x 512 complex
// doubles in the reference layout, multiplied by `scale`.
__global__ void __launch_bounds__(256) k_poly_to_lagrange(Tables T, const int32_t* __restrict__ in,
                                                          double* __restrict__ out, int npoly,
                                                          double scale) {
    extern __shared__ __align__(128) char smem[];
    cpx<double>* tables = reinterpret_cast<cpx<double>*>(smem);
    load_tables<double>(tables, T);
    __syncthreads();
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int poly = blockIdx.x * (blockDim.x >> 6) + g;
    if (poly >= npoly) return;
    char* gbase = smem + kConvTableBytes + (size_t)g * kConvGroupBytes;
    double* coef = reinterpret_cast<double*>(gbase);
    FftScratch<double> s = scratch_at<double>(gbase + kN * sizeof(double));
    const int32_t* src = in + (size_t)poly * kN;
    for (int i = t; i < kN; i += 64) coef[i] = (double)src[i];
    group_sync(1 + g);
    cpx<double> v[8];
    twisted_forward64(coef, v, s, twiddles_at<double>(tables), tables + kTabPsi, t, 1 + g);
    double* dst = out + (size_t)poly * kN;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        int ref;
        bool cj;
        engine_to_ref_index(freq_of(t, q), &ref, &cj);
        dst[2 * ref] = v[q].x * scale;
        dst[2 * ref + 1] = (cj ? -v[q].y : v[q].y) * scale;
    }
}

// TorusPolynomial_fft: reference-layout values (torus / 2^32 scale) ->
// Torus32 coefficients, truncating like TorusPolynomial_fft.cpp:39-41.
__global__ void __launch_bounds__(256) k_lagrange_to_torus(Tables T, const double* __restrict__ in,
                                                           int32_t* __restrict__ out, int npoly) {
    extern __shared__ __align__(128) char smem[];
    cpx<double>* tables = reinterpret_cast<cpx<double>*>(smem);
    load_tables<double>(tables, T);
    __syncthreads();
    const int g = threadIdx.x >> 6, t = threadIdx.x & 63;
    const int poly = blockIdx.x * (blockDim.x >> 6) + g;
    if (poly >= npoly) return;
    char* gbase = smem + kConvTableBytes + (size_t)g * kConvGroupBytes;
    FftScratch<double> s = scratch_at<double>(gbase + kN * sizeof(double));
    const double* src = in + (size_t)poly * kN;
    cpx<double> v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        int ref;
        bool cj;
        engine_to_ref_index(freq_of(t, q), &ref, &cj);
        const double re = src[2 * ref], im = src[2 * ref + 1];
        v[q] = {re, cj ? -im : im};
    }
    fft512_inverse(v, s, twiddles_at<double>(tables), t, 1 + g);
    const double sc = 4294967296.0 / 512.0;
    int32_t* dst = out + (size_t)poly * kN;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const cpx<double> z = cmulc(v[q], tables[kTabPsi + t + 64 * q]);
        dst[t + 64 * q] = (int32_t)(uint32_t)(uint64_t)__double2ll_rz(z.x * sc);
        dst[t + 64 * q + kHalf] = (int32_t)(uint32_t)(uint64_t)__double2ll_rz(z.y * sc);
    }
}

// reference layout <-> engine FP64 layout, values multiplied by `scale`
__global__ void k_ref_to_engine64(const double* __restrict__ ref, cpx<double>* __restrict__ eng,
                                  int npoly, double scale) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npoly * kHalf) return;
    const int poly = idx / kHalf, e = idx % kHalf;
    const int t = e & 63, q = e >> 6;
    int r;
    bool cj;
    engine_to_ref_index(freq_of(t, q), &r, &cj);
    const double re = ref[(size_t)poly * kN + 2 * r], im = ref[(size_t)poly * kN + 2 * r + 1];
    eng[(size_t)poly * kHalf + key_index<double>(t, q)] = {re * scale, (cj ? -im : im) * scale};
}

__global__ void k_engine64_to_ref(const cpx<double>* __restrict__ eng, double* __restrict__ ref,
                                  int npoly, double scale) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npoly * kHalf) return;
    const int poly = idx / kHalf, e = idx % kHalf;
    const int t = e & 63, q = e >> 6;
    int r;
    bool cj;
    engine_to_ref_index(freq_of(t, q), &r, &cj);
    const cpx<double> v = eng[(size_t)poly * kHalf + key_index<double>(t, q)];
    ref[(size_t)poly * kN + 2 * r] = v.x * scale;
    ref[(size_t)poly * kN + 2 * r + 1] = (cj ? -v.y : v.y) * scale;
}

// LagrangeHalfCPolynomialAddMul (tGswFFTExternMulToTLwe.cpp:172-180)
__global__ void k_lagrange_addmul(const double* __restrict__ a, const double* __restrict__ b,
                                  double* __restrict__ acc, size_t total) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const double ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
    acc[2 * i] += ar * br - ai * bi;
    acc[2 * i + 1] += ar * bi + ai * br;
}

// ----------------------------------------------------------------------
// small kernels
// ----------------------------------------------------------------------
__device__ __forceinline__ void gate_coeffs(int gate, int32_t e8, int32_t e4, int32_t* c,
                                            int32_t* sa, int32_t* sb) {
    switch (gate) {
    case 0: *c = e8; *sa = -1; *sb = -1; break;   // NAND
    case 1: *c = -e8; *sa = 1; *sb = 1; break;    // AND
    case 2: *c = e8; *sa = 1; *sb = 1; break;     // OR
    case 3: *c = e4; *sa = 2; *sb = 2; break;     // XOR
    case 4: *c = -e4; *sa = -2; *sb = -2; break;  // XNOR
    case 5: *c = -e8; *sa = -1; *sb = -1; break;  // NOR
    case 6: *c = -e8; *sa = -1; *sb = 1; break;   // ANDNY
    case 7: *c = -e8; *sa = 1; *sb = -1; break;   // ANDYN
    case 8: *c = e8; *sa = -1; *sb = 1; break;    // ORNY
    case 9: *c = e8; *sa = 1; *sb = -1; break;    // ORYN
    default: *c = 0; *sa = 0; *sb = 0; break;
    }
}

__global__ void k_gate_combine(int n, const int32_t* __restrict__ gates, int uniform_gate,
                               const int32_t* __restrict__ ca, const int32_t* __restrict__ cb,
                               int32_t* __restrict__ out, int count) {
    const size_t width = (size_t)n + 1;
    const size_t total = (size_t)count * width;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t c = idx / width;
        const int i = (int)(idx - c * width);
        const int gate = gates ? gates[c] : uniform_gate;
        int32_t k0, sa, sb;
        gate_coeffs(gate, 1 << 29, 1 << 30, &k0, &sa, &sb);
        uint32_t v = (i == n) ? (uint32_t)k0 : 0u;
        v += (uint32_t)sa * (uint32_t)ca[idx];
        v += (uint32_t)sb * (uint32_t)cb[idx];
        out[idx] = (int32_t)v;
    }
}

__global__ void k_lwe_add2_const(const int32_t* __restrict__ u1, const int32_t* __restrict__ u2,
                                 int32_t* __restrict__ out, int width, int32_t mu, int count) {
    const size_t total = (size_t)count * width;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        uint32_t v = (uint32_t)u1[i] + (uint32_t)u2[i];
        if ((int)(i % width) == width - 1) v += (uint32_t)mu;
        out[i] = (int32_t)v;
    }
}

__global__ void k_mul_by_xai_minus_one(const int32_t* __restrict__ in,
                                       const int32_t* __restrict__ ai, int32_t* __restrict__ out,
                                       int polys_per_item, int count) {
    const size_t total = (size_t)count * polys_per_item * kN;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t poly = idx / kN;
        const int x = (int)(idx - poly * kN);
        const int a = ai[poly / polys_per_item];
        const int32_t* p = in + poly * kN;
        out[idx] = (int32_t)((uint32_t)rot_coef(p, x, a) - (uint32_t)p[x]);
    }
}

__global__ void k_extract(const int32_t* __restrict__ acc, int32_t* __restrict__ out, int count) {
    const int c = blockIdx.x;
    if (c >= count) return;
    const int32_t* a = acc + (size_t)c * 2 * kN;
    int32_t* o = out + (size_t)c * (kN + 1);
    for (int i = threadIdx.x; i < kN; i += blockDim.x)
        o[i] = i == 0 ? a[0] : (int32_t)(0u - (uint32_t)a[kN - i]);
    if (threadIdx.x == 0) o[kN] = a[kN];
}

template <typename Kern>
cudaError_t set_smem(Kern k, size_t bytes) {
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

uint32_t decomp_offset(int l, int Bgbit) {
    // constants.h:24 (2164391936 for l = 3, Bgbit = 7)
    uint32_t o = 0;
    for (int i = 0; i < l; ++i) o += 1u << (32 - (i + 1) * Bgbit);
    return o * (uint32_t)(1 << (Bgbit - 1));
}

KParams make_kparams(const DevParams& P) {
    KParams kp;
    kp.n = P.n;
    kp.Bgbit = P.Bgbit;
    kp.split = P.split_bits;
    kp.offset = decomp_offset(P.l, P.Bgbit);
    return kp;
}

// The blind-rotation arguments of items [off, off + cnt) of a batch.
EpArgs slice_blind_rotate(const DevParams& P, const EpArgs& a, int off, int cnt) {
    EpArgs b = a;
    const size_t o = (size_t)off;
    if (a.acc_in) b.acc_in = a.acc_in + o * 2 * kN;
    if (a.acc_out) b.acc_out = a.acc_out + o * 2 * kN;
    if (a.bara) b.bara = a.bara + o * P.n;
    if (a.x) b.x = a.x + o * (P.n + 1);
    if (a.lwe_out) b.lwe_out = a.lwe_out + o * (kN + 1);
    if (a.tv) b.tv = a.tv + o * a.tv_stride;
    b.count = cnt;
    return b;
}

template <typename R, int PARTS, int MODE, int GROUPS, int L>
cudaError_t launch_ep_t(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    const size_t smem = SmemPlan<R, (L > PARTS ? L : PARTS)>::total(GROUPS);
    auto kern = k_external_product<R, PARTS, MODE, GROUPS, L>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    const int grid = (a.count + GROUPS - 1) / GROUPS;
    kern<<<grid, 64 * GROUPS, smem, st>>>(kp, T, a);
    return cudaGetLastError();
}

template <typename R, int PARTS, int GROUPS, int L, bool INLINE, int S = 4, int NB = 1>
cudaError_t launch_ring_t(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    using Plan = RingPlan<R, PARTS, GROUPS, L, S, NB>;
    auto kern = k_blind_rotate_ring<R, PARTS, GROUPS, L, S, INLINE, NB>;
    cudaError_t e = set_smem(kern, Plan::total);
    if (e != cudaSuccess) return e;
    const int grid = (a.count + GROUPS - 1) / GROUPS;
    kern<<<grid, 64 * GROUPS + (INLINE ? 0 : 32), Plan::total, st>>>(kp, T, a);
    return cudaGetLastError();
}

template <typename R, int PARTS, int PAIRS, int L, int S>
cudaError_t launch_pair_t(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    using Plan = PairPlan<R, PARTS, PAIRS, L, S>;
    auto kern = k_blind_rotate_pair<R, PARTS, PAIRS, L, S>;
    cudaError_t e = set_smem(kern, Plan::total);
    if (e != cudaSuccess) return e;
    const int grid = (a.count + PAIRS - 1) / PAIRS;
    kern<<<grid, 128 * PAIRS, Plan::total, st>>>(kp, T, a);
    return cudaGetLastError();
}

template <int L>
cudaError_t launch_spread(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    using Plan = SpreadPlan<L>;
    auto kern = k_blind_rotate_spread<L>;
    cudaError_t e = set_smem(kern, Plan::total);
    if (e != cudaSuccess) return e;
    kern<<<a.count, 128 * L, Plan::total, st>>>(kp, T, a);
    return cudaGetLastError();
}

template <int L>
cudaError_t launch_spread2(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    using Plan = Spread2Plan<L>;
    auto kern = k_blind_rotate_spread2<L>;
    cudaError_t e = set_smem(kern, Plan::request);
    if (e != cudaSuccess) return e;
    kern<<<2 * a.count, 64 * L, Plan::request, st>>>(kp, T, a);
    return cudaGetLastError();
}

// FP64: one ciphertext per cluster of two CTAs
template <int L>
cudaError_t launch_spread2_f64(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    if (a.count <= 0) return cudaSuccess;
    const KParams kp = make_kparams(P);
    using Plan = Spread2F64Plan<L>;
    auto kern = k_blind_rotate_spread2_f64<L>;
    cudaError_t e = set_smem(kern, Plan::request);
    if (e != cudaSuccess) return e;
    kern<<<2 * a.count, 64 * L, Plan::request, st>>>(kp, T, a);
    return cudaGetLastError();
}

// split-FP32 pair kernel with `per_cta` (1..3) ciphertexts per CTA
template <int L>
cudaError_t launch_pair_fp32(const DevParams& P, const Tables& T, const EpArgs& a, int per_cta,
                             cudaStream_t st) {
    // a 4-row ring: deeper rings (6, 8 rows) measured slower, the shared
    // memory they take comes out of the L1 cache
    if (per_cta <= 1) return launch_pair_t<float, 2, 1, L, 4>(P, T, a, st);
    if (per_cta == 2) return launch_pair_t<float, 2, 2, L, 4>(P, T, a, st);
    return launch_pair_t<float, 2, 3, L, 4>(P, T, a, st);
}

// Batched ring kernels: 4 per CTA with a step's l forward transforms run
// together (250 registers, 8 warps per SM), or 6 per CTA with transforms two
// at a time (168 registers, 12 warps per SM).
template <int L>
cudaError_t launch_ring_batched(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    return launch_ring_t<float, 2, 4, L, true, 4, (L > 2 ? L : 2)>(P, T, a, st);
}
template <int L>
cudaError_t launch_ring_pairs(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st) {
    return launch_ring_t<float, 2, 6, L, true, 4, 2>(P, T, a, st);
}

// Automatic shape of a split-FP32 blind rotation over `count` ciphertexts.
// Measured per launch (default set): a wave of 6 per SM on
// launch_ring_pairs 6.6 ms (138K gates/s), of 4 per SM on
// launch_ring_batched 4.6 ms (132K/s), whatever the fill of the wave; the
// spread kernel over a two-SM cluster 1.35 ms for up to one per two SMs;
// the spread kernel 1.85 ms at 1 per SM (3.7 ms for two waves); the pair
// kernel 2.6 ms at 1 per SM, 3.3 ms at 2, 5.1 ms at 3.  So: whole waves of
// 6 per SM; a remainder of at most one per two SMs on the cluster spread
// kernel, of at most 1 per SM on the spread kernel, of 2 per SM on the pair
// kernel, of at most 4 per SM as one launch_ring_batched wave, else one
// more 6-per-SM wave.
//
// fixed_order (shape 15): the pair kernel, which adds its two halves' partial
// products and so may round differently, is replaced by the spread kernel
// (two waves for 2 per SM, 3.8 ms against 3.3 ms): every launch then sums
// the 2l key rows in the same order, and a ciphertext's result does not
// depend on the batch it runs in -- what a server that mixes requests needs.
template <int L>
cudaError_t launch_auto_fp32(const DevParams& P, const Tables& T, const EpArgs& a, cudaStream_t st,
                             bool fixed_order = false) {
    const int wave = 6 * kSmCount;
    const int full = (a.count / wave) * wave;
    const int rest = a.count - full;
    if (rest == 0 || rest > 4 * kSmCount) return launch_ring_pairs<L>(P, T, a, st);
    if (full) {
        cudaError_t e = launch_ring_pairs<L>(P, T, slice_blind_rotate(P, a, 0, full), st);
        if (e != cudaSuccess) return e;
    }
    const EpArgs tail = slice_blind_rotate(P, a, full, rest);
    if (rest > 2 * kSmCount) return launch_ring_batched<L>(P, T, tail, st);
    if (rest > kSmCount && !fixed_order) return launch_pair_fp32<L>(P, T, tail, 2, st);
    if (rest > kSmCount / 2) return launch_spread<L>(P, T, tail, st);
    return launch_spread2<L>(P, T, tail, st);
}

// FP64: ~250 registers per thread and 2 x L exchange buffers of 9 KB per
// group, so 3 groups (192 threads) per CTA.  split-FP32: GROUPS groups.
template <int L>
cudaError_t launch_ep_l(const DevParams& P, Form f, EpMode mode, const Tables& T, const EpArgs& a,
                        int groups, cudaStream_t st) {
    if (f == kFormFp64) {
        switch (mode) {
        case kEpPlain: return launch_ep_t<double, 1, kEpPlain, 3, L>(P, T, a, st);
        case kEpMuxRotate: return launch_ep_t<double, 1, kEpMuxRotate, 3, L>(P, T, a, st);
        default:
            // 0: automatic -- up to one ciphertext per SM on the cluster
            // kernel (one or two waves: 21.6 ms each, against about 57 ms for
            // a wave of the 3-per-CTA kernel), larger batches 3 per CTA with
            // L2-direct key reads; 3: L2-direct; 4: shared key ring; 16:
            // cluster kernel
            if (groups == 16 || (groups == 0 && a.count <= kSmCount))
                return launch_spread2_f64<L>(P, T, a, st);
            if (groups == 3 || groups == 0) return launch_ep_t<double, 1, kEpBlindRotate, 3, L>(P, T, a, st);
            return launch_ring_t<double, 1, 4, L, true>(P, T, a, st);
        }
    }
    switch (mode) {
    case kEpPlain: return launch_ep_t<float, 2, kEpPlain, 4, L>(P, T, a, st);
    case kEpMuxRotate: return launch_ep_t<float, 2, kEpMuxRotate, 4, L>(P, T, a, st);
    default:
        if (groups == 0) return launch_auto_fp32<L>(P, T, a, st);
        if (groups == 15) return launch_auto_fp32<L>(P, T, a, st, true);
        if (groups == 16) return launch_spread2<L>(P, T, a, st);
        // 1, 2, 4: L2-direct key reads; 5: shared ring fed by a producer
        // warp; 6, 7, 8: shared ring fed in line by one consumer thread;
        // 9: shared ring, 4 per CTA, a step's l forward transforms run
        // together; 10: shared ring, 6 per CTA, transforms two at a time;
        // 11, 12, 13: pair kernel with 1, 2, 3 ciphertexts per CTA;
        // 15: the automatic shape in fixed summation order (no pair kernel);
        // 16: spread over a cluster of two CTAs
        if (groups >= 11 && groups <= 13) return launch_pair_fp32<L>(P, T, a, groups - 10, st);
        if (groups == 9) return launch_ring_batched<L>(P, T, a, st);
        if (groups == 10) return launch_ring_pairs<L>(P, T, a, st);
        if (groups == 14) return launch_spread<L>(P, T, a, st);
        if (groups == 1) return launch_ep_t<float, 2, kEpBlindRotate, 1, L>(P, T, a, st);
        if (groups == 2) return launch_ep_t<float, 2, kEpBlindRotate, 2, L>(P, T, a, st);
        if (groups == 4) return launch_ep_t<float, 2, kEpBlindRotate, 4, L>(P, T, a, st);
        if (groups == 5) return launch_ring_t<float, 2, 5, L, false>(P, T, a, st);
        if (groups == 7) return launch_ring_t<float, 2, 7, L, true>(P, T, a, st);
        if (groups == 8) return launch_ring_t<float, 2, 8, L, true>(P, T, a, st);
        return launch_ring_t<float, 2, 6, L, true>(P, T, a, st);
    }
}

}  // namespace

// ----------------------------------------------------------------------
// host-side tables and launchers
// ----------------------------------------------------------------------
static void sincos_2pi_frac(long k, long M, double* c, double* s) {
    k %= M;
    const long q = (4 * k) / M;
    const long r = k - q * (M / 4);
    double cr, sr;
    if (8 * r <= M) {
        const double a = 2.0 * M_PI * (double)r / (double)M;
        cr = cos(a);
        sr = sin(a);
    } else {
        const double a = 2.0 * M_PI * (double)(M / 4 - r) / (double)M;
        cr = sin(a);
        sr = cos(a);
    }
    switch (q) {
    case 0: *c = cr; *s = sr; break;
    case 1: *c = -sr; *s = cr; break;
    case 2: *c = -cr; *s = -sr; break;
    default: *c = sr; *s = -cr; break;
    }
}

void make_twiddles_host(double* h) {
    // layout of Tables: [q][t] W^(tq) | [q][j] W^(8jq) | [q][t] psi^t W^(tq) | psi^x,
    // W = e^{2 pi i/512}, psi = e^{pi i/1024}
    for (int q = 0; q < 8; ++q)
        for (int t = 0; t < 64; ++t)
            sincos_2pi_frac(t * q, 512, &h[2 * (kTabA + q * 64 + t)], &h[2 * (kTabA + q * 64 + t) + 1]);
    for (int q = 0; q < 8; ++q)
        for (int j = 0; j < 8; ++j)
            sincos_2pi_frac(8 * j * q, 512, &h[2 * (kTabB + q * 8 + j)], &h[2 * (kTabB + q * 8 + j) + 1]);
    // psi^t W^(tq) = e^{2 pi i (t + 4 t q) / 2048}
    for (int q = 0; q < 8; ++q)
        for (int t = 0; t < 64; ++t)
            sincos_2pi_frac(t + 4 * t * q, 2048, &h[2 * (kTabT + q * 64 + t)], &h[2 * (kTabT + q * 64 + t) + 1]);
    for (int x = 0; x < 512; ++x)
        sincos_2pi_frac(x, 2048, &h[2 * (kTabPsi + x)], &h[2 * (kTabPsi + x) + 1]);
}

int twiddle_table_entries() { return kTabSize; }

size_t tgsw_fft_bytes(const DevParams& P, Form f) {
    const size_t rows = (size_t)(P.k + 1) * P.l;
    if (f == kFormFp64) return rows * 2 * kHalf * sizeof(cpx<double>);
    return rows * 2 * 2 * kHalf * sizeof(cpx<float>);
}

cudaError_t launch_tgsw_to_fft(const DevParams& P, Form f, const Tables& T, const int32_t* tgsw,
                               void* out, int count, cudaStream_t st) {
    const int npoly = count * (P.k + 1) * P.l * (P.k + 1);
    if (npoly <= 0) return cudaSuccess;
    const int groups = 4;
    const size_t smem = kConvTableBytes + groups * kConvGroupBytes;
    const int grid = (npoly + groups - 1) / groups;
    cudaError_t e;
    if (f == kFormFp64) {
        e = set_smem(k_tgsw_to_fft<kFormFp64>, smem);
        if (e != cudaSuccess) return e;
        k_tgsw_to_fft<kFormFp64><<<grid, 64 * groups, smem, st>>>(T, tgsw, out, npoly, 0);
    } else {
        e = set_smem(k_tgsw_to_fft<kFormSplitFp32>, smem);
        if (e != cudaSuccess) return e;
        k_tgsw_to_fft<kFormSplitFp32><<<grid, 64 * groups, smem, st>>>(T, tgsw, out, npoly,
                                                                       P.split_bits);
    }
    return cudaGetLastError();
}

cudaError_t launch_tgsw_from_fft64(const DevParams& P, const Tables& T, const void* in,
                                   int32_t* tgsw, int count, cudaStream_t st) {
    const int npoly = count * (P.k + 1) * P.l * (P.k + 1);
    if (npoly <= 0) return cudaSuccess;
    const int groups = 4;
    const size_t smem = kConvTableBytes + groups * kConvGroupBytes;
    cudaError_t e = set_smem(k_fft64_to_tgsw, smem);
    if (e != cudaSuccess) return e;
    k_fft64_to_tgsw<<<(npoly + groups - 1) / groups, 64 * groups, smem, st>>>(T, in, tgsw, npoly);
    return cudaGetLastError();
}

cudaError_t launch_lagrange_ref_to_engine64(const double* ref, void* eng, int npoly, double scale,
                                            cudaStream_t st) {
    const int total = npoly * kHalf;
    if (total <= 0) return cudaSuccess;
    k_ref_to_engine64<<<(total + 255) / 256, 256, 0, st>>>(ref, reinterpret_cast<cpx<double>*>(eng),
                                                          npoly, scale);
    return cudaGetLastError();
}

cudaError_t launch_engine64_to_lagrange_ref(const void* eng, double* ref, int npoly, double scale,
                                            cudaStream_t st) {
    const int total = npoly * kHalf;
    if (total <= 0) return cudaSuccess;
    k_engine64_to_ref<<<(total + 255) / 256, 256, 0, st>>>(
        reinterpret_cast<const cpx<double>*>(eng), ref, npoly, scale);
    return cudaGetLastError();
}

int blind_rotate_tail_start(Form f, int groups, int count) {
    // launch_auto_fp32's split: whole 6-per-SM waves, then a remainder of
    // at most 4 per SM that runs as its own launch on part of the SMs
    if (f != kFormSplitFp32 || (groups != 0 && groups != 15)) return 0;
    const int wave = 6 * kSmCount;
    const int full = (count / wave) * wave;
    const int rest = count - full;
    return full > 0 && rest > 0 && rest <= 4 * kSmCount ? full : 0;
}

cudaError_t launch_external_product(const DevParams& P, Form f, EpMode mode, const Tables& T,
                                    const EpArgs& a, int groups, cudaStream_t st) {
    switch (P.l) {
    case 2: return launch_ep_l<2>(P, f, mode, T, a, groups, st);
    case 3: return launch_ep_l<3>(P, f, mode, T, a, groups, st);
    default: return cudaErrorInvalidValue;  // decomposition lengths 2 and 3 are built
    }
}

cudaError_t launch_gate_combine(const DevParams& P, const int32_t* gates, int32_t uniform_gate,
                                const int32_t* ca, const int32_t* cb, int32_t* out, int count,
                                cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const size_t total = (size_t)count * (P.n + 1);
    const int blocks = (int)((total + 255) / 256 < 8192 ? (total + 255) / 256 : 8192);
    k_gate_combine<<<blocks, 256, 0, st>>>(P.n, gates, uniform_gate, ca, cb, out, count);
    return cudaGetLastError();
}

cudaError_t launch_lwe_add2_const(const int32_t* u1, const int32_t* u2, int32_t* out,
                                  int32_t width, int32_t mu, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const size_t total = (size_t)count * width;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_lwe_add2_const<<<blocks, 256, 0, st>>>(u1, u2, out, width, mu, count);
    return cudaGetLastError();
}

cudaError_t launch_mul_by_xai_minus_one(const DevParams& P, const int32_t* in, const int32_t* ai,
                                        int32_t* out, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const size_t total = (size_t)count * (P.k + 1) * kN;
    const int blocks = (int)((total + 255) / 256 < 8192 ? (total + 255) / 256 : 8192);
    k_mul_by_xai_minus_one<<<blocks, 256, 0, st>>>(in, ai, out, P.k + 1, count);
    return cudaGetLastError();
}

cudaError_t launch_extract(const DevParams& P, const int32_t* acc, int32_t* out, int count,
                           cudaStream_t st) {
    (void)P;
    if (count <= 0) return cudaSuccess;
    k_extract<<<count, 256, 0, st>>>(acc, out, count);
    return cudaGetLastError();
}

cudaError_t launch_poly_to_lagrange(const DevParams& P, const Tables& T, const int32_t* in,
                                    double* out, int count, double scale, cudaStream_t st) {
    (void)P;
    if (count <= 0) return cudaSuccess;
    const int groups = 4;
    const size_t smem = kConvTableBytes + groups * kConvGroupBytes;
    cudaError_t e = set_smem(k_poly_to_lagrange, smem);
    if (e != cudaSuccess) return e;
    k_poly_to_lagrange<<<(count + groups - 1) / groups, 64 * groups, smem, st>>>(T, in, out, count,
                                                                                 scale);
    return cudaGetLastError();
}

cudaError_t launch_lagrange_to_torus(const DevParams& P, const Tables& T, const double* in,
                                     int32_t* out, int count, cudaStream_t st) {
    (void)P;
    if (count <= 0) return cudaSuccess;
    const int groups = 4;
    const size_t smem = kConvTableBytes + groups * kConvGroupBytes;
    cudaError_t e = set_smem(k_lagrange_to_torus, smem);
    if (e != cudaSuccess) return e;
    k_lagrange_to_torus<<<(count + groups - 1) / groups, 64 * groups, smem, st>>>(T, in, out,
                                                                                  count);
    return cudaGetLastError();
}

cudaError_t launch_lagrange_addmul(const double* a, const double* b, double* acc, int npoly,
                                   int half, cudaStream_t st) {
    const size_t total = (size_t)npoly * half;
    if (total == 0) return cudaSuccess;
    k_lagrange_addmul<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a, b, acc, total);
    return cudaGetLastError();
}

}  // namespace tfhe_gb300
