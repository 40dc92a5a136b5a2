// fft512.cuh -- negacyclic transform for N = 1024 as a 512-point complex FFT.
//
// A real polynomial a(X) mod X^1024 + 1 is folded into z_j = a_j + i a_{j+512}
// (j < 512) and twisted by psi^j, psi = e^{i pi / 1024}.  The 512-point DFT
// with kernel W = e^{+2 pi i / 512} then gives Z_m = a(psi^(4m+1)): the
// evaluations of a at half of the odd 2048-th roots of unity; the other half
// are their conjugates.  The reference computes the same evaluations with a
// 2048-point transform of the antiperiodic extension
// (tfhe_blindRotate_FFT/tGswFFTExternMulToTLwe.cpp:97-130, "ifft") and with a
// Hermitian placement on the way back (TorusPolynomial_fft.cpp:4-43); this
// form does a quarter of that work.
//
// Work split: 64 threads (two warps) per transform, 8 points per thread,
// three radix-8 passes in registers with two exchanges through shared memory.
//   forward (decimation in frequency):
//     pass A  thread t: points t + 64r            -> out positions t + 64q
//     pass B  thread t=(b,j): 64b + j + 8r          -> 64b + j + 8q
//     pass C  thread t: 8t + r                      -> 8t + q (registers)
//   position 64qA + 8qB + qC holds frequency qA + 8qB + 64qC.  The pointwise
//   product works in that order; the key is stored in it, so no reordering.
//   inverse (decimation in time) runs the passes backwards, input from
//   registers (positions 8t + q) to natural order (positions t + 64q).
// Shared scratch: two ping-pong buffers of interleaved complex values, padded
// p + p/8 so the strided exchanges are (almost) free of bank conflicts; the
// twiddles are stored per pass in the order the threads read them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tfhe_gb300 {

template <typename R>
struct __align__(2 * sizeof(R)) cpx {
    R x, y;
};

template <typename R>
__device__ __forceinline__ cpx<R> cadd(cpx<R> a, cpx<R> b) {
    return {a.x + b.x, a.y + b.y};
}
template <typename R>
__device__ __forceinline__ cpx<R> csub(cpx<R> a, cpx<R> b) {
    return {a.x - b.x, a.y - b.y};
}
template <typename R>
__device__ __forceinline__ cpx<R> cmul(cpx<R> a, cpx<R> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename R>
__device__ __forceinline__ cpx<R> cmulc(cpx<R> a, cpx<R> b) {
    return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
// acc + a * w
template <typename R>
__device__ __forceinline__ cpx<R> cmac(cpx<R> acc, cpx<R> a, cpx<R> w) {
    return cadd(acc, cmul(a, w));
}

// ---- FP32: packed pair arithmetic ---------------------------------------
// A complex float is one 64-bit register pair and add/mul/fma.f32x2 (sm_100
// and later) work on both halves in one instruction, so complex adds take
// one instruction and complex products two.  Measured on GB300 (instruction
// counts of isolated loops): a whole-pair negation, a broadcast {x, x} of
// one half and the swap-and-negate {-y, x} of i * a cost nothing extra as
// multiplicands; an FMA by a literal +-1 becomes an add, and an add whose
// addend is swapped costs about one more instruction, so i-multiplied
// addends inside the radix-8 butterfly stay scalar.
__device__ __forceinline__ float2 pk(cpx<float> a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ cpx<float> unpk(float2 a) { return {a.x, a.y}; }
__device__ __forceinline__ float2 bc(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 times_i(cpx<float> a) { return make_float2(-a.y, a.x); }
__device__ __forceinline__ float2 times_minus_i(cpx<float> a) { return make_float2(a.y, -a.x); }

__device__ __forceinline__ cpx<float> cadd(cpx<float> a, cpx<float> b) {
    return unpk(__fadd2_rn(pk(a), pk(b)));
}
__device__ __forceinline__ cpx<float> csub(cpx<float> a, cpx<float> b) {
    return unpk(__fadd2_rn(pk(a), make_float2(-b.x, -b.y)));
}
// a w = w.x a + w.y (i a)
__device__ __forceinline__ cpx<float> cmul(cpx<float> a, cpx<float> w) {
    return unpk(__ffma2_rn(times_i(a), bc(w.y), __fmul2_rn(pk(a), bc(w.x))));
}
// a conj(w) = w.x a + w.y (-i a)
__device__ __forceinline__ cpx<float> cmulc(cpx<float> a, cpx<float> w) {
    return unpk(__ffma2_rn(times_minus_i(a), bc(w.y), __fmul2_rn(pk(a), bc(w.x))));
}
__device__ __forceinline__ cpx<float> cmac(cpx<float> acc, cpx<float> a, cpx<float> w) {
    return unpk(__ffma2_rn(times_i(a), bc(w.y), __ffma2_rn(pk(a), bc(w.x), pk(acc))));
}

constexpr int kFftPoints = 512;
constexpr int kFftThreads = 64;
constexpr int kScratchStride = 576;  // 512 + 512/8 padding

__device__ __forceinline__ int spad(int p) { return p + (p >> 3); }

// Shared-memory slot of point p in an exchange buffer, chosen so that every
// access pattern of the three passes (A: p = t + 64q, B: p = 64(t/8) +
// t%8 + 8r, C: p = 8t + r over the lanes t of a warp) is free of bank
// conflicts.  FP32 (8-byte points, half-warp wavefronts): an XOR of the low
// four bits with a function of p/16 -- padding would leave pass A with a
// two-way conflict.  FP64 (16-byte points, quarter-warp wavefronts): one pad
// slot every 8 points.
template <typename R>
__device__ __forceinline__ int slot(int p);
template <>
__device__ __forceinline__ int slot<float>(int p) {
    const int k = p >> 4;
    return p ^ ((k & 7) | ((k & 4) << 1));
}
template <>
__device__ __forceinline__ int slot<double>(int p) { return spad(p); }

// FP32 8-point DFT on packed pairs: the same butterflies as dft8 below, the
// multiplications by w and w^3 as two packed instructions each, the
// i-multiplied terms (w^2 and the last stage's e3) as scalar adds.
template <int S>
__device__ __forceinline__ void dft8_f32(cpx<float> (&v)[8]) {
    constexpr float h = 0.70710678118654752440f;
    cpx<float> b[8];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        b[r] = cadd(v[r], v[r + 4]);
        b[r + 4] = csub(v[r], v[r + 4]);
    }
    // b5 *= (1 + S i) h = h b5 + S h (i b5);  b7 *= (-1 + S i) h
    b[5] = unpk(__ffma2_rn(times_i(b[5]), bc(S * h), __fmul2_rn(pk(b[5]), bc(h))));
    b[7] = unpk(__ffma2_rn(times_i(b[7]), bc(S * h), __fmul2_rn(make_float2(-b[7].x, -b[7].y), bc(h))));
    {  // c = b0, b1, b2, b3
        const cpx<float> e0 = cadd(b[0], b[2]), e1 = csub(b[0], b[2]);
        const cpx<float> e2 = cadd(b[1], b[3]), d = csub(b[1], b[3]);
        v[0] = cadd(e0, e2);
        v[4] = csub(e0, e2);
        v[2] = {e1.x - S * d.y, e1.y + S * d.x};  // e1 + S i d
        v[6] = {e1.x + S * d.y, e1.y - S * d.x};
    }
    {  // c = b4, b5, S i b6, b7
        const cpx<float> e0 = {b[4].x - S * b[6].y, b[4].y + S * b[6].x};
        const cpx<float> e1 = {b[4].x + S * b[6].y, b[4].y - S * b[6].x};
        const cpx<float> e2 = cadd(b[5], b[7]), d = csub(b[5], b[7]);
        v[1] = cadd(e0, e2);
        v[5] = csub(e0, e2);
        v[3] = {e1.x - S * d.y, e1.y + S * d.x};
        v[7] = {e1.x + S * d.y, e1.y - S * d.x};
    }
}

// 8-point DFT, y_q = sum_r v_r w^{rq}, w = e^{S 2 pi i / 8}.
template <int S, typename R>
__device__ __forceinline__ void dft8(cpx<R> (&v)[8]) {
    if constexpr (sizeof(R) == 4) {
        dft8_f32<S>(v);
    } else {
        const R h = (R)0.70710678118654752440084436210485;
        cpx<R> b[8];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            b[r] = cadd(v[r], v[r + 4]);
            b[r + 4] = csub(v[r], v[r + 4]);
        }
        {  // b5 *= w = (1 + S i) h
            const R x = b[5].x, y = b[5].y;
            b[5] = {(x - S * y) * h, (y + S * x) * h};
        }
        {  // b6 *= w^2 = S i
            const R x = b[6].x, y = b[6].y;
            b[6] = {-S * y, S * x};
        }
        {  // b7 *= w^3 = (-1 + S i) h
            const R x = b[7].x, y = b[7].y;
            b[7] = {(-x - S * y) * h, (S * x - y) * h};
        }
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const cpx<R> c0 = b[4 * half + 0], c1 = b[4 * half + 1];
            const cpx<R> c2 = b[4 * half + 2], c3 = b[4 * half + 3];
            const cpx<R> e0 = cadd(c0, c2), e1 = csub(c0, c2), e2 = cadd(c1, c3);
            const cpx<R> d = csub(c1, c3);
            const cpx<R> e3 = {-S * d.y, S * d.x};
            v[half + 0] = cadd(e0, e2);
            v[half + 2] = cadd(e1, e3);
            v[half + 4] = csub(e0, e2);
            v[half + 6] = csub(e1, e3);
        }
    }
}

__device__ __forceinline__ void group_sync(int bar_id) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(kFftThreads) : "memory");
}

// Two ping-pong exchange buffers of kScratchStride interleaved complex values.
template <typename R>
struct FftScratch {
    cpx<R>* b0;
    cpx<R>* b1;
};

// Twiddles laid out so that a warp reads consecutive (or identical) words:
//   a[q * 64 + t] = W^(t q)      pass A / A'   (W = e^{+2 pi i / 512})
//   b[q * 8 + j]  = W^(8 j q)    pass B / B'
template <typename R>
struct FftTwiddles {
    const cpx<R>* a;
    const cpx<R>* b;
};

// Forward transform.  In: v[r] = z[t + 64r].  Out: v[q] = position 8t + q.
template <typename R>
__device__ __forceinline__ void fft512_forward(cpx<R> (&v)[8], const FftScratch<R>& s,
                                               const FftTwiddles<R>& tw, int t, int bar_id) {
    // pass A
    dft8<1>(v);
#pragma unroll
    for (int q = 1; q < 8; ++q) v[q] = cmul(v[q], tw.a[q * 64 + t]);
#pragma unroll
    for (int q = 0; q < 8; ++q) s.b0[slot<R>(t + 64 * q)] = v[q];
    group_sync(bar_id);
    // pass B
    const int b = t >> 3, j = t & 7;
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = s.b0[slot<R>(64 * b + j + 8 * r)];
    dft8<1>(v);
#pragma unroll
    for (int q = 1; q < 8; ++q) v[q] = cmul(v[q], tw.b[q * 8 + j]);
#pragma unroll
    for (int q = 0; q < 8; ++q) s.b1[slot<R>(64 * b + j + 8 * q)] = v[q];
    group_sync(bar_id);
    // pass C
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = s.b1[slot<R>(8 * t + r)];
    dft8<1>(v);
}

// Inverse transform (unnormalised: returns 512 z).  In: v[q] = position
// 8t + q.  Out: v[q] = z[t + 64q].
template <typename R>
__device__ __forceinline__ void fft512_inverse(cpx<R> (&v)[8], const FftScratch<R>& s,
                                               const FftTwiddles<R>& tw, int t, int bar_id) {
    // pass C'
    dft8<-1>(v);
#pragma unroll
    for (int q = 0; q < 8; ++q) s.b0[slot<R>(8 * t + q)] = v[q];
    group_sync(bar_id);
    // pass B'
    const int b = t >> 3, j = t & 7;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        v[r] = s.b0[slot<R>(64 * b + j + 8 * r)];
        if (r) v[r] = cmulc(v[r], tw.b[r * 8 + j]);
    }
    dft8<-1>(v);
#pragma unroll
    for (int q = 0; q < 8; ++q) s.b1[slot<R>(64 * b + j + 8 * q)] = v[q];
    group_sync(bar_id);
    // pass A'
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        v[r] = s.b1[slot<R>(t + 64 * r)];
        if (r) v[r] = cmulc(v[r], tw.a[r * 64 + t]);
    }
    dft8<-1>(v);
}

// Per-thread exchange slots of the FP32 swizzle, in closed form for each
// access pattern (computed once per thread; an access is then an immediate
// offset or one XOR):
//   A: slot(t + 64q)          = 64q + (q odd ? a1 : a0)
//   B: slot(64(t/8) + t%8 + 8r) = b_base + 16(r/2) + (b_x ^ (8(r%2) | r/2))
//   C: slot(8t + r)           = c_base + (r ^ c_z)
// FP64 keeps the padded layout (slot<double>), computed per access.
struct FftIdx {
    int a0, a1, b_base, b_x, c_base, c_z;
};

__device__ __forceinline__ FftIdx make_fft_idx(int t) {
    const int b = t >> 3, j = t & 7;
    const int gC = ((t >> 1) & 7) | (((t >> 1) & 4) << 1);
    FftIdx x;
    x.a0 = t ^ (t >> 4);
    x.a1 = t ^ ((t >> 4) | 12);
    x.b_base = 64 * b;
    x.b_x = j ^ (12 * (b & 1));
    x.c_base = (8 * t) ^ (gC & 8);
    x.c_z = gC & 7;
    return x;
}

template <typename R>
__device__ __forceinline__ int slot_a(const FftIdx& x, int t, int q) {
    if constexpr (sizeof(R) == 4) return 64 * q + ((q & 1) ? x.a1 : x.a0);
    else return slot<R>(t + 64 * q);
}
template <typename R>
__device__ __forceinline__ int slot_b(const FftIdx& x, int t, int r) {
    if constexpr (sizeof(R) == 4) return x.b_base + 16 * (r >> 1) + (x.b_x ^ ((8 * (r & 1)) | (r >> 1)));
    else return slot<R>(64 * (t >> 3) + (t & 7) + 8 * r);
}
template <typename R>
__device__ __forceinline__ int slot_c(const FftIdx& x, int t, int r) {
    if constexpr (sizeof(R) == 4) return x.c_base + (r ^ x.c_z);
    else return slot<R>(8 * t + r);
}

// ----------------------------------------------------------------------
// Transforms with the negacyclic twist folded in.  Point x = t + 64r of a
// thread is twisted by psi^x = psi^t c_r, c_r = psi^(64 r) = e^{i pi r/16}:
// the compile-time c_r multiply the inputs, and psi^t, common to the
// thread's radix-8 block, joins pass A's twiddles in the table
// tw.a[q * 64 + t] = psi^t W^(t q) (q = 0..7).  The inverse mirrors it:
// conj(psi^t W^(t r)) on pass A''s inputs, conj(c_q) on its outputs.  Same
// number of roundings as a separate twist, and no psi^x loads.
// ----------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ cpx<R> twist_c(int r) {
    // e^{i pi r / 16}, r = 0..7
    constexpr double kC[8][2] = {{1.0, 0.0},
                                 {0.9807852804032304, 0.19509032201612825},
                                 {0.9238795325112867, 0.3826834323650898},
                                 {0.8314696123025452, 0.5555702330196022},
                                 {0.7071067811865476, 0.7071067811865475},
                                 {0.5555702330196023, 0.8314696123025452},
                                 {0.38268343236508984, 0.9238795325112867},
                                 {0.19509032201612833, 0.9807852804032304}};
    return {(R)kC[r][0], (R)kC[r][1]};
}

// In: v[r] = untwisted folded point t + 64r.  Out: v[q] = position 8t + q
// of the transform of the twisted sequence.  tw.a = psi^t W^(tq) table.
// With NB > 1 every twiddle is loaded once and applied to all NB point sets
// (the compiler cannot merge the loads across the exchange stores).
template <int NB, typename R>
__device__ __forceinline__ void fft512_forward_tw_multi(cpx<R> (&v)[NB][8], const FftScratch<R> (&s)[NB],
                                                        const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                        int bar_id) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 1; r < 8; ++r) v[b][r] = cmul(v[b][r], twist_c<R>(r));
        dft8<1>(v[b]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const cpx<R> w = tw.a[q * 64 + t];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][q] = cmul(v[b][q], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) s[b].b0[slot_a<R>(ix, t, q)] = v[b][q];
    group_sync(bar_id);
    const int j = t & 7;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 0; r < 8; ++r) v[b][r] = s[b].b0[slot_b<R>(ix, t, r)];
        dft8<1>(v[b]);
    }
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        const cpx<R> w = tw.b[q * 8 + j];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][q] = cmul(v[b][q], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) s[b].b1[slot_b<R>(ix, t, q)] = v[b][q];
    group_sync(bar_id);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 0; r < 8; ++r) v[b][r] = s[b].b1[slot_c<R>(ix, t, r)];
        dft8<1>(v[b]);
    }
}

// In: v[q] = position 8t + q.  Out: v[q] = 512 z[t + 64q] untwisted (times
// psi^-(t + 64q)), not yet divided by 512.
template <int NB, typename R>
__device__ __forceinline__ void fft512_inverse_tw_multi(cpx<R> (&v)[NB][8], const FftScratch<R> (&s)[NB],
                                                        const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                        int bar_id) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 0; q < 8; ++q) s[b].b0[slot_c<R>(ix, t, q)] = v[b][q];
    }
    group_sync(bar_id);
    const int j = t & 7;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        if (r == 0) {
#pragma unroll
            for (int b = 0; b < NB; ++b) v[b][0] = s[b].b0[slot_b<R>(ix, t, 0)];
        } else {
            const cpx<R> w = tw.b[r * 8 + j];
#pragma unroll
            for (int b = 0; b < NB; ++b) v[b][r] = cmulc(s[b].b0[slot_b<R>(ix, t, r)], w);
        }
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 0; q < 8; ++q) s[b].b1[slot_b<R>(ix, t, q)] = v[b][q];
    }
    group_sync(bar_id);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const cpx<R> w = tw.a[r * 64 + t];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][r] = cmulc(s[b].b1[slot_a<R>(ix, t, r)], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 1; q < 8; ++q) v[b][q] = cmulc(v[b][q], twist_c<R>(q));
    }
}

template <typename R>
__device__ __forceinline__ void fft512_forward_tw(cpx<R> (&v)[8], const FftScratch<R>& s,
                                                  const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                  int bar_id) {
    fft512_forward_tw_multi<1>(*reinterpret_cast<cpx<R>(*)[1][8]>(&v),
                               *reinterpret_cast<const FftScratch<R>(*)[1]>(&s), tw, ix, t, bar_id);
}

template <typename R>
__device__ __forceinline__ void fft512_inverse_tw(cpx<R> (&v)[8], const FftScratch<R>& s,
                                                  const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                  int bar_id) {
    fft512_inverse_tw_multi<1>(*reinterpret_cast<cpx<R>(*)[1][8]>(&v),
                               *reinterpret_cast<const FftScratch<R>(*)[1]>(&s), tw, ix, t, bar_id);
}

// ----------------------------------------------------------------------
// In-place forms: one exchange buffer per transform.  Pass B reads and
// writes the same positions of a thread, and the exchange between passes B
// and C stays within groups of 8 consecutive lanes (position 8t + r is
// written by lane 8(t/8) + r), so it needs only __syncwarp; the exchange
// between passes A and B crosses the two warps and keeps the group barrier.
// A caller that runs two transforms on one buffer with no group barrier
// between them would race (the second's pass A writes against the first's
// pass C reads in the other warp): it alternates two buffers instead.  The
// arithmetic is that of fft512_forward_tw_multi / fft512_inverse_tw_multi,
// bit for bit.
// ----------------------------------------------------------------------
template <int NB, typename R>
__device__ __forceinline__ void fft512_forward_ip(cpx<R> (&v)[NB][8], cpx<R>* const (&x)[NB],
                                                  const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                  int bar_id) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 1; r < 8; ++r) v[b][r] = cmul(v[b][r], twist_c<R>(r));
        dft8<1>(v[b]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const cpx<R> w = tw.a[q * 64 + t];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][q] = cmul(v[b][q], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) x[b][slot_a<R>(ix, t, q)] = v[b][q];
    group_sync(bar_id);
    const int j = t & 7;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 0; r < 8; ++r) v[b][r] = x[b][slot_b<R>(ix, t, r)];
        dft8<1>(v[b]);
    }
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        const cpx<R> w = tw.b[q * 8 + j];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][q] = cmul(v[b][q], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) x[b][slot_b<R>(ix, t, q)] = v[b][q];
    __syncwarp();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int r = 0; r < 8; ++r) v[b][r] = x[b][slot_c<R>(ix, t, r)];
        dft8<1>(v[b]);
    }
}

template <int NB, typename R>
__device__ __forceinline__ void fft512_inverse_ip(cpx<R> (&v)[NB][8], cpx<R>* const (&x)[NB],
                                                  const FftTwiddles<R>& tw, const FftIdx& ix, int t,
                                                  int bar_id) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 0; q < 8; ++q) x[b][slot_c<R>(ix, t, q)] = v[b][q];
    }
    __syncwarp();
    const int j = t & 7;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        if (r == 0) {
#pragma unroll
            for (int b = 0; b < NB; ++b) v[b][0] = x[b][slot_b<R>(ix, t, 0)];
        } else {
            const cpx<R> w = tw.b[r * 8 + j];
#pragma unroll
            for (int b = 0; b < NB; ++b) v[b][r] = cmulc(x[b][slot_b<R>(ix, t, r)], w);
        }
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 0; q < 8; ++q) x[b][slot_b<R>(ix, t, q)] = v[b][q];
    }
    group_sync(bar_id);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const cpx<R> w = tw.a[r * 64 + t];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b][r] = cmulc(x[b][slot_a<R>(ix, t, r)], w);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        dft8<-1>(v[b]);
#pragma unroll
        for (int q = 1; q < 8; ++q) v[b][q] = cmulc(v[b][q], twist_c<R>(q));
    }
}

template <typename R>
__device__ __forceinline__ void fft512_forward_ip1(cpx<R> (&v)[8], cpx<R>* x, const FftTwiddles<R>& tw,
                                                   const FftIdx& ix, int t, int bar_id) {
    cpx<R>* const xs[1] = {x};
    fft512_forward_ip<1>(*reinterpret_cast<cpx<R>(*)[1][8]>(&v), xs, tw, ix, t, bar_id);
}

template <typename R>
__device__ __forceinline__ void fft512_inverse_ip1(cpx<R> (&v)[8], cpx<R>* x, const FftTwiddles<R>& tw,
                                                   const FftIdx& ix, int t, int bar_id) {
    cpx<R>* const xs[1] = {x};
    fft512_inverse_ip<1>(*reinterpret_cast<cpx<R>(*)[1][8]>(&v), xs, tw, ix, t, bar_id);
}

// Frequency held at (thread t, register q) after the forward transform.
__host__ __device__ __forceinline__ int freq_of(int t, int q) {
    return (t >> 3) + 8 * (t & 7) + 64 * q;
}

// Storage index of (thread t, register q) in one 512-point key polynomial.
// FP32: pairs of complex per 16-byte load, [q/2][t][q%2]; FP64: [q][t].
template <typename R>
__host__ __device__ __forceinline__ int key_index(int t, int q);
template <>
__host__ __device__ __forceinline__ int key_index<float>(int t, int q) {
    return ((q >> 1) * 64 + t) * 2 + (q & 1);
}
template <>
__host__ __device__ __forceinline__ int key_index<double>(int t, int q) {
    return q * 64 + t;
}

}  // namespace tfhe_gb300
