// engine.h -- internal launch interface of the GB300 TFHE engine.
// The public C ABI is include/tfhe_gpu.h; capi.cpp implements it on top of
// these launchers.  Everything here is device-resident: pointers are device
// pointers, sizes are element counts, launches go to the given stream.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tfhe_gb300 {

// Streaming multiprocessors of a GB300 (two dies of 76): launch shapes are
// sized in waves of this many CTAs.
constexpr int kSmCount = 152;

// Precision forms of the transform.
enum Form {
    kFormFp64 = 0,       // FP64 transform and product, truncating conversion
    kFormSplitFp32 = 1,  // FP32 transform; key split K = Khi 2^s + Klo
    kNumForms = 2
};

struct DevParams {
    int32_t n, N, k, l, Bgbit, ks_t, ks_basebit;
    int32_t split_bits;  // s of the split-FP32 form
};

// Bytes of one TGSW sample (kpl rows x 2 polys) in the engine FFT layout.
size_t tgsw_fft_bytes(const DevParams& P, Form f);

// Transform tables, twiddle_table_entries() complex values: the radix-8
// passes' twiddles W^(tq) and W^(8jq) (W = e^{2 pi i/512}) in the order the
// threads read them, then psi^x = e^{i pi x/1024}.  `host64` receives
// 2 * twiddle_table_entries() doubles (re, im interleaved).
int twiddle_table_entries();
void make_twiddles_host(double* host64);

struct Tables {
    const void* tw64;  // twiddle_table_entries() double2
    const void* tw32;  // twiddle_table_entries() float2
};

// TGSW (time domain, count x kpl x 2 x N int32) -> engine FFT layout.
cudaError_t launch_tgsw_to_fft(const DevParams& P, Form f, const Tables& T,
                               const int32_t* tgsw, void* out, int count,
                               cudaStream_t st);
// Engine FFT layout -> time domain (FP64 form only; rounds to nearest).
cudaError_t launch_tgsw_from_fft64(const DevParams& P, const Tables& T,
                                   const void* in, int32_t* tgsw, int count,
                                   cudaStream_t st);
// Reference Lagrange layout (values at w^(2m+1), torus/2^32 scale, per
// polynomial N/2 complex doubles) <-> engine FFT64 layout of integer-scaled
// values.  Used to import a TGswSampleFFT in the reference's format.
cudaError_t launch_lagrange_ref_to_engine64(const double* ref, void* eng,
                                            int npoly, double scale,
                                            cudaStream_t st);
cudaError_t launch_engine64_to_lagrange_ref(const void* eng, double* ref,
                                            int npoly, double scale,
                                            cudaStream_t st);

// Modes of the external-product kernel.
enum EpMode { kEpPlain = 0, kEpMuxRotate = 1, kEpBlindRotate = 2 };

struct EpArgs {
    // kEpPlain / kEpMuxRotate: in/out TLWE (count x 2N), gsw per item
    // (gsw_stride bytes apart; 0 = shared), a per item (MuxRotate).
    // kEpBlindRotate: acc from `acc_in` + `bara` (count x n) or from the LWE
    // samples `x` (count x (n+1)) and `mu`; results to `acc_out` and/or the
    // extracted samples `lwe_out` (count x (N+1)).
    const int32_t* acc_in;
    int32_t* acc_out;
    const int32_t* bara;
    const int32_t* x;
    int32_t mu;
    int32_t* lwe_out;
    const void* gsw;
    size_t gsw_stride;
    int count;
    int32_t* err;  // device status word: set to 3 (timeout) by a bounded wait
    // kEpBlindRotate from x: test vector polynomial (N int32, item c at
    // tv + c * tv_stride) instead of the constant mu; nullptr = constant mu
    const int32_t* tv;
    int32_t tv_stride;
    // self-test of the bounded waits: the key-row ring's producer issues
    // nothing, so every consumer wait runs out (tfhe_gpu_selftest_timeout)
    int32_t stall_keys;
};

cudaError_t launch_external_product(const DevParams& P, Form f, EpMode mode,
                                    const Tables& T, const EpArgs& a,
                                    int groups_per_cta, cudaStream_t st);

// Gate linear combination: out = c + sa * ca + sb * cb (per item gate).
cudaError_t launch_gate_combine(const DevParams& P, const int32_t* gates,
                                int32_t uniform_gate, const int32_t* ca,
                                const int32_t* cb, int32_t* out, int count,
                                cudaStream_t st);
// u1 + u2 + (0, mu) on extracted samples (bootsMUX middle step).
cudaError_t launch_lwe_add2_const(const int32_t* u1, const int32_t* u2,
                                  int32_t* out, int32_t width, int32_t mu,
                                  int count, cudaStream_t st);
cudaError_t launch_mul_by_xai_minus_one(const DevParams& P, const int32_t* in,
                                        const int32_t* ai, int32_t* out,
                                        int count, cudaStream_t st);
cudaError_t launch_extract(const DevParams& P, const int32_t* acc,
                           int32_t* out, int count, cudaStream_t st);

// Lagrange processor: count polynomials.
cudaError_t launch_poly_to_lagrange(const DevParams& P, const Tables& T,
                                    const int32_t* in, double* out, int count,
                                    double scale, cudaStream_t st);
cudaError_t launch_lagrange_to_torus(const DevParams& P, const Tables& T,
                                     const double* in, int32_t* out, int count,
                                     cudaStream_t st);
cudaError_t launch_lagrange_addmul(const double* a, const double* b,
                                   double* acc, int npoly, int half,
                                   cudaStream_t st);

// Where the automatic split-FP32 blind rotation of `count` ciphertexts
// starts its remainder launch (one that leaves SMs idle), or 0 when it is a
// single launch or another shape is set.
int blind_rotate_tail_start(Form f, int groups, int count);

// Key switching: in (count x (kN+1)) -> out (count x (n+1)); ks rows are
// `row_stride` int32 apart, layout [kN][t][base][row_stride].
cudaError_t launch_keyswitch(const DevParams& P, const int32_t* ks,
                             int32_t row_stride, const int32_t* in,
                             int32_t* out, int count, cudaStream_t st);

// Finish n TGSW encryptions whose rows hold masks a and noise b = e (host
// RNG, exact order): b += sum_i a_i * s_i (negacyclic, TLWE key s, N k
// int32) and the gadget term lwe_key[row / kpl] * 2^(32 - (j+1) Bgbit) on
// coefficient 0 of polynomial i of row (i, j).  bk: device, n x kpl x
// (k+1) x N int32, in place.
cudaError_t launch_tgsw_finish(const DevParams& P, int32_t* bk, const int32_t* tlwe_key,
                               const int32_t* lwe_key, cudaStream_t st);

}  // namespace tfhe_gb300

// Host key generation (keygen.cpp).  With bk_products false the rows of the
// bootstrapping key are left with their masks and noise only, for
// launch_tgsw_finish; the RNG stream is the same either way.
#include "../../include/tfhe_gpu.h"
namespace tfhe_gb300 {
tfhe_gpu_status gate_keyset_host(const tfhe_params* P, int32_t* lwe_key, int32_t* tlwe_key,
                                 int32_t* ks, int32_t* bk, bool bk_products);
}  // namespace tfhe_gb300
