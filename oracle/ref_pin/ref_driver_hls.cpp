// ref_driver_hls.cpp -- flat-array entry points over the reference's own
// hot-path kernels (kernel/src/tfhe_blindRotate_FFT/*.cpp with the SPIRAL
// Pease FFT, tfhe_bootstrap_woKS_FFT.cpp, mulByXaiOrCopy.cpp), compiled
// unmodified on the CPU against the stand-in HLS headers in shim_hls/.
// Test infrastructure: the oracle pin tests call these.
#include <string.h>

#include <vector>

#include "fpga_constants.h"

// C++-linkage helpers defined in tGswFFTExternMulToTLwe.cpp
void decompose(IntPolynomial_FPGA* result, TorusPolynomial_FPGA* sample);
void ifft(LagrangeHalfCPolynomial_FPGA& result, const IntPolynomial_FPGA& source);
extern "C" void tfhe_blindRotate_FFT(TLweSample_FPGA* accum_FPGA, Torus32_FPGA* in_bara,
                                     TGswSampleFFT_FPGA* in_bkFFT, TLweSample_FPGA* output);
extern "C" void tfhe_bootstrap_woKS_FFT(hls::stream<Torus32_FPGA>& in_mu,
                                        hls::stream<Torus32_FPGA, n>& in_x_a,
                                        hls::stream<Torus32_FPGA>& in_x_b,
                                        hls::stream<Torus32_FPGA, N>& out_testvect,
                                        hls::stream<Torus32_FPGA, n>& out_bara,
                                        hls::stream<Torus32_FPGA>& out_barb);
extern "C" void mulByXaiOrCopy(hls::stream<Torus32_FPGA, N>& in_v, hls::stream<Torus32_FPGA>& in_barb,
                               hls::stream<Torus32_FPGA, N>& out_testvect);

namespace {
void load_tlwe(TLweSample_FPGA* s, const int32_t* flat) {
    memset(s, 0, sizeof(*s));
    for (int i = 0; i <= k; ++i) memcpy(s->a[i].coefsT, flat + i * N, sizeof(int32_t) * N);
    memcpy(s->b.coefsT, flat + k * N, sizeof(int32_t) * N);
}
void store_tlwe(int32_t* flat, const TLweSample_FPGA* s) {
    for (int i = 0; i <= k; ++i) memcpy(flat + i * N, s->a[i].coefsT, sizeof(int32_t) * N);
}
// flat TGSW in the reference Lagrange convention: [kpl][k+1][N/2][2]
void load_tgsw_fft(TGswSampleFFT_FPGA* g, const double* flat) {
    memset(g, 0, sizeof(*g));
    for (int p = 0; p < param_kpl; ++p)
        for (int j = 0; j <= k; ++j)
            for (int m = 0; m < N / 2; ++m) {
                const double* v = flat + (((size_t)p * (k + 1) + j) * (N / 2) + m) * 2;
                g->all_samples[p].a[j].coefsC[m] = cplx(v[0], v[1]);
            }
}
}  // namespace

extern "C" {

int32_t refh_params(int32_t* out) {
    out[0] = n; out[1] = N; out[2] = k; out[3] = bk_l; out[4] = bk_Bgbit;
    out[5] = ks_length; out[6] = ks_basebit;
    return 7;
}

void refh_decompose(const int32_t* in, int32_t* out) {
    TorusPolynomial_FPGA s;
    memcpy(s.coefsT, in, sizeof(int32_t) * N);
    IntPolynomial_FPGA r[bk_l];
    decompose(r, &s);
    for (int p = 0; p < bk_l; ++p) memcpy(out + p * N, r[p].coefs, sizeof(int32_t) * N);
}

void refh_decomp_h(const int32_t* in, int32_t* out) {
    TorusPolynomial_FPGA s;
    memcpy(s.coefsT, in, sizeof(int32_t) * N);
    IntPolynomial_FPGA r[bk_l];
    tGswTorus32PolynomialDecompH(s, r);
    for (int p = 0; p < bk_l; ++p) memcpy(out + p * N, r[p].coefs, sizeof(int32_t) * N);
}

void refh_int_ifft(const int32_t* in, double* out) {
    IntPolynomial_FPGA s;
    memcpy(s.coefs, in, sizeof(int32_t) * N);
    LagrangeHalfCPolynomial_FPGA r;
    ifft(r, s);
    for (int m = 0; m < N / 2; ++m) {
        out[2 * m] = r.coefsC[m].real();
        out[2 * m + 1] = r.coefsC[m].imag();
    }
}

void refh_torus_fft(const double* in, int32_t* out) {
    LagrangeHalfCPolynomial_FPGA p;
    for (int m = 0; m < N / 2; ++m) p.coefsC[m] = cplx(in[2 * m], in[2 * m + 1]);
    TorusPolynomial_FPGA r;
    TorusPolynomial_fft(p, &r);
    memcpy(out, r.coefsT, sizeof(int32_t) * N);
}

// accum (k+1) x N in/out; gsw: one TGSW in the reference Lagrange layout
void refh_extern_mul(int32_t* accum, const double* gsw) {
    TLweSample_FPGA* acc = new TLweSample_FPGA;
    TGswSampleFFT_FPGA* g = new TGswSampleFFT_FPGA;
    load_tlwe(acc, accum);
    load_tgsw_fft(g, gsw);
    tGswFFTExternMulToTLwe_FPGA(acc, g);
    store_tlwe(accum, acc);
    delete g;
    delete acc;
}

void refh_mux_rotate(int32_t* result, const int32_t* accum, const double* bki, int32_t barai) {
    TLweSample_FPGA* res = new TLweSample_FPGA;
    TLweSample_FPGA* acc = new TLweSample_FPGA;
    TGswSampleFFT_FPGA* g = new TGswSampleFFT_FPGA;
    load_tlwe(acc, accum);
    memset(res, 0, sizeof(*res));
    load_tgsw_fft(g, bki);
    tfhe_MuxRotate_FFT_FPGA(res, acc, g, barai);
    store_tlwe(result, res);
    delete g;
    delete acc;
    delete res;
}

// The blind rotation the reference intends: tfhe_MuxRotate_FFT_FPGA over all
// `steps` entries of bara, skipping zeros (tfhe_blindRotate_FFT.cpp:112-128
// with the loop bound restored).  bk: steps TGSW in the Lagrange layout.
void refh_blind_rotate(int32_t* accum, const double* bk, const int32_t* bara, int32_t steps) {
    TLweSample_FPGA* a = new TLweSample_FPGA;
    TLweSample_FPGA* b = new TLweSample_FPGA;
    TGswSampleFFT_FPGA* g = new TGswSampleFFT_FPGA;
    load_tlwe(a, accum);
    memset(b, 0, sizeof(*b));
    const size_t tgsw = (size_t)param_kpl * (k + 1) * N;
    for (int32_t i = 0; i < steps; ++i) {
        if (bara[i] == 0) continue;
        load_tgsw_fft(g, bk + i * tgsw);
        tfhe_MuxRotate_FFT_FPGA(b, a, g, bara[i]);
        TLweSample_FPGA* s = a;
        a = b;
        b = s;
    }
    store_tlwe(accum, a);
    delete g;
    delete a;
    delete b;
}

// The kernel as shipped (its loop runs i < 1); bk holds bk[0] only, which is
// all the shipped loop reads.
void refh_blind_rotate_shipped(int32_t* accum, const double* bk0, const int32_t* bara) {
    TLweSample_FPGA* acc = new TLweSample_FPGA;
    TLweSample_FPGA* out = new TLweSample_FPGA;
    TGswSampleFFT_FPGA* g = new TGswSampleFFT_FPGA;
    std::vector<int32_t> ba(bara, bara + n);
    load_tlwe(acc, accum);
    memset(out, 0, sizeof(*out));
    load_tgsw_fft(g, bk0);
    tfhe_blindRotate_FFT(acc, ba.data(), g, out);
    store_tlwe(accum, out);
    delete g;
    delete out;
    delete acc;
}

// tfhe_bootstrap_woKS_FFT (modulus switch + test vector) and mulByXaiOrCopy
void refh_bootstrap_front(const int32_t* x, int32_t mu, int32_t* testvect, int32_t* bara,
                          int32_t* barb, int32_t* rotated) {
    hls::stream<Torus32_FPGA> in_mu, in_x_b, out_barb, in_barb2;
    hls::stream<Torus32_FPGA, n> in_x_a, out_bara;
    hls::stream<Torus32_FPGA, N> out_tv, in_v, out_rot;
    in_mu << mu;
    for (int i = 0; i < n; ++i) in_x_a << x[i];
    in_x_b << x[n];
    tfhe_bootstrap_woKS_FFT(in_mu, in_x_a, in_x_b, out_tv, out_bara, out_barb);
    for (int i = 0; i < N; ++i) testvect[i] = out_tv.read();
    for (int i = 0; i < n; ++i) bara[i] = out_bara.read();
    *barb = out_barb.read();
    for (int i = 0; i < N; ++i) in_v << testvect[i];
    in_barb2 << *barb;
    mulByXaiOrCopy(in_v, in_barb2, out_rot);
    for (int i = 0; i < N; ++i) rotated[i] = out_rot.read();
}

}  // extern "C"
