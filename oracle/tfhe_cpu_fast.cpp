/*
 * tfhe_cpu_fast.cpp -- a faster CPU gate bootstrap, for timing only.
 *
 * BASELINE INFRASTRUCTURE ONLY.  Only tests/ and the cpu_baseline leg of
 * bench.py load this library; the engine never links or calls it, and it
 * is not the oracle (oracle/tfhe_oracle.cpp is).
 *
 * The oracle restates the reference's own method: a 2N-point transform of
 * the antiperiodic extension for every polynomial product
 * (tfhe_blindRotate_FFT/tGswFFTExternMulToTLwe.cpp:97-130,
 * TorusPolynomial_fft.cpp:4-43).  The upstream TFHE library that the
 * reference links (test_bench/Makefile:6) evaluates the same products with
 * an N/2-point complex transform instead, about a quarter of the work.  This
 * file is a CPU implementation in that style, so that the CPU figure beside
 * the GPU engine is not only the slow method:
 *   - fold a(X) mod X^N + 1 into z_j = a_j + i a_{j+N/2}, twist by psi^j
 *     (psi = e^{i pi/N}), N/2-point DFT: Z_m = a(psi^(4m+1));
 *   - radix-2 decimation in frequency forward (natural in, bit-reversed
 *     out) and decimation in time inverse (bit-reversed in, natural out),
 *     so the pointwise products need no permutation; split real and
 *     imaginary arrays so that the loops vectorise;
 *   - double precision; the products are integer-valued, and the conversion
 *     back truncates toward zero like TorusPolynomial_fft.cpp:40.
 * The gate sequence, decomposition, rotation, extraction and key switch are
 * the same integer steps as the oracle (cited there).  Results decrypt like
 * the oracle's; phases differ by FFT rounding only (tests/test_cpu_fast.py).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tfhe_oracle.h"

namespace {

constexpr int kMaxLog = 12;

struct Transform {
    int M = 0;                      // complex points (N/2)
    int logM = 0;
    std::vector<double> tw_re, tw_im;  // per DIF stage s (half = M >> (s+1)): W^(k M/len), k < half
    std::vector<int> tw_off;           // offset of stage s in tw_*
    std::vector<double> psi_re, psi_im;  // psi^j, j < M

    void init(int N) {
        M = N / 2;
        logM = 0;
        while ((1 << logM) < M) ++logM;
        tw_off.assign(logM + 1, 0);
        tw_re.clear();
        tw_im.clear();
        for (int s = 0; s < logM; ++s) {
            const int len = M >> s, half = len / 2;
            tw_off[s] = (int)tw_re.size();
            for (int k = 0; k < half; ++k) {
                const double a = 2.0 * M_PI * (double)k / (double)len;
                tw_re.push_back(std::cos(a));
                tw_im.push_back(std::sin(a));
            }
        }
        psi_re.resize(M);
        psi_im.resize(M);
        for (int j = 0; j < M; ++j) {
            const double a = M_PI * (double)j / (double)N;
            psi_re[j] = std::cos(a);
            psi_im[j] = std::sin(a);
        }
    }

    // In: re/im = folded coefficients (natural order).  Out: the twisted
    // transform in bit-reversed order.  Kernel W = e^{+2 pi i / M}.
    void forward(double* __restrict__ re, double* __restrict__ im) const {
        for (int j = 0; j < M; ++j) {
            const double x = re[j], y = im[j];
            re[j] = x * psi_re[j] - y * psi_im[j];
            im[j] = x * psi_im[j] + y * psi_re[j];
        }
        for (int s = 0; s < logM; ++s) {
            const int len = M >> s, half = len / 2;
            const double* __restrict__ wr = tw_re.data() + tw_off[s];
            const double* __restrict__ wi = tw_im.data() + tw_off[s];
            for (int b = 0; b < M; b += len) {
                double* __restrict__ ur = re + b;
                double* __restrict__ ui = im + b;
                double* __restrict__ vr = re + b + half;
                double* __restrict__ vi = im + b + half;
                for (int k = 0; k < half; ++k) {
                    const double dr = ur[k] - vr[k], di = ui[k] - vi[k];
                    ur[k] += vr[k];
                    ui[k] += vi[k];
                    vr[k] = dr * wr[k] - di * wi[k];
                    vi[k] = dr * wi[k] + di * wr[k];
                }
            }
        }
    }

    // In: bit-reversed spectrum.  Out: M times the untwisted folded
    // coefficients (natural order), still to be divided by M.
    void inverse(double* __restrict__ re, double* __restrict__ im) const {
        for (int s = logM - 1; s >= 0; --s) {
            const int len = M >> s, half = len / 2;
            const double* __restrict__ wr = tw_re.data() + tw_off[s];
            const double* __restrict__ wi = tw_im.data() + tw_off[s];
            for (int b = 0; b < M; b += len) {
                double* __restrict__ ur = re + b;
                double* __restrict__ ui = im + b;
                double* __restrict__ vr = re + b + half;
                double* __restrict__ vi = im + b + half;
                for (int k = 0; k < half; ++k) {
                    // v * conj(w)
                    const double tr = vr[k] * wr[k] + vi[k] * wi[k];
                    const double ti = vi[k] * wr[k] - vr[k] * wi[k];
                    vr[k] = ur[k] - tr;
                    vi[k] = ui[k] - ti;
                    ur[k] += tr;
                    ui[k] += ti;
                }
            }
        }
        for (int j = 0; j < M; ++j) {
            const double x = re[j], y = im[j];
            re[j] = x * psi_re[j] + y * psi_im[j];
            im[j] = y * psi_re[j] - x * psi_im[j];
        }
    }
};

inline int32_t mod_switch_from_torus32(int32_t phase, int32_t Msize) {
    const uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    const uint64_t phase64 = ((uint64_t)(int64_t)phase << 32) + interv / 2;
    return (int32_t)(phase64 / interv);
}

inline int32_t mod_switch_to_torus32(int32_t mu, int32_t Msize) {
    const uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    return (int32_t)(uint32_t)(((uint64_t)(int64_t)mu * interv) >> 32);
}

}  // namespace

struct cpuf_ctx {
    orc_params P;
    Transform tf;
    std::vector<double> bk_re, bk_im;  // [n][kpl][k+1][N/2]
    const int32_t* ks;                 // caller's key-switching key, kept alive by the caller
};

namespace {

// Scratch of one thread.
struct Work {
    std::vector<int32_t> acc, x, u;
    std::vector<uint32_t> t;
    std::vector<double> dre, dim, ore, oim;
    std::vector<int32_t> bara;
    void init(const orc_params& P) {
        const int N = P.N, M = N / 2, kpl = (P.k + 1) * P.l;
        acc.assign((size_t)(P.k + 1) * N, 0);
        x.assign(P.n + 1, 0);
        u.assign((size_t)P.k * N + 1, 0);
        t.assign(N, 0);
        dre.assign((size_t)kpl * M, 0.0);
        dim.assign((size_t)kpl * M, 0.0);
        ore.assign((size_t)(P.k + 1) * M, 0.0);
        oim.assign((size_t)(P.k + 1) * M, 0.0);
        bara.assign(P.n, 0);
    }
};

// acc <- acc + BK_i [(X^a - 1) acc]  (one MuxRotate step)
void mux_rotate(const cpuf_ctx* c, Work& w, int i, int32_t a) {
    const orc_params& P = c->P;
    const int N = P.N, M = N / 2, k = P.k, l = P.l, kpl = (k + 1) * l;
    const int Bgbit = P.Bgbit, halfBg = 1 << (Bgbit - 1);
    const uint32_t mask = (1u << Bgbit) - 1;
    uint32_t offset = 0;
    for (int p = 0; p < l; ++p) offset += 1u << (32 - (p + 1) * Bgbit);
    offset *= (uint32_t)halfBg;
    for (int q = 0; q <= k; ++q) {
        const uint32_t* in = reinterpret_cast<const uint32_t*>(w.acc.data()) + (size_t)q * N;
        uint32_t* t = w.t.data();
        // (X^a - 1) in, negacyclic, a in [0, 2N)  (tfhe_MuxRotate_FFT.cpp:5-24)
        if (a < N) {
            for (int j = 0; j < a; ++j) t[j] = 0u - in[j - a + N] - in[j];
            for (int j = a; j < N; ++j) t[j] = in[j - a] - in[j];
        } else {
            const int aa = a - N;
            for (int j = 0; j < aa; ++j) t[j] = in[j - aa + N] - in[j];
            for (int j = aa; j < N; ++j) t[j] = 0u - in[j - aa] - in[j];
        }
        for (int j = 0; j < N; ++j) t[j] += offset;
        for (int p = 0; p < l; ++p) {
            const int decal = 32 - (p + 1) * Bgbit;
            double* re = w.dre.data() + (size_t)(q * l + p) * M;
            double* im = w.dim.data() + (size_t)(q * l + p) * M;
            for (int j = 0; j < M; ++j) {
                re[j] = (double)((int32_t)((t[j] >> decal) & mask) - halfBg);
                im[j] = (double)((int32_t)((t[j + M] >> decal) & mask) - halfBg);
            }
            c->tf.forward(re, im);
        }
    }
    std::fill(w.ore.begin(), w.ore.end(), 0.0);
    std::fill(w.oim.begin(), w.oim.end(), 0.0);
    const size_t step = (size_t)kpl * (k + 1) * M;
    for (int p = 0; p < kpl; ++p) {
        const double* __restrict__ dr = w.dre.data() + (size_t)p * M;
        const double* __restrict__ di = w.dim.data() + (size_t)p * M;
        for (int j = 0; j <= k; ++j) {
            const size_t off = (size_t)i * step + ((size_t)p * (k + 1) + j) * M;
            const double* __restrict__ kr = c->bk_re.data() + off;
            const double* __restrict__ ki = c->bk_im.data() + off;
            double* __restrict__ orr = w.ore.data() + (size_t)j * M;
            double* __restrict__ oi = w.oim.data() + (size_t)j * M;
            for (int m = 0; m < M; ++m) {
                orr[m] += dr[m] * kr[m] - di[m] * ki[m];
                oi[m] += dr[m] * ki[m] + di[m] * kr[m];
            }
        }
    }
    const double inv = 1.0 / (double)M;
    for (int j = 0; j <= k; ++j) {
        double* re = w.ore.data() + (size_t)j * M;
        double* im = w.oim.data() + (size_t)j * M;
        c->tf.inverse(re, im);
        uint32_t* dst = reinterpret_cast<uint32_t*>(w.acc.data()) + (size_t)j * N;
        for (int m = 0; m < M; ++m) {
            dst[m] += (uint32_t)(uint64_t)(int64_t)(re[m] * inv);
            dst[m + M] += (uint32_t)(uint64_t)(int64_t)(im[m] * inv);
        }
    }
}

void boots_gate(const cpuf_ctx* c, Work& w, int32_t gate, const int32_t* ca, const int32_t* cb,
                int32_t* out) {
    const orc_params& P = c->P;
    const int n = P.n, N = P.N, k = P.k, Nx2 = 2 * N;
    const int32_t e8 = mod_switch_to_torus32(1, 8), e4 = mod_switch_to_torus32(1, 4);
    // gate constants: the same table as orc_gate_combine
    int32_t cst = 0, sa = 0, sb = 0;
    switch (gate) {
    case ORC_GATE_NAND: cst = e8;  sa = -1; sb = -1; break;
    case ORC_GATE_AND:  cst = -e8; sa = 1;  sb = 1;  break;
    case ORC_GATE_OR:   cst = e8;  sa = 1;  sb = 1;  break;
    case ORC_GATE_XOR:  cst = e4;  sa = 2;  sb = 2;  break;
    case ORC_GATE_XNOR: cst = -e4; sa = -2; sb = -2; break;
    case ORC_GATE_NOR:  cst = -e8; sa = -1; sb = -1; break;
    case ORC_GATE_ANDNY: cst = -e8; sa = -1; sb = 1; break;
    case ORC_GATE_ANDYN: cst = -e8; sa = 1;  sb = -1; break;
    case ORC_GATE_ORNY: cst = e8;  sa = -1; sb = 1;  break;
    case ORC_GATE_ORYN: cst = e8;  sa = 1;  sb = -1; break;
    default: break;
    }
    for (int i = 0; i <= n; ++i)
        w.x[i] = (int32_t)((i == n ? (uint32_t)cst : 0u) + (uint32_t)sa * (uint32_t)ca[i] +
                           (uint32_t)sb * (uint32_t)cb[i]);
    // prologue: modulus switch, acc = (0, X^(2N - barb) mu)
    const int32_t barb = mod_switch_from_torus32(w.x[n], Nx2);
    for (int i = 0; i < n; ++i) w.bara[i] = mod_switch_from_torus32(w.x[i], Nx2);
    std::fill(w.acc.begin(), w.acc.end(), 0);
    int32_t* b = w.acc.data() + (size_t)k * N;
    const int32_t rot = barb == 0 ? 0 : Nx2 - barb;
    for (int j = 0; j < N; ++j) {
        // X^rot * sum_j e8 X^j, negacyclic
        const int src = j - rot;
        const int s = ((src % Nx2) + Nx2) % Nx2;
        b[j] = s < N ? e8 : (int32_t)(0u - (uint32_t)e8);
    }
    for (int i = 0; i < n; ++i)
        if (w.bara[i] != 0) mux_rotate(c, w, i, w.bara[i]);
    // extraction (coefficient 0)
    for (int q = 0; q < k; ++q) {
        const int32_t* a = w.acc.data() + (size_t)q * N;
        w.u[(size_t)q * N] = a[0];
        for (int j = 1; j < N; ++j) w.u[(size_t)q * N + j] = (int32_t)(0u - (uint32_t)a[N - j]);
    }
    w.u[(size_t)k * N] = w.acc[(size_t)k * N];
    // key switch
    const int n_in = k * N, t = P.ks_t, basebit = P.ks_basebit, base = 1 << basebit;
    const uint32_t prec_offset = 1u << (32 - (1 + basebit * t));
    const uint32_t kmask = (uint32_t)base - 1;
    uint32_t* o = reinterpret_cast<uint32_t*>(out);
    for (int q = 0; q < n; ++q) o[q] = 0;
    o[n] = (uint32_t)w.u[n_in];
    for (int i = 0; i < n_in; ++i) {
        const uint32_t aibar = (uint32_t)w.u[i] + prec_offset;
        for (int j = 0; j < t; ++j) {
            const uint32_t d = (aibar >> (32 - (j + 1) * basebit)) & kmask;
            if (d == 0) continue;
            const uint32_t* row =
                reinterpret_cast<const uint32_t*>(c->ks) + ((size_t)(i * t + j) * base + d) * (n + 1);
            for (int q = 0; q <= n; ++q) o[q] -= row[q];
        }
    }
}

}  // namespace

extern "C" {

// bk: the bootstrapping key in the time domain (n x kpl x (k+1) x N int32);
// ks: the key-switching key (kN x t x base x (n+1) int32), not copied.
cpuf_ctx* cpuf_create(const orc_params* P, const int32_t* bk, const int32_t* ks) {
    if (!P || !bk || !ks || P->N < 4 || P->N > (1 << kMaxLog) || (P->N & (P->N - 1))) return nullptr;
    cpuf_ctx* c = new cpuf_ctx;
    c->P = *P;
    c->ks = ks;
    c->tf.init(P->N);
    const int N = P->N, M = N / 2, kpl = (P->k + 1) * P->l;
    const size_t polys = (size_t)P->n * kpl * (P->k + 1);
    c->bk_re.resize(polys * M);
    c->bk_im.resize(polys * M);
    for (size_t p = 0; p < polys; ++p) {
        const int32_t* src = bk + p * N;
        double* re = c->bk_re.data() + p * M;
        double* im = c->bk_im.data() + p * M;
        for (int j = 0; j < M; ++j) {
            re[j] = (double)src[j];
            im[j] = (double)src[j + M];
        }
        c->tf.forward(re, im);
    }
    return c;
}

void cpuf_destroy(cpuf_ctx* c) { delete c; }

void cpuf_boots_gates(const cpuf_ctx* c, const int32_t* gates, const int32_t* ca, const int32_t* cb,
                      int32_t* out, int32_t count, int32_t threads) {
    const size_t wd = (size_t)c->P.n + 1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        Work w;
        w.init(c->P);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int32_t g = 0; g < count; ++g)
            boots_gate(c, w, gates[g], ca + g * wd, cb + g * wd, out + g * wd);
    }
    (void)threads;
}

}  // extern "C"
