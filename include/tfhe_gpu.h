/*
 * tfhe_gpu.h -- C ABI of the GB300 TFHE gate-bootstrapping engine.
 *
 * The engine is the GPU replacement of the TFHE bootstrapping path of
 * shreks99/fpga-tfhe.  Every entry point below names the reference function
 * it replaces (paths inside that project).  Conventions:
 *   - plain pointers and sizes, no C++ types;
 *   - "device batch" entry points take DEVICE pointers (cudaMalloc'd or from
 *     any allocator) to `count` items laid out back to back and a CUDA stream
 *     (cudaStream_t passed as void*, NULL = the context's stream); they
 *     enqueue work and return without synchronising;
 *   - "_host" entry points take HOST buffers, copy in, compute, copy out and
 *     synchronise (the end-to-end form a drop-in caller uses);
 *   - every call returns a status; nothing exits the process (the reference
 *     host exits on OpenCL errors, kernel/src/include/host.h:13-18);
 *   - a context owns its device memory (keys, tables, scratch); one context
 *     per host thread, or serialise calls externally.
 *
 * Data layouts (int32 = Torus32, arithmetic mod 2^32):
 *   LWE sample        int32[n + 1]             a[0..n-1], b
 *   extracted sample  int32[k N + 1]
 *   TLWE sample       int32[(k + 1) N]          a[0..k-1], then b
 *   TGSW sample       int32[(k+1) l][(k+1)][N]  row p = i l + j
 *   bootstrapping key n TGSW samples of the bits of the LWE key
 *   key-switching key int32[k N][t][2^basebit][n + 1]
 *   Lagrange polynomial double[N/2][2]: values at w^(2m+1), w = e^{i pi/N}
 *                      (the reference's LagrangeHalfCPolynomial_FPGA,
 *                      kernel/src/include/polynomials.h:15-17)
 */
#ifndef TFHE_GPU_H
#define TFHE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tfhe_gpu_status {
    TFHE_GPU_OK = 0,
    TFHE_GPU_BAD_PARAM = 1,    /* invalid argument or unsupported parameter set */
    TFHE_GPU_OOM = 2,          /* device or pinned host allocation failed       */
    TFHE_GPU_TIMEOUT = 3,      /* a bounded device wait gave up                 */
    TFHE_GPU_DEVICE_ERROR = 4, /* CUDA reported an error (see last_error)       */
    TFHE_GPU_NO_KEY = 5        /* the key needed by the call was not uploaded   */
} tfhe_gpu_status;

/* Precision form of the negacyclic transform. */
typedef enum tfhe_gpu_form {
    TFHE_GPU_FP64 = 0,       /* FP64 transform, reference truncating rounding  */
    TFHE_GPU_SPLIT_FP32 = 1  /* FP32 transform; key split K = Khi 2^s + Klo    */
} tfhe_gpu_form;

#define TFHE_GPU_FORM_MASK(f) (1u << (f))

/* Gate identifiers of the batched gate entry points. */
typedef enum tfhe_gpu_gate {
    TFHE_GATE_NAND = 0, TFHE_GATE_AND = 1, TFHE_GATE_OR = 2, TFHE_GATE_XOR = 3,
    TFHE_GATE_XNOR = 4, TFHE_GATE_NOR = 5, TFHE_GATE_ANDNY = 6,
    TFHE_GATE_ANDYN = 7, TFHE_GATE_ORNY = 8, TFHE_GATE_ORYN = 9
} tfhe_gpu_gate;

/* Parameter set (kernel/src/include/constants.h:26-53). */
typedef struct tfhe_params {
    int32_t n;          /* LWE dimension (630)                     */
    int32_t N;          /* ring degree (1024; the only one built)  */
    int32_t k;          /* TLWE mask polynomials (1)               */
    int32_t l;          /* decomposition length (3)                */
    int32_t Bgbit;      /* log2 decomposition base (7)             */
    int32_t ks_t;       /* key-switch length (8)                   */
    int32_t ks_basebit; /* log2 key-switch base (2)                */
    int32_t split_bits; /* s of the split-FP32 key split; 0 = auto */
    double lwe_alpha;   /* LWE / key-switch noise stdev            */
    double tlwe_alpha;  /* TLWE / bootstrapping key noise stdev    */
} tfhe_params;

typedef struct tfhe_gpu_ctx tfhe_gpu_ctx;

/* ---- context ---------------------------------------------------------- */

/* The 110-bit default gate set of the reference (constants.h:26-40). */
void tfhe_gpu_default_params(tfhe_params* out);
/* Create a context on `device`; uploads the transform tables. */
tfhe_gpu_status tfhe_gpu_create(const tfhe_params* params, int32_t device,
                                tfhe_gpu_ctx** out);
void tfhe_gpu_destroy(tfhe_gpu_ctx* ctx);
const char* tfhe_gpu_status_string(tfhe_gpu_status s);
/* Human-readable detail of the last failure on this context. */
const char* tfhe_gpu_last_error(const tfhe_gpu_ctx* ctx);
/* The parameters in use (split_bits resolved). */
tfhe_gpu_status tfhe_gpu_get_params(const tfhe_gpu_ctx* ctx, tfhe_params* out);
/* The context's own stream (as void*). */
void* tfhe_gpu_stream(const tfhe_gpu_ctx* ctx);
/* Wait for all work of the context's stream; TFHE_GPU_TIMEOUT if a kernel's
 * bounded wait gave up since the last check. */
tfhe_gpu_status tfhe_gpu_synchronize(tfhe_gpu_ctx* ctx);
/* Bytes of one TGSW sample in the engine's transform layout. */
size_t tfhe_gpu_tgsw_fft_bytes(const tfhe_gpu_ctx* ctx, tfhe_gpu_form form);
/* Device bytes the context holds (keys, tables, scratch). */
size_t tfhe_gpu_device_bytes(const tfhe_gpu_ctx* ctx);

/* Launch shape of the blind-rotation kernel of `form`.  split-FP32:
 *   0 = automatic: whole waves of 6 ciphertexts per SM on shape 10; a
 *       remainder of at most one per two SMs on shape 16, of at most 1 per
 *       SM on shape 14, of 2 per SM on the pair kernel, of at most 4 per SM
 *       as one shape-9 wave, else one more shape-10 wave;
 *   1, 2, 4 = ciphertexts (64 threads each) per CTA, key rows read from L2
 *       by every ciphertext;
 *   5 = 5 per CTA, key rows streamed once per CTA into a shared-memory ring
 *       by a producer warp;
 *   6, 7, 8 = that many per CTA, the same ring fed by one consumer thread;
 *   9 = 4 per CTA on the same ring, each step's l forward and 2 inverse
 *       transforms run together (about 250 registers a thread);
 *   10 = 6 per CTA on the same ring, transforms two at a time;
 *   11, 12, 13 = pair kernel: two 64-thread halves per ciphertext (about
 *       half the latency), 1, 2, 3 ciphertexts per CTA, shared ring;
 *   14 = spread kernel: one ciphertext over 2l groups of 64 threads; per
 *       step each group runs one forward transform, and four of them
 *       multiply all rows for one output part and transform it back (lowest
 *       latency), key rows from L2;
 *   15 = automatic in fixed summation order: as 0, with the spread kernel
 *       (two waves) in place of the pair kernel, whose two halves' partial
 *       products round differently; every launch then sums the key rows in
 *       the same order, and a ciphertext's result is the same bit for bit
 *       whatever batch it runs in (the gate server uses it);
 *   16 = the spread kernel over a cluster of two CTAs on two SMs: each CTA
 *       holds one accumulator polynomial, runs its l forward transforms and
 *       owns its output polynomial; transformed digits cross SMs as
 *       asynchronous stores into the peer's shared memory, counted on its
 *       mbarrier (lowest latency: about 1.33 ms for a single gate's blind
 *       rotation).
 * FP64: 0 = automatic (the default): the two-SM cluster kernel for up to
 * one ciphertext per SM (one or two waves), else 3; 3 = L2-direct key
 * reads, 3 per CTA;
 * 4 = shared key ring fed in line; 16 = the cluster kernel (one owner group
 * per CTA: the FP64 key has one part).  Engine tuning knob, no counterpart
 * in the reference (its kernel is a single HLS work-item). */
tfhe_gpu_status tfhe_gpu_set_groups_per_cta(tfhe_gpu_ctx* ctx, tfhe_gpu_form form,
                                            int32_t groups);
int32_t tfhe_gpu_get_groups_per_cta(const tfhe_gpu_ctx* ctx, tfhe_gpu_form form);

/* ---- keys --------------------------------------------------------------- */

/* Upload the bootstrapping key in the time domain (host int32,
 * n x TGSW) and build the transform-domain copies of the forms in
 * `form_mask`.  Replaces the key the reference hands to the FPGA as
 * TGswSampleFFT_FPGA[n] (tfhe_blindRotate_FFT_tb.cpp:295-297, 342). */
tfhe_gpu_status tfhe_gpu_upload_bootstrapping_key(tfhe_gpu_ctx* ctx,
                                                  const int32_t* bk,
                                                  uint32_t form_mask);
/* Upload the bootstrapping key in the reference's transform format:
 * n x (k+1)l x (k+1) Lagrange polynomials, values of torus/2^32 at
 * w^(2m+1) (the a[] arrays of TGswSampleFFT_FPGA, tgswsample.h:8-16). */
tfhe_gpu_status tfhe_gpu_upload_bootstrapping_key_fft(tfhe_gpu_ctx* ctx,
                                                      const double* bk_fft,
                                                      uint32_t form_mask);
/* Upload the key-switching key (host int32 [kN][t][base][n+1]),
 * lwe-keyswitch-functions.cpp:85-99, 163-215. */
tfhe_gpu_status tfhe_gpu_upload_keyswitch_key(tfhe_gpu_ctx* ctx, const int32_t* ks);

/* Both cloud keys at once: the bootstrapping key (time domain, as
 * tfhe_gpu_upload_bootstrapping_key) and the key-switching key (as
 * tfhe_gpu_upload_keyswitch_key).  The upstream cloud keyset the test bench
 * loads (test_bench/server/cloud.c:42-44) carries exactly these two. */
tfhe_gpu_status tfhe_gpu_upload_cloud_key(tfhe_gpu_ctx* ctx, const int32_t* bk,
                                          const int32_t* ks, uint32_t form_mask);

/* Key generation for this context, with the bootstrapping key's arithmetic
 * on the GPU: the LWE key, TLWE key, key-switching key and every random
 * value of the bootstrapping key are drawn on the host in the order of
 * tfhe_client_gate_keyset (same generator state, bit-identical keys); the n
 * (k+1) l products a * s and the gadget terms are computed on the device,
 * and the key goes straight into the forms of form_mask together with the
 * key-switching key.  bk may be NULL; else it receives the time-domain key
 * (for export).  Upstream new_random_gate_bootstrapping_secret_keyset
 * (test_bench/client/alice.c:17) plus the key upload. */
tfhe_gpu_status tfhe_gpu_gate_keyset(tfhe_gpu_ctx* ctx, int32_t* lwe_key, int32_t* tlwe_key,
                                     int32_t* ks, int32_t* bk, uint32_t form_mask);

/* TGSW samples (device, count x TGSW int32) -> engine transform layout
 * (device, count x tfhe_gpu_tgsw_fft_bytes). Upstream tGswToFftConvert. */
tfhe_gpu_status tfhe_gpu_tgsw_to_fft(tfhe_gpu_ctx* ctx, const int32_t* tgsw,
                                     void* out, int32_t count,
                                     tfhe_gpu_form form, void* stream);

/* ---- Lagrange processor (FFT processor of LagrangeHalfCPolynomial) ----- */

/* IntPolynomial -> Lagrange (tGswFFTExternMulToTLwe.cpp:97-130, the correct
 * form of IntPolynomial_ifft, IntPolynomial_ifft.cpp:5-29). Device batch. */
tfhe_gpu_status tfhe_gpu_IntPolynomial_ifft(tfhe_gpu_ctx* ctx, const int32_t* polys,
                                            double* out, int32_t count, void* stream);
/* TorusPolynomial -> Lagrange, torus/2^32 scale (upstream
 * TorusPolynomial_ifft, the key conversion). Device batch. */
tfhe_gpu_status tfhe_gpu_TorusPolynomial_ifft(tfhe_gpu_ctx* ctx, const int32_t* polys,
                                              double* out, int32_t count, void* stream);
/* Lagrange -> TorusPolynomial, truncating (TorusPolynomial_fft.cpp:4-43,
 * tLweFromFFTConvert.cpp:4-24). Device batch. */
tfhe_gpu_status tfhe_gpu_TorusPolynomial_fft(tfhe_gpu_ctx* ctx, const double* in,
                                             int32_t* polys, int32_t count, void* stream);
/* accum += a * b pointwise (tGswFFTExternMulToTLwe.cpp:172-180). */
tfhe_gpu_status tfhe_gpu_LagrangeHalfCPolynomialAddMul(tfhe_gpu_ctx* ctx, double* accum,
                                                       const double* a, const double* b,
                                                       int32_t count, void* stream);

/* ---- hot path ------------------------------------------------------------ */

/* out = (X^{a_i} - 1) in, per TLWE sample i (tfhe_MuxRotate_FFT.cpp:5-33). */
tfhe_gpu_status tfhe_gpu_tLweMulByXaiMinusOne(tfhe_gpu_ctx* ctx, int32_t* out,
                                              const int32_t* ai, const int32_t* in,
                                              int32_t count, void* stream);
/* accum_i <- TGSW_i [x] accum_i (tGswFFTExternMulToTLwe.cpp:203-247).
 * gsw: engine layout (tfhe_gpu_tgsw_to_fft), `gsw_per_item` 1 = one TGSW
 * per sample, 0 = one TGSW shared by all. In place on device TLWEs. */
tfhe_gpu_status tfhe_gpu_tGswFFTExternMulToTLwe(tfhe_gpu_ctx* ctx, int32_t* accum,
                                                const void* gsw, int32_t gsw_per_item,
                                                int32_t count, tfhe_gpu_form form,
                                                void* stream);
/* result_i = TGSW_i [x] ((X^{a_i} - 1) accum_i) + accum_i
 * (tfhe_MuxRotate_FFT.cpp:56-85). */
tfhe_gpu_status tfhe_gpu_tfhe_MuxRotate_FFT(tfhe_gpu_ctx* ctx, int32_t* result,
                                            const int32_t* accum, const void* gsw,
                                            int32_t gsw_per_item, const int32_t* barai,
                                            int32_t count, tfhe_gpu_form form,
                                            void* stream);
/* Blind rotation of each accumulator by its bara[n] with the context's
 * bootstrapping key, all n steps, skipping bara_i = 0
 * (tfhe_blindRotate_FFT.cpp:61-147). In place. */
tfhe_gpu_status tfhe_gpu_tfhe_blindRotate_FFT(tfhe_gpu_ctx* ctx, int32_t* accum,
                                              const int32_t* bara, int32_t count,
                                              tfhe_gpu_form form, void* stream);
/* Sample extraction TLWE -> LWE(kN) (upstream tLweExtractLweSample). */
tfhe_gpu_status tfhe_gpu_tLweExtractLweSample(tfhe_gpu_ctx* ctx, int32_t* out,
                                              const int32_t* accum, int32_t count,
                                              void* stream);
/* Key switch LWE(kN) -> LWE(n) with the context's key
 * (lwe-keyswitch-functions.cpp:228-241).  out must not overlap in. */
tfhe_gpu_status tfhe_gpu_lweKeySwitch(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* in,
                                      int32_t count, void* stream);
/* Bootstrap without key switch: LWE(n) -> LWE(kN) with test vector mu
 * (upstream tfhe_bootstrap_woKS_FFT; front end
 * tfhe_bootstrap_woKS_FFT.cpp:27-73, mulByXaiOrCopy.cpp:3-44). */
tfhe_gpu_status tfhe_gpu_tfhe_bootstrap_woKS_FFT(tfhe_gpu_ctx* ctx, int32_t* out,
                                                 const int32_t* x, int32_t mu,
                                                 int32_t count, tfhe_gpu_form form,
                                                 void* stream);
/* Programmable bootstrap: the constant test vector mu of the gate bootstrap
 * (tfhe_bootstrap_woKS_FFT.cpp:63-66) replaced by a polynomial tv (device,
 * N int32; tv_stride = 0 shares one vector, N gives item c its own at
 * tv + c N).  The output encrypts F(phase) where F(j) = tv[j] for
 * j = round(2N phase) < N and -tv[j - N] above (negacyclic), i.e. a lookup
 * table on the phase (tfhe_client_test_vector builds tv from a table).
 * keyswitch = 1: out is count x (n+1) after the key switch; 0: count x
 * (kN+1) extracted samples.  Device batch. */
tfhe_gpu_status tfhe_gpu_bootstrap_tv(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* x,
                                      const int32_t* tv, int32_t tv_stride, int32_t count,
                                      tfhe_gpu_form form, int32_t keyswitch, void* stream);
/* Full bootstrap LWE(n) -> LWE(n) (upstream tfhe_bootstrap_FFT). */
tfhe_gpu_status tfhe_gpu_tfhe_bootstrap_FFT(tfhe_gpu_ctx* ctx, int32_t* out,
                                            const int32_t* x, int32_t mu, int32_t count,
                                            tfhe_gpu_form form, void* stream);

/* ---- gates (the calls of test_bench/server/cloud.c:10-35) ------------- */

/* Batched gates, one gate type for all: out_i = GATE(ca_i, cb_i).
 * Upstream bootsNAND/AND/OR/XOR/... ; the OR linear combination is
 * tfhe_blindRotate_FFT_tb.cpp:267-276. Device batch. */
tfhe_gpu_status tfhe_gpu_bootsGate(tfhe_gpu_ctx* ctx, int32_t gate, int32_t* out,
                                   const int32_t* ca, const int32_t* cb, int32_t count,
                                   tfhe_gpu_form form, void* stream);
/* Batched gates with a gate id per item (device int32[count]). */
tfhe_gpu_status tfhe_gpu_bootsGates(tfhe_gpu_ctx* ctx, const int32_t* gates, int32_t* out,
                                    const int32_t* ca, const int32_t* cb, int32_t count,
                                    tfhe_gpu_form form, void* stream);
/* Batched bootsMUX: out = a ? b : c (cloud.c:11,27). Device batch. */
tfhe_gpu_status tfhe_gpu_bootsMUX(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* a,
                                  const int32_t* b, const int32_t* c, int32_t count,
                                  tfhe_gpu_form form, void* stream);
/* Host-buffer form of tfhe_gpu_bootsGates: copies in, computes, copies out,
 * synchronises. `gates` may be NULL with `uniform_gate` used for all. */
tfhe_gpu_status tfhe_gpu_bootsGates_host(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                         int32_t uniform_gate, int32_t* out,
                                         const int32_t* ca, const int32_t* cb,
                                         int32_t count, tfhe_gpu_form form);
/* One circuit layer over several contexts -- normally one per GPU, each with
 * its own copy of the keys (the reference partitions nothing; this is the
 * engine's multi-GPU form of tfhe_gpu_bootsGates_host).  The `count` gates
 * are cut into nctx contiguous shards of sizes differing by at most one,
 * shard i runs on ctxs[i] through tfhe_gpu_bootsGates_host (one host thread
 * per context, all concurrently), and writes its outputs into its slice of
 * `out`, so the outputs come back in layer order.  The contexts must be
 * distinct and share the parameter set; each is used by this call only
 * until it returns.  On an error the first failing context's status is
 * returned (tfhe_gpu_last_error of that context says why). */
tfhe_gpu_status tfhe_gpu_bootsGates_host_split(tfhe_gpu_ctx* const* ctxs, int32_t nctx,
                                               const int32_t* gates, int32_t uniform_gate,
                                               int32_t* out, const int32_t* ca, const int32_t* cb,
                                               int32_t count, tfhe_gpu_form form);
/* Host-buffer form of tfhe_gpu_bootsMUX. */
tfhe_gpu_status tfhe_gpu_bootsMUX_host(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* a,
                                       const int32_t* b, const int32_t* c, int32_t count,
                                       tfhe_gpu_form form);

/* Same result as tfhe_gpu_bootsGates, but the call allocates no memory: its
 * intermediate samples live in a fixed 3.4 MB device array built into the
 * library (held on every GPU that loads it), for callers that must not
 * allocate inside a call (fixed memory budgets, latency-critical loops where
 * cudaMalloc/cudaFree would synchronise the device, frameworks that own all
 * device memory).  No counterpart in the reference.  Limit: count x
 * (n + 1 + kN + 1) int32 words <= 847,872 (512 gates of the default set);
 * larger calls return TFHE_GPU_BAD_PARAM.  The first call in each CUDA
 * context of a device looks up the array's address (make it before any
 * stream capture); a later context, e.g. after cudaDeviceReset, gets its own
 * lookup.  Calls that
 * overlap on the GPU share the array and race: serialise them. */
tfhe_gpu_status tfhe_gpu_bootsGates_noalloc(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                            int32_t* out, const int32_t* ca,
                                            const int32_t* cb, int32_t count,
                                            tfhe_gpu_form form, void* stream);

/* Self-test of the device-side failure path: runs one blind rotation of
 * `count` samples with the current launch shape of `form` whose key-row
 * stream is never started, so every bounded wait in the kernel runs out
 * (after about 2 s; the first one to give up tells the rest of its CTA to
 * stop waiting).  Returns what the host sees: TFHE_GPU_TIMEOUT for the
 * shared-ring shapes; TFHE_GPU_OK for the L2-direct shapes, which have no
 * waits.  The context stays usable.  No counterpart in the reference. */
tfhe_gpu_status tfhe_gpu_selftest_timeout(tfhe_gpu_ctx* ctx, tfhe_gpu_form form, int32_t count);

/* Measured FP32 FMA-pipe peak of `device` in TFLOP/s (and the probe's
 * duration in ms): independent chains of packed FP32 fused multiply-adds on
 * every SM, timed with CUDA events, best of 3 after a warm-up.  The
 * blind-rotation kernels' roofline is quoted against it.  No counterpart in
 * the reference.  iters = 65536 runs about 20 ms on a GB300. */
tfhe_gpu_status tfhe_gpu_measure_fp32_peak(int32_t device, int32_t iters, double* tflops, double* ms);
/* The same for the FP64 FMA pipe (independent FP64 FMA chains), the roof of
 * the plain FP64 form.  No counterpart in the reference.  iters = 2048 runs
 * about 30 ms on a GB300 (its FP64 rate is about 1/64 of its FP32 rate). */
tfhe_gpu_status tfhe_gpu_measure_fp64_peak(int32_t device, int32_t iters, double* tflops, double* ms);

/* ---- CUDA graph of a gate batch; launch-shape autotuner ----------------- */
/* Capture the whole gate pipeline of one batch (combination, blind rotation
 * and extraction, key switch) over fixed device buffers into a CUDA graph,
 * replayed by tfhe_gpu_graph_launch with one submission.  The graph owns its
 * intermediate buffers; the caller's buffers and the context's keys must
 * outlive it (re-uploading a key frees the old one: rebuild the graph after
 * that).  Creation runs the batch once eagerly.  No counterpart in the
 * reference (the FPGA kernel is enqueued per call). */
typedef struct tfhe_gpu_graph tfhe_gpu_graph;
tfhe_gpu_status tfhe_gpu_graph_gates_create(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                            int32_t uniform_gate, int32_t* out,
                                            const int32_t* ca, const int32_t* cb,
                                            int32_t count, tfhe_gpu_form form,
                                            tfhe_gpu_graph** graph);
tfhe_gpu_status tfhe_gpu_graph_launch(tfhe_gpu_graph* graph, void* stream);
/* Kernel nodes of the graph (the engine kernels one launch runs). */
int32_t tfhe_gpu_graph_kernel_count(const tfhe_gpu_graph* graph);
void tfhe_gpu_graph_destroy(tfhe_gpu_graph* graph);

/* Time the blind-rotation launch shapes of `form` (tfhe_gpu_set_groups_per_cta)
 * on `count` synthetic ciphertexts with CUDA events, keep the fastest as the
 * context's shape and return it with its time.  The first candidate (the
 * automatic shape) is kept unless another shape is more than 2 % faster. */
tfhe_gpu_status tfhe_gpu_autotune(tfhe_gpu_ctx* ctx, tfhe_gpu_form form, int32_t count,
                                  int32_t* best_shape, float* best_ms);

/* ---- serving: continuous-batching gate server (test_bench/server/cloud.c) */
/* The test_bench server runs one client's circuit gate by gate
 * (cloud.c:9-36, 39-74).  The engine's server admits circuits from many
 * clients into a device ciphertext pool of `pool_slots` slots (admission by
 * device memory: a circuit waits until its wires fit), and each
 * tfhe_gpu_server_step runs every ready gate of every admitted circuit as one
 * batch (at most `max_batch` bootstraps), so requests that arrive while
 * others run share their launches.  A circuit is a list of gates
 * {type, in0, in1, in2}: types 0..9 as tfhe_gpu_gate, 10 = MUX (in0 ? in1 :
 * in2), 11 = NOT, 12 = COPY, 13 = CONSTANT (in0 = the bit); wire ids
 * [0, ninputs) are the inputs, ninputs + g the output of gate g, and a
 * gate's inputs must be earlier wires.  Ticks are pipelined: a gate can be
 * scheduled once its inputs are scheduled (ticks run in order on the
 * context's stream), so a step enqueues its tick without waiting for the
 * one before; at most two ticks are in flight, and a step retires the ticks
 * it finds complete (outputs of finished circuits copied back inside the
 * tick, pool slots freed). */
typedef struct tfhe_gpu_server tfhe_gpu_server;
tfhe_gpu_status tfhe_gpu_server_create(tfhe_gpu_ctx* ctx, int32_t pool_slots, int32_t max_batch,
                                       tfhe_gpu_form form, tfhe_gpu_server** out);
void tfhe_gpu_server_destroy(tfhe_gpu_server* srv);
const char* tfhe_gpu_server_last_error(const tfhe_gpu_server* srv);
/* Queue a circuit; input_ct is host int32[ninputs][n+1]. */
tfhe_gpu_status tfhe_gpu_server_submit(tfhe_gpu_server* srv, const int32_t* gates, int32_t ngates,
                                       int32_t ninputs, const int32_t* input_ct,
                                       const int32_t* output_wires, int32_t noutputs,
                                       int64_t* request_id);
/* One tick: retire completed ticks, admit, enqueue every schedulable gate
 * (up to max_batch bootstraps) as one batch; with nothing to schedule it
 * waits for the oldest tick in flight.  *ran = gates enqueued (0 when there
 * was nothing to run).  max_batch must be at least 2 (a MUX is two
 * bootstraps); a circuit needs at least one gate. */
tfhe_gpu_status tfhe_gpu_server_step(tfhe_gpu_server* srv, int32_t* ran);
/* Outputs of a finished request (host int32[noutputs][n+1]); *done = 0 while
 * queued or running; latency from submission to completion in seconds. */
tfhe_gpu_status tfhe_gpu_server_poll(tfhe_gpu_server* srv, int64_t request_id, int32_t* out,
                                     int32_t* done, double* latency_s);
/* stats[0..7]: queued, active, free slots, bootstraps run, busy seconds,
 * gate latencies recorded, request latencies recorded, pool slots; gate
 * (ready -> done) and request latencies copied up to cap[0], cap[1] entries
 * (the server keeps the most recent 2^22 to 2^23 of each). */
tfhe_gpu_status tfhe_gpu_server_stats(tfhe_gpu_server* srv, double* stats, double* gate_lat,
                                      double* req_lat, int64_t* cap);

/* ---- client side (host): keygen, encryption, decryption --------------- */
/* Exact semantics of the reference's numeric functions
 * (kernel/src/numeric-functions.cpp:11-76, lwe-functions.cpp:21-93) and of
 * the upstream keyset generation they belong to.  Host-only, no GPU use. */

void tfhe_client_set_seed(const uint32_t* values, int32_t size);
/* new_random_gate_bootstrapping_secret_keyset: LWE key (n), TLWE key (kN),
 * key-switching key and time-domain bootstrapping key, in that RNG order. */
tfhe_gpu_status tfhe_client_gate_keyset(const tfhe_params* params, int32_t* lwe_key,
                                        int32_t* tlwe_key, int32_t* ks, int32_t* bk);
/* bootsSymEncrypt of `count` bits into count x (n+1) samples. */
tfhe_gpu_status tfhe_client_encrypt_bits(const tfhe_params* params, const int32_t* bits,
                                         int32_t count, const int32_t* lwe_key,
                                         int32_t* out);
/* Encrypt arbitrary Torus32 messages mu[count] (lweSymEncrypt,
 * lwe-functions.cpp:40-53), e.g. modSwitchToTorus32(m, 2p) for the padded
 * messages of a programmable bootstrap. */
tfhe_gpu_status tfhe_client_encrypt_phases(const tfhe_params* params, const int32_t* mu,
                                           int32_t count, const int32_t* lwe_key, int32_t* out);
/* Test vector of a lookup table on p messages with a padding bit (message m
 * encrypted at phase m/(2p)): tv[j] = table[m] over m's window, -table[0]
 * over the top half-window (negacyclic wrap onto message 0). */
tfhe_gpu_status tfhe_client_test_vector(int32_t N, const int32_t* table, int32_t p, int32_t* tv);
/* bootsSymDecrypt: bit = phase > 0. */
tfhe_gpu_status tfhe_client_decrypt_bits(const tfhe_params* params, const int32_t* samples,
                                         int32_t count, const int32_t* lwe_key,
                                         int32_t* bits);
/* phase b - <a, s> of count samples of dimension `dim`. */
void tfhe_client_phases(const int32_t* samples, int32_t count, int32_t dim,
                        const int32_t* key, int32_t* phases);
/* modSwitchToTorus32 (numeric-functions.cpp:71-76). */
int32_t tfhe_client_mod_switch_to_torus32(int32_t mu, int32_t Msize);

#ifdef __cplusplus
}
#endif
#endif
