// keyfile.cpp -- the engine's versioned binary format for parameter sets,
// keys and ciphertexts (include/tfhe_keyfile.h), and loading a cloud key
// file into a context.  Host code; no GPU use except in
// tfhe_gpu_upload_cloud_key_file.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/tfhe_gpu.h"
#include "../../include/tfhe_keyfile.h"

namespace {

constexpr char kMagic[8] = {'T', 'F', 'H', 'E', 'G', 'B', '3', 'K'};
constexpr size_t kHeaderBytes = 32;
constexpr size_t kParamBytes = 64;

static_assert(sizeof(int32_t) == 4 && sizeof(double) == 8, "sizes");

bool host_is_little_endian() {
    const uint32_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

uint32_t fnv1a(uint32_t h, const void* data, size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < bytes; ++i) {
        h ^= p[i];
        h *= 16777619u;
    }
    return h;
}
constexpr uint32_t kFnvSeed = 2166136261u;

bool params_sane(const tfhe_params& P) {
    return P.n > 0 && P.n <= (1 << 16) && P.N > 0 && P.N <= (1 << 16) && (P.N & (P.N - 1)) == 0 &&
           P.k >= 1 && P.k <= 8 && P.l >= 1 && P.l <= 16 && P.Bgbit >= 1 && P.Bgbit * P.l <= 32 &&
           P.ks_t >= 1 && P.ks_basebit >= 1 && P.ks_t * P.ks_basebit <= 32 && P.ks_basebit <= 8;
}

int64_t bk_words(const tfhe_params& P) {
    return (int64_t)P.n * (P.k + 1) * P.l * (P.k + 1) * P.N;
}
int64_t ks_words(const tfhe_params& P) {
    return (int64_t)P.k * P.N * P.ks_t * ((int64_t)1 << P.ks_basebit) * (P.n + 1);
}

void pack_params(const tfhe_params& P, unsigned char* out) {
    std::memset(out, 0, kParamBytes);
    const int32_t iv[8] = {P.n, P.N, P.k, P.l, P.Bgbit, P.ks_t, P.ks_basebit, P.split_bits};
    std::memcpy(out, iv, sizeof(iv));
    std::memcpy(out + 32, &P.lwe_alpha, 8);
    std::memcpy(out + 40, &P.tlwe_alpha, 8);
}

void unpack_params(const unsigned char* in, tfhe_params* P) {
    int32_t iv[8];
    std::memcpy(iv, in, sizeof(iv));
    P->n = iv[0];
    P->N = iv[1];
    P->k = iv[2];
    P->l = iv[3];
    P->Bgbit = iv[4];
    P->ks_t = iv[5];
    P->ks_basebit = iv[6];
    P->split_bits = iv[7];
    std::memcpy(&P->lwe_alpha, in + 32, 8);
    std::memcpy(&P->tlwe_alpha, in + 40, 8);
}

// A record writer: the payload is assembled piecewise; the header (with the
// checksum) is written first, so the pieces are checksummed before writing.
struct Piece {
    const void* data;
    size_t bytes;
};

tfhe_gpu_status write_record(FILE* f, uint32_t kind, const std::vector<Piece>& pieces) {
    if (!f || !host_is_little_endian()) return TFHE_GPU_BAD_PARAM;
    uint64_t total = 0;
    uint32_t h = kFnvSeed;
    for (const Piece& p : pieces) {
        if (p.bytes && !p.data) return TFHE_GPU_BAD_PARAM;
        total += p.bytes;
        h = fnv1a(h, p.data, p.bytes);
    }
    unsigned char hdr[kHeaderBytes] = {};
    std::memcpy(hdr, kMagic, 8);
    const uint32_t version = TFHE_KEYFILE_VERSION;
    std::memcpy(hdr + 8, &version, 4);
    std::memcpy(hdr + 12, &kind, 4);
    std::memcpy(hdr + 16, &total, 8);
    std::memcpy(hdr + 24, &h, 4);
    if (std::fwrite(hdr, 1, kHeaderBytes, f) != kHeaderBytes) return TFHE_GPU_DEVICE_ERROR;
    for (const Piece& p : pieces)
        if (p.bytes && std::fwrite(p.data, 1, p.bytes, f) != p.bytes) return TFHE_GPU_DEVICE_ERROR;
    return TFHE_GPU_OK;
}

struct Header {
    uint32_t version, kind, checksum;
    uint64_t payload;
};

bool read_header(FILE* f, Header* h) {
    unsigned char hdr[kHeaderBytes];
    if (std::fread(hdr, 1, kHeaderBytes, f) != kHeaderBytes) return false;
    if (std::memcmp(hdr, kMagic, 8) != 0) return false;
    std::memcpy(&h->version, hdr + 8, 4);
    std::memcpy(&h->kind, hdr + 12, 4);
    std::memcpy(&h->payload, hdr + 16, 8);
    std::memcpy(&h->checksum, hdr + 24, 4);
    return h->version == TFHE_KEYFILE_VERSION;
}

// Reads a whole record of `kind` into memory after checking its header,
// size and checksum.  On failure the stream is put back where it was.
tfhe_gpu_status read_record(FILE* f, uint32_t kind, std::vector<unsigned char>* payload,
                            tfhe_params* P) {
    if (!f || !host_is_little_endian()) return TFHE_GPU_BAD_PARAM;
    const long start = std::ftell(f);
    auto rewind_fail = [&]() {
        if (start >= 0) std::fseek(f, start, SEEK_SET);
        return TFHE_GPU_BAD_PARAM;
    };
    Header h;
    if (!read_header(f, &h) || h.kind != kind || h.payload < kParamBytes ||
        h.payload > ((uint64_t)1 << 40))
        return rewind_fail();
    unsigned char pb[kParamBytes];
    if (std::fread(pb, 1, kParamBytes, f) != kParamBytes) return rewind_fail();
    tfhe_params p;
    unpack_params(pb, &p);
    if (!params_sane(p)) return rewind_fail();
    // expected payload size from the parameters
    uint64_t want = kParamBytes;
    switch (kind) {
    case TFHE_KEYFILE_PARAMS: break;
    case TFHE_KEYFILE_CLOUD_KEY: want += 8 + 4 * (uint64_t)(bk_words(p) + ks_words(p)); break;
    case TFHE_KEYFILE_SECRET_KEY:
        want += 4 * (uint64_t)(p.n + p.k * p.N) + 8 + 4 * (uint64_t)(bk_words(p) + ks_words(p));
        break;
    case TFHE_KEYFILE_CIPHERTEXTS: {
        uint64_t count = 0;
        if (h.payload < kParamBytes + 8 || std::fread(&count, 1, 8, f) != 8) return rewind_fail();
        if (count > ((uint64_t)1 << 32)) return rewind_fail();
        want += 8 + count * (4 * (uint64_t)(p.n + 1) + 8);
        if (std::fseek(f, -8, SEEK_CUR) != 0) return rewind_fail();
        break;
    }
    default: return rewind_fail();
    }
    if (h.payload != want) return rewind_fail();
    payload->resize(h.payload);
    std::memcpy(payload->data(), pb, kParamBytes);
    const size_t rest = h.payload - kParamBytes;
    if (rest && std::fread(payload->data() + kParamBytes, 1, rest, f) != rest) return rewind_fail();
    if (fnv1a(kFnvSeed, payload->data(), payload->size()) != h.checksum) return rewind_fail();
    if (P) *P = p;
    return TFHE_GPU_OK;
}

void copy_out(void* dst, const unsigned char* src, size_t bytes) {
    if (dst && bytes) std::memcpy(dst, src, bytes);
}

}  // namespace

extern "C" {

int64_t tfhe_keyfile_bk_words(const tfhe_params* P) { return P && params_sane(*P) ? bk_words(*P) : 0; }
int64_t tfhe_keyfile_ks_words(const tfhe_params* P) { return P && params_sane(*P) ? ks_words(*P) : 0; }

tfhe_gpu_status tfhe_keyfile_peek(FILE* f, int32_t* kind, tfhe_params* params, int64_t* items) {
    if (!f) return TFHE_GPU_BAD_PARAM;
    const long start = std::ftell(f);
    Header h;
    unsigned char pb[kParamBytes];
    uint64_t count = 1;
    bool ok = read_header(f, &h) && h.payload >= kParamBytes &&
              std::fread(pb, 1, kParamBytes, f) == kParamBytes;
    if (ok && h.kind == TFHE_KEYFILE_CIPHERTEXTS)
        ok = h.payload >= kParamBytes + 8 && std::fread(&count, 1, 8, f) == 8;
    if (start >= 0) std::fseek(f, start, SEEK_SET);
    if (!ok) return TFHE_GPU_BAD_PARAM;
    tfhe_params p;
    unpack_params(pb, &p);
    if (!params_sane(p)) return TFHE_GPU_BAD_PARAM;
    if (kind) *kind = (int32_t)h.kind;
    if (params) *params = p;
    if (items) *items = (int64_t)count;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_keyfile_write_params(FILE* f, const tfhe_params* P) {
    if (!P || !params_sane(*P)) return TFHE_GPU_BAD_PARAM;
    unsigned char pb[kParamBytes];
    pack_params(*P, pb);
    return write_record(f, TFHE_KEYFILE_PARAMS, {{pb, kParamBytes}});
}

tfhe_gpu_status tfhe_keyfile_write_cloud_key(FILE* f, const tfhe_params* P, const int32_t* bk,
                                             const int32_t* ks) {
    if (!P || !params_sane(*P) || !bk || !ks) return TFHE_GPU_BAD_PARAM;
    unsigned char pb[kParamBytes];
    pack_params(*P, pb);
    const uint32_t dom[2] = {0, 0};
    return write_record(f, TFHE_KEYFILE_CLOUD_KEY,
                        {{pb, kParamBytes}, {dom, 8}, {bk, 4 * (size_t)bk_words(*P)},
                         {ks, 4 * (size_t)ks_words(*P)}});
}

tfhe_gpu_status tfhe_keyfile_write_secret_key(FILE* f, const tfhe_params* P, const int32_t* lwe_key,
                                              const int32_t* tlwe_key, const int32_t* bk,
                                              const int32_t* ks) {
    if (!P || !params_sane(*P) || !lwe_key || !tlwe_key || !bk || !ks) return TFHE_GPU_BAD_PARAM;
    unsigned char pb[kParamBytes];
    pack_params(*P, pb);
    const uint32_t dom[2] = {0, 0};
    return write_record(f, TFHE_KEYFILE_SECRET_KEY,
                        {{pb, kParamBytes}, {lwe_key, 4 * (size_t)P->n},
                         {tlwe_key, 4 * (size_t)P->k * P->N}, {dom, 8},
                         {bk, 4 * (size_t)bk_words(*P)}, {ks, 4 * (size_t)ks_words(*P)}});
}

tfhe_gpu_status tfhe_keyfile_write_ciphertexts(FILE* f, const tfhe_params* P, const int32_t* samples,
                                               const double* variance, int64_t count) {
    if (!P || !params_sane(*P) || count < 0 || (count && !samples)) return TFHE_GPU_BAD_PARAM;
    unsigned char pb[kParamBytes];
    pack_params(*P, pb);
    const uint64_t c = (uint64_t)count;
    std::vector<double> zeros;
    if (!variance) {
        zeros.assign((size_t)count, 0.0);
        variance = zeros.data();
    }
    return write_record(f, TFHE_KEYFILE_CIPHERTEXTS,
                        {{pb, kParamBytes}, {&c, 8}, {samples, 4 * (size_t)count * (P->n + 1)},
                         {variance, 8 * (size_t)count}});
}

tfhe_gpu_status tfhe_keyfile_read_params(FILE* f, tfhe_params* params) {
    std::vector<unsigned char> buf;
    return read_record(f, TFHE_KEYFILE_PARAMS, &buf, params);
}

tfhe_gpu_status tfhe_keyfile_read_cloud_key(FILE* f, tfhe_params* params, int32_t* bk, int32_t* ks) {
    std::vector<unsigned char> buf;
    tfhe_params P;
    tfhe_gpu_status s = read_record(f, TFHE_KEYFILE_CLOUD_KEY, &buf, &P);
    if (s != TFHE_GPU_OK) return s;
    uint32_t dom;
    std::memcpy(&dom, buf.data() + kParamBytes, 4);
    if (dom != 0) return TFHE_GPU_BAD_PARAM;
    const unsigned char* p = buf.data() + kParamBytes + 8;
    copy_out(bk, p, 4 * (size_t)bk_words(P));
    copy_out(ks, p + 4 * (size_t)bk_words(P), 4 * (size_t)ks_words(P));
    if (params) *params = P;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_keyfile_read_secret_key(FILE* f, tfhe_params* params, int32_t* lwe_key,
                                             int32_t* tlwe_key, int32_t* bk, int32_t* ks) {
    std::vector<unsigned char> buf;
    tfhe_params P;
    tfhe_gpu_status s = read_record(f, TFHE_KEYFILE_SECRET_KEY, &buf, &P);
    if (s != TFHE_GPU_OK) return s;
    const unsigned char* p = buf.data() + kParamBytes;
    copy_out(lwe_key, p, 4 * (size_t)P.n);
    p += 4 * (size_t)P.n;
    copy_out(tlwe_key, p, 4 * (size_t)P.k * P.N);
    p += 4 * (size_t)P.k * P.N;
    uint32_t dom;
    std::memcpy(&dom, p, 4);
    if (dom != 0) return TFHE_GPU_BAD_PARAM;
    p += 8;
    copy_out(bk, p, 4 * (size_t)bk_words(P));
    copy_out(ks, p + 4 * (size_t)bk_words(P), 4 * (size_t)ks_words(P));
    if (params) *params = P;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_keyfile_read_ciphertexts(FILE* f, tfhe_params* params, int32_t* samples,
                                              double* variance, int64_t* count) {
    if (!count || *count < 0) return TFHE_GPU_BAD_PARAM;
    const long start = std::ftell(f);
    std::vector<unsigned char> buf;
    tfhe_params P;
    tfhe_gpu_status s = read_record(f, TFHE_KEYFILE_CIPHERTEXTS, &buf, &P);
    if (s != TFHE_GPU_OK) return s;
    uint64_t c;
    std::memcpy(&c, buf.data() + kParamBytes, 8);
    if ((samples || variance) && c > (uint64_t)*count) {
        if (start >= 0) std::fseek(f, start, SEEK_SET);
        return TFHE_GPU_BAD_PARAM;
    }
    const unsigned char* p = buf.data() + kParamBytes + 8;
    copy_out(samples, p, 4 * (size_t)c * (P.n + 1));
    copy_out(variance, p + 4 * (size_t)c * (P.n + 1), 8 * (size_t)c);
    *count = (int64_t)c;
    if (params) *params = P;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_keyfile_save_cloud_key(const char* path, const tfhe_params* params,
                                            const int32_t* bk, const int32_t* ks) {
    if (!path) return TFHE_GPU_BAD_PARAM;
    FILE* f = std::fopen(path, "wb");
    if (!f) return TFHE_GPU_BAD_PARAM;
    tfhe_gpu_status s = tfhe_keyfile_write_cloud_key(f, params, bk, ks);
    if (std::fclose(f) != 0 && s == TFHE_GPU_OK) s = TFHE_GPU_DEVICE_ERROR;
    return s;
}

tfhe_gpu_status tfhe_keyfile_load_cloud_key(const char* path, tfhe_params* params, int32_t* bk,
                                            int32_t* ks) {
    if (!path) return TFHE_GPU_BAD_PARAM;
    FILE* f = std::fopen(path, "rb");
    if (!f) return TFHE_GPU_BAD_PARAM;
    tfhe_gpu_status s = tfhe_keyfile_read_cloud_key(f, params, bk, ks);
    std::fclose(f);
    return s;
}

tfhe_gpu_status tfhe_gpu_upload_cloud_key_file(tfhe_gpu_ctx* ctx, const char* path,
                                               uint32_t form_mask) {
    if (!ctx || !path) return TFHE_GPU_BAD_PARAM;
    FILE* f = std::fopen(path, "rb");
    if (!f) return TFHE_GPU_BAD_PARAM;
    int32_t kind = 0;
    tfhe_params P;
    tfhe_gpu_status s = tfhe_keyfile_peek(f, &kind, &P, nullptr);
    tfhe_params C;
    if (s == TFHE_GPU_OK) s = tfhe_gpu_get_params(ctx, &C);
    if (s == TFHE_GPU_OK && (P.n != C.n || P.N != C.N || P.k != C.k || P.l != C.l ||
                             P.Bgbit != C.Bgbit || P.ks_t != C.ks_t || P.ks_basebit != C.ks_basebit))
        s = TFHE_GPU_BAD_PARAM;
    std::vector<int32_t> bk, ks;
    if (s == TFHE_GPU_OK) {
        bk.resize((size_t)bk_words(P));
        ks.resize((size_t)ks_words(P));
        if (kind == TFHE_KEYFILE_CLOUD_KEY)
            s = tfhe_keyfile_read_cloud_key(f, nullptr, bk.data(), ks.data());
        else if (kind == TFHE_KEYFILE_SECRET_KEY)
            s = tfhe_keyfile_read_secret_key(f, nullptr, nullptr, nullptr, bk.data(), ks.data());
        else
            s = TFHE_GPU_BAD_PARAM;
    }
    std::fclose(f);
    if (s == TFHE_GPU_OK) s = tfhe_gpu_upload_cloud_key(ctx, bk.data(), ks.data(), form_mask);
    return s;
}

}  // extern "C"
