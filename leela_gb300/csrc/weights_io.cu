// weights_io.cu -- a weight file format for the nets, so trained weights can
// replace the compiled-in arrays the reference expects (its NN.cpp /
// NN128.cpp / NNValue.cpp define `const std::array<float,N>` globals,
// Network.cpp:54-137; those files are absent).
//
// File layout (little-endian):
//   "LGWF", u32 version (1), u32 n_nets, u32 0
//   per net: char name[16], i32 shape[11] (the lg_net_desc fields c_in ..
//            precision in order), u32 0, u64 count (72 bytes), count x f32,
//            zero pad to a multiple of 16 bytes
//   u64 FNV-1a of every preceding byte, "LGWFEND\0"
// The weights of a net are the flat lg_net_desc array (per conv W[O][C][k][k]
// then b[O], then the value FCs), i.e. the reference's arrays concatenated.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lg_kernels.h"

namespace {

constexpr uint32_t kVersion = 1;

uint64_t fnv1a(const unsigned char *p, size_t n, uint64_t h = 1469598103934665603ULL) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

void put(std::vector<unsigned char> &b, const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    b.insert(b.end(), c, c + n);
}

void desc_shape(const lg_net_desc *d, int32_t sh[11]) {
    const int v[11] = {d->c_in,   d->width1,     d->width,     d->n3x3,      d->head_k,   d->act,
                       d->act_head, d->value_head, d->fc_hidden, d->value_map, d->precision};
    for (int i = 0; i < 11; ++i) sh[i] = v[i];
}

}  // namespace

extern "C" int lg_weights_save(const char *path, const lg_net_desc *descs, const char *const *names, int n) {
    if (!path || !descs || n < 1 || n > 1024) {
        lg_set_error("lg_weights_save: bad arguments");
        return LG_ERR_ARG;
    }
    std::vector<unsigned char> b;
    put(b, "LGWF", 4);
    uint32_t hdr[3] = {kVersion, (uint32_t)n, 0};
    put(b, hdr, sizeof hdr);
    for (int i = 0; i < n; ++i) {
        const lg_net_desc *d = &descs[i];
        size_t count = lg_weight_count(d);
        if (count == 0 || !d->weights) {
            lg_set_error("lg_weights_save: net %d has an invalid description", i);
            return LG_ERR_ARG;
        }
        char name[16] = {0};
        if (names && names[i]) std::strncpy(name, names[i], 15);
        put(b, name, 16);
        int32_t sh[11];
        desc_shape(d, sh);
        put(b, sh, sizeof sh);
        uint32_t zero = 0;
        put(b, &zero, 4);
        uint64_t c64 = count;
        put(b, &c64, 8);
        put(b, d->weights, count * sizeof(float));
        while (b.size() % 16) b.push_back(0);
    }
    uint64_t h = fnv1a(b.data(), b.size());
    put(b, &h, 8);
    put(b, "LGWFEND", 8);
    std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) {
        lg_set_error("cannot write %s", tmp.c_str());
        return LG_ERR_ARG;
    }
    bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        lg_set_error("write of %s failed", path);
        return LG_ERR_ARG;
    }
    return LG_OK;
}

// Net `index` of the file: its description (desc->weights = weights), name
// and weights.  With weights == NULL only *count_out and the description
// are filled, so that the caller can size its buffer.  Returns the number of
// nets in the file, or < 0 on error (bad magic, version, checksum, size).
extern "C" int lg_weights_load(const char *path, int index, lg_net_desc *desc, char *name16, float *weights,
                               size_t capacity, size_t *count_out) {
    if (!path || index < 0) {
        lg_set_error("lg_weights_load: bad arguments");
        return LG_ERR_ARG;
    }
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        lg_set_error("cannot open %s", path);
        return LG_ERR_ARG;
    }
    std::vector<unsigned char> b;
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + got);
    std::fclose(f);
    if (b.size() < 32 || std::memcmp(b.data(), "LGWF", 4) != 0 ||
        std::memcmp(b.data() + b.size() - 8, "LGWFEND", 8) != 0) {
        lg_set_error("%s: not a weight file (or truncated)", path);
        return LG_ERR_ARG;
    }
    uint64_t h;
    std::memcpy(&h, b.data() + b.size() - 16, 8);
    if (fnv1a(b.data(), b.size() - 16) != h) {
        lg_set_error("%s: checksum mismatch", path);
        return LG_ERR_ARG;
    }
    uint32_t hdr[3];
    std::memcpy(hdr, b.data() + 4, sizeof hdr);
    if (hdr[0] != kVersion) {
        lg_set_error("%s: version %u not supported", path, hdr[0]);
        return LG_ERR_ARG;
    }
    const int n = (int)hdr[1];
    if (index >= n) {
        lg_set_error("%s holds %d nets", path, n);
        return LG_ERR_ARG;
    }
    size_t off = 16;
    const size_t end = b.size() - 16;
    for (int i = 0; i < n; ++i) {
        // record header: name[16], shape i32[11], u32 0, u64 count = 72 bytes
        if (off + 72 > end) {
            lg_set_error("%s: truncated record", path);
            return LG_ERR_ARG;
        }
        char nm[16];
        std::memcpy(nm, b.data() + off, 16);
        int32_t sh[11];
        std::memcpy(sh, b.data() + off + 16, sizeof sh);
        uint64_t count;
        std::memcpy(&count, b.data() + off + 64, 8);
        off += 72;
        if (off + count * sizeof(float) > end) {
            lg_set_error("%s: truncated weights", path);
            return LG_ERR_ARG;
        }
        if (i == index) {
            lg_net_desc d{};
            d.c_in = sh[0]; d.width1 = sh[1]; d.width = sh[2]; d.n3x3 = sh[3]; d.head_k = sh[4];
            d.act = sh[5]; d.act_head = sh[6]; d.value_head = sh[7]; d.fc_hidden = sh[8];
            d.value_map = sh[9]; d.precision = sh[10];
            if (lg_weight_count(&d) != count) {
                lg_set_error("%s: net %d holds %llu weights, its shape needs %zu", path, i,
                             (unsigned long long)count, lg_weight_count(&d));
                return LG_ERR_ARG;
            }
            if (count_out) *count_out = count;
            if (name16) {
                std::memcpy(name16, nm, 16);
                name16[15] = 0;
            }
            if (weights) {
                if (capacity < count) {
                    lg_set_error("lg_weights_load: buffer holds %zu floats, need %llu", capacity,
                                 (unsigned long long)count);
                    return LG_ERR_ARG;
                }
                std::memcpy(weights, b.data() + off, count * sizeof(float));
            }
            d.weights = weights;
            if (desc) *desc = d;
            return n;
        }
        off += count * sizeof(float);
        off = (off + 15) & ~(size_t)15;
    }
    lg_set_error("%s: net %d not found", path, index);
    return LG_ERR_ARG;
}
