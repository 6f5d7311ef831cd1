// config_io.cpp — the reference's two creature file formats (ml-rs/config.rs).
//
//   seed/{name}.json   (config.rs:14-47; written by
//                       train/generate_kernel_json.py:195-215)
//   kernels/{name}_{n}.bin  (config.rs:49-125; generate_kernel_json.py:182-192)
//
// and a binary twin of the seed format (no reference counterpart), which
// holds exactly the fields of the JSON so a conversion either way is
// lossless.  All little-endian:
//
//   offset 0   8 bytes  magic "CNSEED01"
//          8   u32      seed_size n
//         12   u32      num_channels C
//         16   u32      num_kernels K
//         20   f32      temp
//         24   u32[K]   the JSON "c0" field (output channel; swapped on load
//                       as config.rs:40 swaps the JSON fields)
//              u32[K]   the JSON "c1" field (input channel)
//              f32[K]   growth_mu, then growth_sigma, then growth_weights
//              zero padding to a multiple of 8 bytes
//              f64[C][n][n]  seed_channels
//
// A small JSON reader of its own (objects, arrays, numbers, strings,
// literals) is enough for the seed format; unknown keys are skipped, as
// serde does for SimConfig.  Failures return a status instead of panicking
// (config.rs:33-34 uses expect).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cella_gpu.h"

namespace cg {
int fail(int code, const char* fmt, ...);
}

namespace {

struct Reader {
    const char* p;
    const char* end;
    std::string err;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool expect(char c) {
        ws();
        if (p < end && *p == c) {
            ++p;
            return true;
        }
        err = std::string("expected '") + c + "'";
        return false;
    }
    bool peek(char c) {
        ws();
        return p < end && *p == c;
    }
    bool string(std::string& out) {
        ws();
        if (p >= end || *p != '"') {
            err = "expected a string";
            return false;
        }
        ++p;
        out.clear();
        while (p < end && *p != '"') {
            if (*p == '\\' && p + 1 < end) ++p;
            out.push_back(*p++);
        }
        if (p >= end) {
            err = "unterminated string";
            return false;
        }
        ++p;
        return true;
    }
    bool number(double& v) {
        ws();
        char* e = nullptr;
        v = std::strtod(p, &e);
        if (e == p) {
            err = "expected a number";
            return false;
        }
        p = e;
        return true;
    }
    bool number_array(std::vector<double>& out) {
        out.clear();
        if (!expect('[')) return false;
        if (peek(']')) {
            ++p;
            return true;
        }
        for (;;) {
            double v;
            if (!number(v)) return false;
            out.push_back(v);
            ws();
            if (p < end && *p == ',') {
                ++p;
                continue;
            }
            return expect(']');
        }
    }
    bool skip_value() {
        ws();
        if (p >= end) {
            err = "unexpected end of file";
            return false;
        }
        if (*p == '"') {
            std::string s;
            return string(s);
        }
        if (*p == '[' || *p == '{') {
            const char open = *p, close = open == '[' ? ']' : '}';
            ++p;
            if (peek(close)) {
                ++p;
                return true;
            }
            for (;;) {
                if (open == '{') {
                    std::string k;
                    if (!string(k) || !expect(':')) return false;
                }
                if (!skip_value()) return false;
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                return expect(close);
            }
        }
        if (std::strncmp(p, "true", 4) == 0 || std::strncmp(p, "null", 4) == 0) {
            p += 4;
            return true;
        }
        if (std::strncmp(p, "false", 5) == 0) {
            p += 5;
            return true;
        }
        double v;
        return number(v);
    }
};

bool read_file(const char* path, std::vector<char>& buf) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize(size_t(sz) + 1);
    size_t got = std::fread(buf.data(), 1, size_t(sz), f);
    std::fclose(f);
    buf[got] = '\0';
    buf.resize(got + 1);
    return got == size_t(sz);
}

constexpr char kSeedMagic[8] = {'C', 'N', 'S', 'E', 'E', 'D', '0', '1'};

size_t seed_bin_header(int K) {
    const size_t h = 24 + size_t(K) * 4 * 5;
    return (h + 7) & ~size_t(7);
}

uint32_t get_u32(const unsigned char* b) {
    return uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
}

float get_f32(const unsigned char* b) {
    const uint32_t u = get_u32(b);
    float v;
    std::memcpy(&v, &u, 4);
    return v;
}

double get_f64(const unsigned char* b) {
    const uint64_t u = uint64_t(get_u32(b)) | (uint64_t(get_u32(b + 4)) << 32);
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

void put_u32(std::vector<unsigned char>& o, uint32_t u) {
    for (int i = 0; i < 4; ++i) o.push_back(static_cast<unsigned char>(u >> (8 * i)));
}

void put_f32(std::vector<unsigned char>& o, float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    put_u32(o, u);
}

template <class T>
T* dup_array(const std::vector<double>& v) {
    T* out = static_cast<T*>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
    if (!out) return nullptr;
    for (size_t i = 0; i < v.size(); ++i) out[i] = T(v[i]);
    return out;
}

}  // namespace

extern "C" {

void cg_free_config(cg_config* c) {
    if (!c) return;
    std::free(c->seed_channels);
    std::free(c->c0);
    std::free(c->c1);
    std::free(c->growth_mu);
    std::free(c->growth_sigma);
    std::free(c->growth_weights);
    std::memset(c, 0, sizeof(*c));
}

int cg_load_config_json(const char* path, cg_config* out) {
    using cg::fail;
    if (!path || !out) return fail(CG_ERR_ARG, "cg_load_config_json: NULL argument");
    std::memset(out, 0, sizeof(*out));
    std::vector<char> buf;
    if (!read_file(path, buf)) return fail(CG_ERR_IO, "cannot read config file %s", path);
    Reader r{buf.data(), buf.data() + buf.size() - 1, {}};
    double seed_size = -1, nch = -1, nk = -1, temp = 1.0;
    std::vector<std::vector<double>> seed;
    std::vector<double> c0, c1, mu, sg, w;
    bool have_c0 = false, have_c1 = false, have_mu = false, have_sg = false, have_w = false;
    bool have_seed = false;
    if (!r.expect('{')) return fail(CG_ERR_FORMAT, "%s: %s", path, r.err.c_str());
    if (!r.peek('}')) {
        for (;;) {
            std::string key;
            if (!r.string(key) || !r.expect(':'))
                return fail(CG_ERR_FORMAT, "%s: %s", path, r.err.c_str());
            bool ok = true;
            if (key == "seed_size") ok = r.number(seed_size);
            else if (key == "num_channels") ok = r.number(nch);
            else if (key == "num_kernels") ok = r.number(nk);
            else if (key == "temp") ok = r.number(temp);
            else if (key == "c0") ok = have_c0 = r.number_array(c0);
            else if (key == "c1") ok = have_c1 = r.number_array(c1);
            else if (key == "growth_mu") ok = have_mu = r.number_array(mu);
            else if (key == "growth_sigma") ok = have_sg = r.number_array(sg);
            else if (key == "growth_weights") ok = have_w = r.number_array(w);
            else if (key == "seed_channels") {
                have_seed = true;
                ok = r.expect('[');
                if (ok && !r.peek(']')) {
                    for (;;) {
                        seed.emplace_back();
                        if (!(ok = r.number_array(seed.back()))) break;
                        r.ws();
                        if (r.p < r.end && *r.p == ',') {
                            ++r.p;
                            continue;
                        }
                        ok = r.expect(']');
                        break;
                    }
                } else if (ok) {
                    ++r.p;
                }
            } else ok = r.skip_value();
            if (!ok) return fail(CG_ERR_FORMAT, "%s: key \"%s\": %s", path, key.c_str(), r.err.c_str());
            r.ws();
            if (r.p < r.end && *r.p == ',') {
                ++r.p;
                continue;
            }
            if (!r.expect('}')) return fail(CG_ERR_FORMAT, "%s: %s", path, r.err.c_str());
            break;
        }
    }
    if (seed_size < 1 || nch < 1 || nk < 1 || !have_seed || !have_c0 || !have_c1 || !have_mu ||
        !have_sg || !have_w)
        return fail(CG_ERR_FORMAT, "%s: missing one of the SimConfig fields (config.rs:15-24)",
                    path);
    const int n = int(seed_size), C = int(nch), K = int(nk);
    const size_t px = size_t(n) * n;
    if (int(seed.size()) != C)
        return fail(CG_ERR_FORMAT, "%s: %zu seed channels, num_channels = %d", path, seed.size(), C);
    for (int c = 0; c < C; ++c)
        if (seed[c].size() != px)
            return fail(CG_ERR_FORMAT, "%s: seed channel %d has %zu values, expected %zu", path, c,
                        seed[c].size(), px);
    if (int(c0.size()) != K || int(c1.size()) != K || int(mu.size()) != K || int(sg.size()) != K ||
        int(w.size()) != K)
        return fail(CG_ERR_FORMAT, "%s: per-kernel arrays must have num_kernels = %d entries",
                    path, K);
    for (int k = 0; k < K; ++k)
        if (c0[k] < 0 || c0[k] >= C || c1[k] < 0 || c1[k] >= C || c0[k] != std::floor(c0[k]) ||
            c1[k] != std::floor(c1[k]))
            return fail(CG_ERR_FORMAT, "%s: kernel %d channel index outside [0, %d)", path, k, C);

    out->seed_size = n;
    out->num_channels = C;
    out->num_kernels = K;
    out->temp = float(temp);
    out->seed_channels = static_cast<double*>(std::malloc(sizeof(double) * C * px));
    // config.rs:40 swaps c0 and c1: JSON c1 is the input channel.
    out->c0 = dup_array<uint32_t>(c1);
    out->c1 = dup_array<uint32_t>(c0);
    out->growth_mu = dup_array<float>(mu);
    out->growth_sigma = dup_array<float>(sg);
    out->growth_weights = dup_array<float>(w);
    if (!out->seed_channels || !out->c0 || !out->c1 || !out->growth_mu || !out->growth_sigma ||
        !out->growth_weights) {
        cg_free_config(out);
        return fail(CG_ERR_OOM, "cg_load_config_json: host allocation failed");
    }
    for (int c = 0; c < C; ++c) std::memcpy(out->seed_channels + c * px, seed[c].data(), sizeof(double) * px);
    return CG_OK;
}

int cg_kernels_bin_size(const char* path, int K, int* src_n) {
    using cg::fail;
    if (!path || !src_n || K < 1) return fail(CG_ERR_ARG, "cg_kernels_bin_size: bad argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(CG_ERR_IO, "cannot read kernel file %s", path);
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fclose(f);
    // config.rs:62-65: bytes per kernel, complex64 elements, integer sqrt.
    const size_t kb = size_t(sz) / size_t(K);
    const size_t elems = kb / 8;
    const size_t s = size_t(std::sqrt(double(elems)));
    if (s == 0 || s * s * 8 * size_t(K) != size_t(sz))
        return fail(CG_ERR_FORMAT, "%s: %ld bytes is not %d square complex64 grids", path, sz, K);
    *src_n = int(s);
    return CG_OK;
}

int cg_load_kernels_bin(const char* path, int K, int target, float* out) {
    using cg::fail;
    if (!out || target < 1) return fail(CG_ERR_ARG, "cg_load_kernels_bin: bad argument");
    int src = 0;
    int rc = cg_kernels_bin_size(path, K, &src);
    if (rc != CG_OK) return rc;
    if (src > target)
        return fail(CG_ERR_UNSUPPORTED,
                    "%s holds %dx%d kernels, larger than the %dx%d target (the reference's "
                    "resample only pads, config.rs:100)",
                    path, src, src, target, target);
    std::vector<char> raw;
    if (!read_file(path, raw)) return fail(CG_ERR_IO, "cannot read kernel file %s", path);
    const size_t sp = size_t(src) * src, tp = size_t(target) * target;
    std::vector<float> tmp;
    for (int k = 0; k < K; ++k) {
        const unsigned char* base =
            reinterpret_cast<const unsigned char*>(raw.data()) + size_t(k) * sp * 8;
        float* dst = out + size_t(k) * tp * 2;
        // little-endian f32 pairs, decoded byte by byte so the host's
        // endianness does not matter (config.rs:77-78 uses from_le_bytes)
        auto rd = [&](size_t i, int part) {
            const unsigned char* b = base + i * 8 + part * 4;
            uint32_t u = uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) |
                         (uint32_t(b[3]) << 24);
            float v;
            std::memcpy(&v, &u, 4);
            return v;
        };
        if (src == target) {
            for (size_t i = 0; i < tp; ++i) {
                dst[2 * i] = rd(i, 0);
                dst[2 * i + 1] = rd(i, 1);
            }
            continue;
        }
        // config.rs:90-116: centre (shift by src/2), zero-pad to the target
        // with offset (target-src)/2, shift back by target/2.
        std::memset(dst, 0, sizeof(float) * 2 * tp);
        const int hs = src / 2, hd = target / 2, pad = (target - src) / 2;
        for (int i = 0; i < src; ++i)
            for (int j = 0; j < src; ++j) {
                const int ci = (i + hs) % src, cj = (j + hs) % src;   // centered[ci][cj] = src[i][j]
                const int pi = pad + ci, pj = pad + cj;                // kernel[pi][pj]
                const int ri = (pi + hd) % target, rj = (pj + hd) % target;
                const size_t si = size_t(i) * src + j, di = size_t(ri) * target + rj;
                dst[2 * di] = rd(si, 0);
                dst[2 * di + 1] = rd(si, 1);
            }
    }
    return CG_OK;
}

int cg_load_config_bin(const char* path, cg_config* out) {
    using cg::fail;
    if (!path || !out) return fail(CG_ERR_ARG, "cg_load_config_bin: NULL argument");
    std::memset(out, 0, sizeof(*out));
    std::vector<char> raw;
    if (!read_file(path, raw)) return fail(CG_ERR_IO, "cannot read seed file %s", path);
    const size_t size = raw.size() - 1;   // read_file appends a NUL
    const auto* b = reinterpret_cast<const unsigned char*>(raw.data());
    if (size < 24 || std::memcmp(b, kSeedMagic, 8) != 0)
        return fail(CG_ERR_FORMAT, "%s: not a binary seed file (magic CNSEED01)", path);
    const uint32_t n = get_u32(b + 8), C = get_u32(b + 12), K = get_u32(b + 16);
    if (n < 1 || n > 65536 || C < 1 || C > 4096 || K < 1 || K > 65536)
        return fail(CG_ERR_FORMAT, "%s: implausible sizes n=%u C=%u K=%u", path, n, C, K);
    const size_t px = size_t(n) * n, head = seed_bin_header(int(K));
    if (size != head + 8 * size_t(C) * px)
        return fail(CG_ERR_FORMAT, "%s: %zu bytes, expected %zu for n=%u C=%u K=%u", path, size,
                    head + 8 * size_t(C) * px, n, C, K);
    const unsigned char* pk = b + 24;
    for (uint32_t k = 0; k < 2 * K; ++k)
        if (get_u32(pk + 4 * k) >= C)
            return fail(CG_ERR_FORMAT, "%s: kernel %u channel index outside [0, %u)", path, k % K, C);
    out->seed_size = int(n);
    out->num_channels = int(C);
    out->num_kernels = int(K);
    out->temp = get_f32(b + 20);
    out->seed_channels = static_cast<double*>(std::malloc(sizeof(double) * C * px));
    out->c0 = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * K));
    out->c1 = static_cast<uint32_t*>(std::malloc(sizeof(uint32_t) * K));
    out->growth_mu = static_cast<float*>(std::malloc(sizeof(float) * K));
    out->growth_sigma = static_cast<float*>(std::malloc(sizeof(float) * K));
    out->growth_weights = static_cast<float*>(std::malloc(sizeof(float) * K));
    if (!out->seed_channels || !out->c0 || !out->c1 || !out->growth_mu || !out->growth_sigma ||
        !out->growth_weights) {
        cg_free_config(out);
        return fail(CG_ERR_OOM, "cg_load_config_bin: host allocation failed");
    }
    for (uint32_t k = 0; k < K; ++k) {
        out->c1[k] = get_u32(pk + 4 * k);             // JSON c0: output channel
        out->c0[k] = get_u32(pk + 4 * (K + k));       // JSON c1: input channel
        out->growth_mu[k] = get_f32(pk + 4 * (2 * K + k));
        out->growth_sigma[k] = get_f32(pk + 4 * (3 * K + k));
        out->growth_weights[k] = get_f32(pk + 4 * (4 * K + k));
    }
    const unsigned char* ps = b + head;
    for (size_t i = 0; i < size_t(C) * px; ++i) out->seed_channels[i] = get_f64(ps + 8 * i);
    return CG_OK;
}

int cg_save_config_bin(const char* path, const cg_config* cfg) {
    using cg::fail;
    if (!path || !cfg || !cfg->seed_channels || !cfg->c0 || !cfg->c1 || !cfg->growth_mu ||
        !cfg->growth_sigma || !cfg->growth_weights)
        return fail(CG_ERR_ARG, "cg_save_config_bin: NULL argument");
    const int n = cfg->seed_size, C = cfg->num_channels, K = cfg->num_kernels;
    if (n < 1 || C < 1 || K < 1) return fail(CG_ERR_ARG, "cg_save_config_bin: empty config");
    for (int k = 0; k < K; ++k)
        if (cfg->c0[k] >= uint32_t(C) || cfg->c1[k] >= uint32_t(C))
            return fail(CG_ERR_ARG, "kernel %d channel index outside [0, %d)", k, C);
    std::vector<unsigned char> o;
    o.reserve(seed_bin_header(K));
    o.insert(o.end(), kSeedMagic, kSeedMagic + 8);
    put_u32(o, uint32_t(n));
    put_u32(o, uint32_t(C));
    put_u32(o, uint32_t(K));
    put_f32(o, cfg->temp);
    for (int k = 0; k < K; ++k) put_u32(o, cfg->c1[k]);   // JSON c0
    for (int k = 0; k < K; ++k) put_u32(o, cfg->c0[k]);   // JSON c1
    for (int k = 0; k < K; ++k) put_f32(o, cfg->growth_mu[k]);
    for (int k = 0; k < K; ++k) put_f32(o, cfg->growth_sigma[k]);
    for (int k = 0; k < K; ++k) put_f32(o, cfg->growth_weights[k]);
    o.resize(seed_bin_header(K), 0);
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(CG_ERR_IO, "cannot write seed file %s", path);
    bool ok = std::fwrite(o.data(), 1, o.size(), f) == o.size();
    // the seed in chunks, little-endian
    const size_t total = size_t(C) * n * n;
    std::vector<unsigned char> chunk;
    for (size_t i = 0; ok && i < total; i += 65536) {
        const size_t m = total - i < 65536 ? total - i : 65536;
        chunk.resize(8 * m);
        for (size_t j = 0; j < m; ++j) {
            uint64_t u;
            std::memcpy(&u, &cfg->seed_channels[i + j], 8);
            for (int q = 0; q < 8; ++q) chunk[8 * j + q] = static_cast<unsigned char>(u >> (8 * q));
        }
        ok = std::fwrite(chunk.data(), 1, chunk.size(), f) == chunk.size();
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return fail(CG_ERR_IO, "writing seed file %s failed", path);
    return CG_OK;
}

}  // extern "C"
